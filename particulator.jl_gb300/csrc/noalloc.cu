// Compaction of a caller-owned population without any device allocation.
//
// Some callers cannot call cudaMalloc: a host that already owns the whole
// device through its own memory pool (a Julia CuArray pool, a framework
// allocator), code that runs where allocation is forbidden or would
// synchronise (a latency-critical loop, a stream that is being captured), or
// an embedding that budgets device memory up front.  For them,
// pcl_compact_noalloc does what pcl_compact does (repack!, population.jl:229-259)
// on device buffers the caller passes in, with its scratch (tile counts, tile
// offsets, the live count) in a file-scope static __device__ array of fixed
// size instead of context allocations.
//
// The array is PCL_NOALLOC_SCRATCH_BYTES (about 197 KB) and every GPU that
// loads the library holds it until the process exits.  All calls share it and
// it keeps the last call's contents, so calls that overlap on the GPU (two
// streams at once, or two host threads) race; serialise them.  Nothing in it
// needs to start at zero: each call writes every tile count and offset it
// reads.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture.  The cache assumes that the device's
// primary context lives until the process exits: after cudaDeviceReset the
// cached address would name memory of the destroyed context.
//
// The input and output buffers must not overlap: the scatter of one tile
// writes below its own input range while other tiles may still read there, so
// an in-place call would race.  Overlapping ranges are refused.
//
// Launch errors are read from each launch's own return code
// (cudaLaunchKernel), so an error left pending by earlier, unrelated work on
// the thread is neither reported as this call's nor cleared by it.
#include <cuda_runtime.h>
#include <mutex>
#include <string>

#include "device.cuh"
#include "../../include/particulator_gb300.h"

namespace pcl {
__global__ void k_compact_count(CompactArgs C);
__global__ void k_compact_scan(CompactArgs C);
__global__ void k_compact_scatter(CompactArgs C);
constexpr int kTile = 2048;

constexpr long long kMaxSlots = PCL_NOALLOC_MAX_SLOTS;
constexpr int kMaxTiles = int((kMaxSlots + kTile - 1) / kTile);
// layout: n_in (8 B), n_out (8 B), pad to 256, tile counts (4 B each), tile offsets (8 B each)
constexpr size_t kOffN = 0;
constexpr size_t kOffNOut = 8;
constexpr size_t kOffCnt = 256;
constexpr size_t kOffOff = kOffCnt + ((size_t(kMaxTiles) * 4 + 255) / 256) * 256;
constexpr size_t kScratchBytes = kOffOff + size_t(kMaxTiles) * 8;
static_assert(kScratchBytes == PCL_NOALLOC_SCRATCH_BYTES, "header constant out of date");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

__global__ void k_noalloc_set_n(unsigned long long* n, long long v) {
    if (threadIdx.x == 0) *n = (unsigned long long)v;
}

static std::mutex g_mu;
static void* g_addr[64];
static bool g_ready[64];
static thread_local std::string g_err;

// Device address of the scratch array for the current device (host code may
// not use the symbol itself: on the host it names a stand-in, not device memory).
static int scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { g_err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return PCL_ERR_CUDA; }
    if (dev < 0 || dev >= 64) { g_err = "device ordinal out of range"; return PCL_ERR_CUDA; }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ready[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            g_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return PCL_ERR_CUDA;
        }
        g_addr[dev] = p;
        g_ready[dev] = true;
    }
    *out = static_cast<unsigned char*>(g_addr[dev]);
    return PCL_OK;
}

const char* noalloc_last_error() { return g_err.c_str(); }

static bool ranges_overlap(const unsigned char* a, const unsigned char* b, size_t len) {
    return a < b + len && b < a + len;
}

}  // namespace pcl

using namespace pcl;

extern "C" int pcl_compact_noalloc(int64_t n, const float* xw, const float* ps, const uint32_t* meta,
                                   float* out_xw, float* out_ps, uint32_t* out_meta, int64_t* n_out,
                                   void* stream) {
    g_err.clear();
    if (n < 0 || (n > 0 && (!xw || !ps || !meta || !out_xw || !out_ps || !out_meta)) || !n_out) {
        g_err = "pcl_compact_noalloc: null buffer or negative size";
        return PCL_ERR_INVALID;
    }
    if (n > kMaxSlots) {
        g_err = "pcl_compact_noalloc: " + std::to_string(n) + " slots exceed PCL_NOALLOC_MAX_SLOTS (" +
                std::to_string(kMaxSlots) + "); use pcl_compact";
        return PCL_ERR_CAPACITY;
    }
    if (n > 0) {
        const size_t b16 = size_t(n) * 16;
        const unsigned char* in_lo[3] = {reinterpret_cast<const unsigned char*>(xw),
                                         reinterpret_cast<const unsigned char*>(ps),
                                         reinterpret_cast<const unsigned char*>(meta)};
        const unsigned char* out_lo[3] = {reinterpret_cast<const unsigned char*>(out_xw),
                                          reinterpret_cast<const unsigned char*>(out_ps),
                                          reinterpret_cast<const unsigned char*>(out_meta)};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                if (ranges_overlap(out_lo[a], in_lo[b], b16) || (a < b && ranges_overlap(out_lo[a], out_lo[b], b16))) {
                    g_err = "pcl_compact_noalloc: input and output buffers overlap (in-place compaction races)";
                    return PCL_ERR_INVALID;
                }
        const unsigned char* nb = reinterpret_cast<const unsigned char*>(n_out);
        for (int a = 0; a < 3; ++a)
            if (nb + sizeof(int64_t) > out_lo[a] && out_lo[a] + b16 > nb) {
                g_err = "pcl_compact_noalloc: n_out lies inside an output buffer";
                return PCL_ERR_INVALID;
            }
    }
    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned long long* dn = reinterpret_cast<unsigned long long*>(base + kOffN);
    unsigned long long* dn_out = reinterpret_cast<unsigned long long*>(base + kOffNOut);
    CompactArgs C = {};
    C.sxw[0] = reinterpret_cast<const float4*>(xw);
    C.sps[0] = reinterpret_cast<const float4*>(ps);
    C.smeta[0] = reinterpret_cast<const uint4*>(meta);
    C.dxw[0] = reinterpret_cast<float4*>(out_xw);
    C.dps[0] = reinterpret_cast<float4*>(out_ps);
    C.dmeta[0] = reinterpret_cast<uint4*>(out_meta);
    C.n = dn;
    C.tile_cnt[0] = reinterpret_cast<unsigned int*>(base + kOffCnt);
    C.tile_off[0] = reinterpret_cast<unsigned long long*>(base + kOffOff);
    C.n_out = dn_out;
    int nt = int(n > 0 ? (n + kTile - 1) / kTile : 1);
    C.ntiles_max = nt;
    long long nv = n;
    void* set_args[2] = {&dn, &nv};
    void* c_args[1] = {&C};
    const dim3 g(nt, 1);
    cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(k_noalloc_set_n), dim3(1), dim3(32), set_args, 0, s);
    if (e == cudaSuccess)
        e = cudaLaunchKernel(reinterpret_cast<const void*>(k_compact_count), g, dim3(256), c_args, 0, s);
    if (e == cudaSuccess)
        e = cudaLaunchKernel(reinterpret_cast<const void*>(k_compact_scan), dim3(1), dim3(1024), c_args, 0, s);
    if (e == cudaSuccess)
        e = cudaLaunchKernel(reinterpret_cast<const void*>(k_compact_scatter), g, dim3(256), c_args, 0, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(n_out, dn_out, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) {
        cudaGetLastError();   // this call's own launch error: not left for the caller's next check
        g_err = std::string("pcl_compact_noalloc: ") + cudaGetErrorString(e);
        return PCL_ERR_CUDA;
    }
    return PCL_OK;
}
