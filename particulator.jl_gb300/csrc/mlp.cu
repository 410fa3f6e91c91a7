// Kernels of the learned inverse-CDF sampler network (mlp.cuh): batched
// forward pass (inference and training), backward pass, Adam update.
//
// Tensor-core path (sm_103a, 5th generation): each CTA of 128 threads owns a
// tile of 128 rows.  Operands are 128 x 128 BF16 tiles in shared memory in the
// canonical K-major layout without swizzle: 8 x 8-element core matrices of
// 128 contiguous bytes, core (r/8, c/8) at ((r/8) * 16 + c/8) * 128 B, so the
// next core matrix along K is 128 B away (leading byte offset) and the next
// 8-row group 2048 B away (stride byte offset).  One elected thread issues
// eight tcgen05.mma (K = 16 each) per 128 x 128 x 128 product into a
// 128-column FP32 accumulator in tensor memory, commits them to an mbarrier,
// and every thread waits (bounded) and reads its own row back with
// tcgen05.ld (warp w owns lanes 32w .. 32w + 31).  D[m][n] = sum_k A(m,k) B(n,k).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "mlp.cuh"

namespace pcl {
namespace mlp {

// ---------------------------------------------------------------- helpers --
__device__ __forceinline__ uint32_t su32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, c) in a 128 x 128 K-major tile (r: M/N index, c: K index)
__device__ __forceinline__ uint32_t toff(int r, int c) {
    return ((((r >> 3) << 4) + (c >> 3)) << 7) + ((r & 7) << 4) + ((c & 7) << 1);
}

// shared-memory matrix descriptor: start address, LBO 128 B, SBO 2048 B,
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(2048u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor, kind::f16: D F32 (bits 4-5 = 1), A BF16 (bits 7-9 = 1),
// B BF16 (bits 10-12 = 1), both K-major, N = 128 (bits 17-22 = N/8), M = 128 (bits 24-28 = M/16)
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mbar_init(uint64_t* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(b)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for completion of phase `ph`; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t ph) {
    uint32_t done = 0;
    for (int it = 0; it < (1 << 22) && !done; ++it) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(su32(b)), "r"(ph)
            : "memory");
        if (!done) __nanosleep(32);
    }
    return done != 0;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 256 tensor-memory columns (two 128 x 128 FP32 accumulators).  Every kernel
// here uses more than a third of an SM's shared memory, so at most two CTAs
// share an SM and their 2 x 256 columns always fit the 512 available.
constexpr uint32_t kTmemCols = 256;

__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}

// D (tensor memory) = / += A (smem tile) x B (smem tile)^T over K = 128
__device__ __forceinline__ void umma_128(uint32_t d, uint32_t sa, uint32_t sb, bool accumulate) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        uint64_t da = sdesc(sa + 256u * k), db = sdesc(sb + 256u * k);
        uint32_t en = (accumulate || k > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
            "l"(da), "l"(db), "r"(kIdesc), "r"(en)
            : "memory");
    }
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

// this thread's row (lane) of 32 accumulator columns starting at `col`
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// GELU in its tanh form (Hendrycks and Gimpel, "Gaussian Error Linear Units",
// 2016): 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))) = z sigmoid(v) with
// v = 2 sqrt(2/pi) (z + 0.044715 z^3): one exponential and one fast quotient
// per unit (v is clamped where sigmoid(v) is already 0 in FP32).
constexpr float kGeluK = 1.5957691216057308f;   // 2 sqrt(2 / pi)
constexpr float kGeluA = 0.044715f;
__device__ __forceinline__ float gelu(float z) {
    const float v = fmaxf(kGeluK * fmaf(kGeluA * z, z * z, z), -80.0f);
    return __fdividef(z, 1.0f + __expf(-v));
}
// d/dz [z sigmoid(v)] = s + z s (1 - s) dv/dz, s = sigmoid(v), dv/dz = K (1 + 3 A z^2)
__device__ __forceinline__ float dgelu(float z) {
    const float z2 = z * z;
    const float v = fmaxf(kGeluK * fmaf(kGeluA * z, z2, z), -80.0f);
    const float s = __fdividef(1.0f, 1.0f + __expf(-v));
    return fmaf(z * s * (1.0f - s), kGeluK * fmaf(3.0f * kGeluA, z2, 1.0f), s);
}

// warp-wide sum, added once to a shared-memory accumulator
__device__ __forceinline__ void warp_sum_add(float* dst, float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(dst, v);
}

// write 8 consecutive K-elements of row r (starting at c, c % 8 == 0) as one 16-B store
__device__ __forceinline__ void st_row8(unsigned char* tile, int r, int c, const float* v) {
    __nv_bfloat162 q0 = __floats2bfloat162_rn(v[0], v[1]), q1 = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 q2 = __floats2bfloat162_rn(v[4], v[5]), q3 = __floats2bfloat162_rn(v[6], v[7]);
    uint4 u;
    u.x = *reinterpret_cast<uint32_t*>(&q0); u.y = *reinterpret_cast<uint32_t*>(&q1);
    u.z = *reinterpret_cast<uint32_t*>(&q2); u.w = *reinterpret_cast<uint32_t*>(&q3);
    *reinterpret_cast<uint4*>(tile + toff(r, c)) = u;
}

// load a [128][128] BF16 row-major matrix into a tile: as is (element (r, c) =
// W[r][c]) or transposed (element (r, c) = W[c][r]).  128 threads.
__device__ void load_tile(unsigned char* tile, const __nv_bfloat16* W, bool transpose) {
    const int t = threadIdx.x;
    const uint4* row = reinterpret_cast<const uint4*>(W + (size_t)t * kH);
    for (int q = 0; q < 16; ++q) {
        uint4 u = row[q];
        if (!transpose) {
            *reinterpret_cast<uint4*>(tile + toff(t, 8 * q)) = u;
        } else {
            const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&u);
            for (int i = 0; i < 8; ++i) *reinterpret_cast<__nv_bfloat16*>(tile + toff(8 * q + i, t)) = e[i];
        }
    }
}

struct Smem {
    unsigned char* base;       // 1024-aligned start of the tiles
    uint64_t* bar;
    uint32_t* tslot;
    float* red;                // per-CTA reductions
};

__device__ __forceinline__ Smem carve(unsigned char* raw, int ntiles) {
    Smem s;
    uintptr_t p = (reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023);
    s.base = reinterpret_cast<unsigned char*>(p);
    unsigned char* tail = s.base + size_t(ntiles) * kTileBytes;
    s.bar = reinterpret_cast<uint64_t*>(tail);
    s.tslot = reinterpret_cast<uint32_t*>(tail + 8);
    s.red = reinterpret_cast<float*>(tail + 64);
    return s;
}

// CTA prologue: mbarrier, tensor memory.  Returns the tensor-memory base.
__device__ __forceinline__ uint32_t setup(Smem& s) {
    if (threadIdx.x == 0) mbar_init(s.bar);
    if ((threadIdx.x >> 5) == 0) tmem_alloc(s.tslot);
    tc_before();
    __syncthreads();
    tc_after();
    return *s.tslot;
}

__device__ __forceinline__ void teardown(uint32_t tbase) {
    tc_before();
    __syncthreads();
    tc_after();
    if ((threadIdx.x >> 5) == 0) tmem_free(tbase);
}

// issue one 128 x 128 x 128 product (thread 0), then every thread waits for it.
// On a timeout the error flag is set and false returned.
__device__ __forceinline__ bool mma_sync(Smem& s, uint32_t d, const unsigned char* A, const unsigned char* B,
                                         bool accumulate, uint32_t& ph, int* err) {
    fence_async_smem();
    tc_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_after();
        umma_128(d, su32(A), su32(B), accumulate);
        umma_commit(s.bar);
    }
    bool ok = mbar_wait(s.bar, ph);
    if (!ok) {
        // give the products in flight a second bounded wait before the caller
        // frees tensor memory and returns
        mbar_wait(s.bar, ph);
        if (threadIdx.x == 0) atomicExch(err, 1);
    }
    ph ^= 1u;
    tc_after();
    return __syncthreads_and(ok) != 0;
}

// ------------------------------------------------------------------ forward --
// One row per thread.  Training forward pass (inference runs k_mlp_infer):
// keeps the activations in tb, accumulates the mean-squared-error loss and the
// gradients of the output layer and of b3, and writes dz3; Y (optional)
// receives the outputs.
__global__ void __launch_bounds__(128, 1) k_mlp_forward(Net net, const float* X, long long n, float* Y, TrainBuf tb,
                                                        const float* T, float* G, double* loss, int* err) {
    extern __shared__ unsigned char raw[];
    Smem s = carve(raw, 3);
    unsigned char* sA = s.base;
    unsigned char* sW2 = s.base + kTileBytes;
    unsigned char* sW3 = s.base + 2 * kTileBytes;
    const int t = threadIdx.x;
    const bool train = (T != nullptr);
    float* r_w4 = s.red;          // [128] dL/dw4
    float* r_b3 = s.red + kH;     // [128] dL/db3
    float* r_b4 = s.red + 2 * kH; // [1] dL/db4, [2] loss
    for (int i = t; i < 2 * kH + 3; i += blockDim.x) s.red[i] = 0.0f;
    load_tile(sW2, net.W2, false);
    load_tile(sW3, net.W3, false);
    uint32_t tbase = setup(s);
    uint32_t ph = 0;
    const float* P = net.P;
    const uint32_t lane_off = uint32_t((t >> 5) * 32) << 16;
    const long long ntiles = (n + kH - 1) / kH;
    bool ok = true;
    for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long long row = tile * kH + t;
        const bool valid = row < n;
        const float x0 = valid ? X[2 * row] : 0.0f, x1 = valid ? X[2 * row + 1] : 0.0f;
        // layer 1 (FP32): h1 = gelu(W1 x + b1)
        for (int c = 0; c < kH; c += 8) {
            float h[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                float z = fmaf(P[oW1 + 2 * (c + i)], x0, fmaf(P[oW1 + 2 * (c + i) + 1], x1, P[ob1 + c + i]));
                if (train && valid) tb.z1[row * kH + c + i] = z;
                h[i] = gelu(z);
            }
            st_row8(sA, t, c, h);
            if (train && valid) {
                __nv_bfloat162* d = reinterpret_cast<__nv_bfloat162*>(tb.h1 + row * kH + c);
                d[0] = __floats2bfloat162_rn(h[0], h[1]); d[1] = __floats2bfloat162_rn(h[2], h[3]);
                d[2] = __floats2bfloat162_rn(h[4], h[5]); d[3] = __floats2bfloat162_rn(h[6], h[7]);
            }
        }
        // layer 2 on the tensor cores: z2 = h1 W2^T (+ b2)
        ok = mma_sync(s, tbase, sA, sW2, false, ph, err);
        if (!ok) break;
        for (int c = 0; c < kH; c += 32) {
            float v[32];
            tmem_ld32(tbase + lane_off + c, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                float z = v[i] + P[ob2 + c + i];
                if (train && valid) tb.z2[row * kH + c + i] = z;
                v[i] = gelu(z);
            }
            if (train && valid) {
                for (int i = 0; i < 32; i += 2)
                    *reinterpret_cast<__nv_bfloat162*>(tb.h2 + row * kH + c + i) = __floats2bfloat162_rn(v[i], v[i + 1]);
            }
#pragma unroll
            for (int i = 0; i < 32; i += 8) st_row8(sA, t, c + i, v + i);
        }
        // layer 3: z3 = h2 W3^T (+ b3)
        ok = mma_sync(s, tbase + 128, sA, sW3, false, ph, err);
        if (!ok) break;
        float y = P[ob4];
        for (int c = 0; c < kH; c += 32) {
            float v[32];
            tmem_ld32(tbase + lane_off + 128 + c, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) y = fmaf(P[ow4 + c + i], gelu(v[i] + P[ob3 + c + i]), y);
        }
        if (!train) {
            if (valid) Y[row] = y;
            continue;
        }
        if (valid && Y) Y[row] = y;
        // output layer backward: L = mean (y - T)^2; z3 is still in tensor memory
        const float e = valid ? y - T[row] : 0.0f;
        const float dy = 2.0f * e / float(n);
        warp_sum_add(&r_b4[2], e * e);
        warp_sum_add(&r_b4[0], dy);
        for (int c = 0; c < kH; c += 32) {
            float v[32];
            tmem_ld32(tbase + lane_off + 128 + c, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const float z = v[i] + P[ob3 + c + i];
                if (valid) tb.z3[row * kH + c + i] = z;
                const float g = dy * P[ow4 + c + i] * dgelu(z);
                warp_sum_add(&r_w4[c + i], dy * gelu(z));
                warp_sum_add(&r_b3[c + i], g);
                v[i] = g;
            }
            if (valid) {
                for (int i = 0; i < 32; i += 2)
                    *reinterpret_cast<__nv_bfloat162*>(tb.dz3 + row * kH + c + i) =
                        __floats2bfloat162_rn(v[i], v[i + 1]);
            }
        }
    }
    teardown(tbase);
    if (train) {
        __syncthreads();
        for (int c = t; c < kH; c += blockDim.x) {
            atomicAdd(&G[ow4 + c], r_w4[c]);
            atomicAdd(&G[ob3 + c], r_b3[c]);
        }
        if (t == 0) {
            atomicAdd(&G[ob4], r_b4[0]);
            atomicAdd(loss, double(r_b4[2]) / double(n));
        }
    }
}

// ---------------------------------------------------------------- infer --
// Inference of up to kMaxNets networks on the same rows, one network per
// blockIdx.y, over min(cap, *n_dev) rows.  512 threads per 128-row tile:
// thread t owns row t % 128 (its warp reads tensor-memory lanes
// 32 (w % 4) .. 32 (w % 4) + 31) and the 32 columns of quarter q = t / 128 in
// every layer, so each row's GELUs are spread over four warps; the output
// layer's four partial sums are added in quarter order in shared memory.
__device__ __forceinline__ void load_tile_q(unsigned char* tile, const __nv_bfloat16* W) {
    const int r = threadIdx.x & (kH - 1), q0 = 4 * (threadIdx.x >> 7);
    const uint4* row = reinterpret_cast<const uint4*>(W + (size_t)r * kH);
#pragma unroll
    for (int q = q0; q < q0 + 4; ++q) *reinterpret_cast<uint4*>(tile + toff(r, 8 * q)) = row[q];
}

__global__ void __launch_bounds__(kInferThreads, 1) k_mlp_infer(NetSet ns, const float* X, long long cap,
                                                                 const unsigned long long* n_dev, int* err) {
    const long long n = n_dev ? min(cap, (long long)*n_dev) : cap;
    const long long ntiles = (n + kH - 1) / kH;
    if ((long long)blockIdx.x >= ntiles) return;   // whole block: before any barrier or tensor memory
    extern __shared__ unsigned char raw[];
    Smem s = carve(raw, 3);
    unsigned char* sA = s.base;
    unsigned char* sW2 = s.base + kTileBytes;
    unsigned char* sW3 = s.base + 2 * kTileBytes;
    const Net net = ns.net[blockIdx.y];
    float* Y = ns.Y[blockIdx.y];
    const int t = threadIdx.x;
    const int r = t & (kH - 1);            // row within the tile
    const int c0 = 32 * (t >> 7);          // first column of this thread's quarter
    load_tile_q(sW2, net.W2);
    load_tile_q(sW3, net.W3);
    uint32_t tbase = setup(s);
    uint32_t ph = 0;
    const float* P = net.P;
    const uint32_t lane_off = uint32_t(((t >> 5) & 3) * 32) << 16;
    float* part = s.red;                   // [4][128] output-layer partial sums
    bool ok = true;
    for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long long row = tile * kH + r;
        const bool valid = row < n;
        const float x0 = valid ? X[2 * row] : 0.0f, x1 = valid ? X[2 * row + 1] : 0.0f;
        for (int c = c0; c < c0 + 32; c += 8) {
            float h[8];
#pragma unroll
            for (int i = 0; i < 8; ++i)
                h[i] = gelu(fmaf(P[oW1 + 2 * (c + i)], x0, fmaf(P[oW1 + 2 * (c + i) + 1], x1, P[ob1 + c + i])));
            st_row8(sA, r, c, h);
        }
        ok = mma_sync(s, tbase, sA, sW2, false, ph, err);
        if (!ok) break;
        {
            float v[32];
            tmem_ld32(tbase + lane_off + c0, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = gelu(v[i] + P[ob2 + c0 + i]);
#pragma unroll
            for (int i = 0; i < 32; i += 8) st_row8(sA, r, c0 + i, v + i);
        }
        ok = mma_sync(s, tbase + 128, sA, sW3, false, ph, err);
        if (!ok) break;
        {
            float v[32];
            tmem_ld32(tbase + lane_off + 128 + c0, v);
            float y = 0.0f;
#pragma unroll
            for (int i = 0; i < 32; ++i) y = fmaf(P[ow4 + c0 + i], gelu(v[i] + P[ob3 + c0 + i]), y);
            part[(t >> 7) * kH + r] = y;
        }
        __syncthreads();
        if (t < kH && valid) Y[row] = P[ob4] + part[r] + part[kH + r] + part[2 * kH + r] + part[3 * kH + r];
        // the next tile writes `part` only after two more block barriers (in mma_sync)
    }
    teardown(tbase);
}

// ------------------------------------------------------- backward (rows) --
// dz2 = (dz3 W3) * gelu'(z2), dz1 = (dz2 W2) * gelu'(z1); gradients of W1,
// b1 and b2.  Writes dz2 for the weight-gradient kernel.
__global__ void __launch_bounds__(128, 1) k_mlp_bwd_a(Net net, const float* X, long long n, TrainBuf tb, float* G,
                                                      int* err) {
    extern __shared__ unsigned char raw[];
    Smem s = carve(raw, 3);
    unsigned char* sA = s.base;
    unsigned char* sW3t = s.base + kTileBytes;   // element (in, out) = W3[out][in]
    unsigned char* sW2t = s.base + 2 * kTileBytes;
    const int t = threadIdx.x;
    float* r_w1 = s.red;            // [128][2]
    float* r_b1 = s.red + 2 * kH;   // [128]
    float* r_b2 = s.red + 3 * kH;   // [128]
    for (int i = t; i < 4 * kH; i += blockDim.x) s.red[i] = 0.0f;
    load_tile(sW3t, net.W3, true);
    load_tile(sW2t, net.W2, true);
    uint32_t tbase = setup(s);
    uint32_t ph = 0;
    const uint32_t lane_off = uint32_t((t >> 5) * 32) << 16;
    const long long ntiles = (n + kH - 1) / kH;
    bool ok = true;
    for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long long row = tile * kH + t;
        const bool valid = row < n;
        // A = dz3 rows
        const uint4* src = reinterpret_cast<const uint4*>(tb.dz3 + (valid ? row : 0) * kH);
        for (int q = 0; q < 16; ++q) {
            uint4 u = valid ? src[q] : make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4*>(sA + toff(t, 8 * q)) = u;
        }
        ok = mma_sync(s, tbase, sA, sW3t, false, ph, err);
        if (!ok) break;
        for (int c = 0; c < kH; c += 32) {
            float v[32];
            tmem_ld32(tbase + lane_off + c, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                float g = valid ? v[i] * dgelu(tb.z2[row * kH + c + i]) : 0.0f;
                v[i] = g;
                warp_sum_add(&r_b2[c + i], g);
            }
            if (valid) {
                for (int i = 0; i < 32; i += 2)
                    *reinterpret_cast<__nv_bfloat162*>(tb.dz2 + row * kH + c + i) =
                        __floats2bfloat162_rn(v[i], v[i + 1]);
            }
#pragma unroll
            for (int i = 0; i < 32; i += 8) st_row8(sA, t, c + i, v + i);
        }
        ok = mma_sync(s, tbase + 128, sA, sW2t, false, ph, err);
        if (!ok) break;
        const float x0 = valid ? X[2 * row] : 0.0f, x1 = valid ? X[2 * row + 1] : 0.0f;
        for (int c = 0; c < kH; c += 32) {
            float v[32];
            tmem_ld32(tbase + lane_off + 128 + c, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                float g = valid ? v[i] * dgelu(tb.z1[row * kH + c + i]) : 0.0f;
                warp_sum_add(&r_w1[2 * (c + i)], g * x0);
                warp_sum_add(&r_w1[2 * (c + i) + 1], g * x1);
                warp_sum_add(&r_b1[c + i], g);
            }
        }
    }
    teardown(tbase);
    __syncthreads();
    for (int i = t; i < 2 * kH; i += blockDim.x) atomicAdd(&G[oW1 + i], r_w1[i]);
    for (int c = t; c < kH; c += blockDim.x) {
        atomicAdd(&G[ob1 + c], r_b1[c]);
        atomicAdd(&G[ob2 + c], r_b2[c]);
    }
}

// --------------------------------------------------- backward (weights) --
// dW3 = dz3^T h2 and dW2 = dz2^T h1, reduced over the batch: each CTA
// accumulates its chunks of 128 rows in tensor memory (K = batch), then adds
// its 128 x 128 partial sums to G.
__global__ void __launch_bounds__(128, 1) k_mlp_bwd_w(long long n, TrainBuf tb, float* G, int* err) {
    extern __shared__ unsigned char raw[];
    Smem s = carve(raw, 4);
    unsigned char* sD3 = s.base;                   // element (o, b) = dz3[b][o]
    unsigned char* sH2 = s.base + kTileBytes;      // element (i, b) = h2[b][i]
    unsigned char* sD2 = s.base + 2 * kTileBytes;
    unsigned char* sH1 = s.base + 3 * kTileBytes;
    const int t = threadIdx.x;
    uint32_t tbase = setup(s);
    uint32_t ph = 0;
    const uint32_t lane_off = uint32_t((t >> 5) * 32) << 16;
    const long long nchunks = (n + kH - 1) / kH;
    bool first = true, ok = true;
    for (long long ch = blockIdx.x; ch < nchunks && ok; ch += gridDim.x) {
        const long long row = ch * kH + t;
        const bool valid = row < n;
        const __nv_bfloat16 zero = __float2bfloat16(0.0f);
        const __nv_bfloat16* a3 = tb.dz3 + (valid ? row : 0) * kH;
        const __nv_bfloat16* a2 = tb.dz2 + (valid ? row : 0) * kH;
        const __nv_bfloat16* b2 = tb.h2 + (valid ? row : 0) * kH;
        const __nv_bfloat16* b1 = tb.h1 + (valid ? row : 0) * kH;
        for (int f = 0; f < kH; ++f) {
            uint32_t o = toff(f, t);
            *reinterpret_cast<__nv_bfloat16*>(sD3 + o) = valid ? a3[f] : zero;
            *reinterpret_cast<__nv_bfloat16*>(sH2 + o) = valid ? b2[f] : zero;
            *reinterpret_cast<__nv_bfloat16*>(sD2 + o) = valid ? a2[f] : zero;
            *reinterpret_cast<__nv_bfloat16*>(sH1 + o) = valid ? b1[f] : zero;
        }
        fence_async_smem();
        tc_before();
        __syncthreads();
        if (t == 0) {
            tc_after();
            umma_128(tbase, su32(sD3), su32(sH2), !first);
            umma_128(tbase + 128, su32(sD2), su32(sH1), !first);
            umma_commit(s.bar);
        }
        bool w = mbar_wait(s.bar, ph);
        if (!w) {
            mbar_wait(s.bar, ph);
            if (t == 0) atomicExch(err, 1);
        }
        ph ^= 1u;
        tc_after();
        ok = __syncthreads_and(w) != 0;
        first = false;
    }
    if (ok && !first) {
        for (int c = 0; c < kH; c += 32) {
            float v[32];
            tmem_ld32(tbase + lane_off + c, v);
            for (int i = 0; i < 32; ++i) atomicAdd(&G[oW3 + t * kH + c + i], v[i]);
            tmem_ld32(tbase + lane_off + 128 + c, v);
            for (int i = 0; i < 32; ++i) atomicAdd(&G[oW2 + t * kH + c + i], v[i]);
        }
    }
    teardown(tbase);
}

// ------------------------------------------------------------------- Adam --
__global__ void k_mlp_adam(float* P, const float* G, float* M, float* V, __nv_bfloat16* W2, __nv_bfloat16* W3,
                           float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNParam; i += gridDim.x * blockDim.x) {
        float g = G[i];
        float m = b1 * M[i] + (1.0f - b1) * g;
        float v = b2 * V[i] + (1.0f - b2) * g * g;
        M[i] = m; V[i] = v;
        float p = P[i] - lr * (m * c1) / (sqrtf(v * c2) + eps);
        P[i] = p;
        if (i >= oW2 && i < oW2 + kH * kH) W2[i - oW2] = __float2bfloat16(p);
        else if (i >= oW3 && i < oW3 + kH * kH) W3[i - oW3] = __float2bfloat16(p);
    }
}

__global__ void k_mlp_sync_bf16(const float* P, __nv_bfloat16* W2, __nv_bfloat16* W3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kH * kH; i += gridDim.x * blockDim.x) {
        W2[i] = __float2bfloat16(P[oW2 + i]);
        W3[i] = __float2bfloat16(P[oW3 + i]);
    }
}

// Minibatch gather: row i of the batch is dataset row h(key, step, i) mod nall
// (a 64-bit mix of the counter; any uniform index generator serves here).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_mlp_gather(const float* Xall, const float* Tall, long long nall, float* X, float* T, int B,
                             uint32_t key0, uint32_t key1, uint32_t step) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    uint64_t h = mix64((uint64_t(key1) << 32 | key0) ^ mix64((uint64_t(step) << 32) | uint32_t(i)));
    long long j = (long long)(h % (uint64_t)nall);
    X[2 * i] = Xall[2 * j];
    X[2 * i + 1] = Xall[2 * j + 1];
    T[i] = Tall[j];
}

}  // namespace mlp
}  // namespace pcl
