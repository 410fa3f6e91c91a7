// Internal interface of the host side of the C ABI (the context, its device
// memory and the step driver), shared by the ctx*.cu translation units.
// Nothing here is part of the C ABI; the helpers are hidden in the library.
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "device.cuh"
#include "physconst.h"
#include "../../include/particulator_gb300.h"
#include "mlp.cuh"

extern "C" int pcl_ratebound_split(int, int, int, int, double, const double*, double, double*, double*);

namespace pcl {
cudaError_t launch_step(int minb, int grid, int threads, size_t smem, cudaStream_t stream, const StepArgs& A);
cudaError_t prepare_step(int minb, size_t smem, bool general, bool event, bool learn);
cudaError_t launch_step_prepared(int minb, int grid, int threads, size_t smem, cudaStream_t stream,
                                 const StepArgs& A);
__global__ void k_learn_hist(StepArgs A, int species, int j, int kind, int nT, long long per_T, int nbins,
                             float hmin, float hmax, unsigned long long sid_base, unsigned int* hist);
__global__ void k_learn_x(const float4* ps, const float4* m2, const unsigned long long* n_dev, long long cap,
                          float* X);
__global__ void k_roulette(float4* xw, uint4* meta, long long n, float pkeep, uint32_t k0, uint32_t k1,
                           unsigned long long* dead);
__global__ void k_split(float4* xw, float4* ps, uint4* meta, long long n, long long cap, float p, double e,
                        int nswarm, uint32_t k0, uint32_t k1, unsigned long long* nslots, unsigned long long* lost);
__global__ void k_roulette_fn(float4* xw, const float4* ps, uint4* meta, long long n, int species, const double* tab,
                              int nt, uint32_t k0, uint32_t k1, unsigned long long* dead);
__global__ void k_split_fn(float4* xw, float4* ps, uint4* meta, long long n, long long cap, int species,
                           const double* tab, int nt, int nswarm, uint32_t k0, uint32_t k1,
                           unsigned long long* nslots, unsigned long long* lost);
__global__ void k_roulette_swarms(float4* xw, uint4* meta, long long n, const float* pkeep, int nswarm, uint32_t k0,
                                  uint32_t k1, unsigned long long* dead);
__global__ void k_swarm_count(const uint4* meta, const unsigned long long* nslots, long long cap, int nswarm,
                              unsigned int* counts);
__global__ void k_roulette_cap(float4* xw, uint4* meta, const unsigned long long* nslots, long long slot_cap,
                               const unsigned int* counts, int nswarm, unsigned long long cap, uint32_t k0,
                               uint32_t k1);
__global__ void k_energy_hist(const float4* xw, const float4* ps, const uint4* meta, const unsigned long long* nslots,
                              long long cap, int species, int swarm, const double* edges, int nb,
                              unsigned long long* counts, double* wsum);
__global__ void k_learn_pick(const float4* m2, const unsigned long long* n_dev, long long cap, const float* Yk,
                             long long stride, LearnPick which, float* Y);
__global__ void k_draw_table(StepArgs A, int species, int j, int kind, long long n, unsigned long long sid_base,
                             float* out, uint32_t* draws);
__global__ void k_draw_net_x(long long n, unsigned long long sid_base, uint32_t k0, uint32_t k1, float* X);
__global__ void k_draw_net_map(StepArgs A, int species, int j, int kind, long long n, const float* Y, float* out);
namespace mlp {
cudaError_t infer_multi(void* const* handles, int nnets, const float* X, const unsigned long long* n_dev,
                        long long cap, float* Y, long long ystride, cudaStream_t stream);
}
__global__ void k_begin(Control* ctl, long long cap0, long long cap1, long long cap2);
__global__ void k_test_wait(Control* ctl, int max_iters);
__global__ void k_begin_spill(Control* ctl, unsigned long long* in_n, unsigned long long* out_n);

__global__ void k_compact_count(CompactArgs C);
__global__ void k_compact_scan(CompactArgs C);
__global__ void k_compact_scatter(CompactArgs C);
__global__ void k_moments(const float4* xw, const float4* ps, const uint4* meta, long long n, int species,
                          double* out);
__global__ void k_swarm_moments(const float4* xw, const float4* ps, const uint4* meta, long long n, int species,
                                int nswarm, double* partial);
__global__ void k_swarm_reduce(const double* partial, int nblocks, int len, double* out);
__global__ void k_test_sampler(StepArgs A, int species, int j, long long n, const float* p_in,
                               const uint32_t* sid, float* out_p, float* out_s, int* out_kind,
                               uint32_t* out_ctr);
size_t step_smem_bytes(int blob_bytes, int threads, bool event);
const char* noalloc_last_error();
constexpr int kTile = 2048;

// Host Philox4x32-10 (same function as the device one; used to draw initial s).
inline void philox_host(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t m0 = uint64_t(0xD2511F53u) * c[0];
        uint64_t m1 = uint64_t(0xCD9E8D57u) * c[2];
        uint32_t hi0 = uint32_t(m0 >> 32), lo0 = uint32_t(m0);
        uint32_t hi1 = uint32_t(m1 >> 32), lo1 = uint32_t(m1);
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

struct SpeciesState {
    bool set = false;
    double cut = INFINITY;   // J
    long long cap = 0;
    int flags = 0;
    float4* xw[2] = {nullptr, nullptr};
    float4* ps[2] = {nullptr, nullptr};
    uint4* meta[2] = {nullptr, nullptr};
    int cur = 0;
    // collision table (host copy, SI)
    int order = 1, nproc = 0, nint = 1;
    double xmax = 1.0;
    std::vector<double> rate, rb;
    int wall_coord = -1;
    double wall_v = 0.0;
    int wall_drop = 1;
    std::vector<pcl_process> procs;
    std::vector<int> sb_index;
    // linear-grid table (table_kind 1)
    int table_kind = 0;
    int lin_n = 0;
    double lin_e0 = 0, lin_e1 = 0;
    // tally-only histogram
    int hist_bins = 0;
    double hist_emin = 0, hist_emax = 0;
    unsigned long long* hist_n = nullptr;
    double* hist_w = nullptr;
};

struct SBTable {
    int Z, ne, ncum;
    std::vector<double> log_energy;  // log J
    std::vector<double> data;        // host copy of the inverse-CDF table (identity)
    float* d_data = nullptr;         // [ne][ncum]
};

struct Ctx {
    pcl_config cfg;
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    SpeciesState sp[3];
    std::vector<SBTable> sb;
    // forcing
    double E[3] = {0, 0, 0}, B[3] = {0, 0, 0};
    int field_kind = 0;
    // species bits: pushed at all, feeling the EM field, feeling the continuum
    // loss (RestrictedPusher / NullPusher / RestrictedForcing)
    int push_mask = 7, field_mask = 7, loss_mask = 7;
    int bfield_kind = 0;
    double bfield_p[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // SI (m, T)
    double field_p[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // SI
    int cl_order = 0, cl_k = 0;
    double cl_xmax = 0;
    std::vector<double> cl_ec, cl_pc;
    // batched swarms
    int nswarm = 0;
    double swarm_safety = 1.1;
    std::vector<double> swarm_E, swarm_Fdt;   // [nswarm][3] V/m, [nswarm] N s
    // blob
    bool blob_dirty = true;
    std::vector<unsigned char> blob;
    float4* d_blob = nullptr;
    size_t d_blob_cap = 0;
    // device control and scratch
    Control* d_ctl = nullptr;
    Control* h_ctl = nullptr;   // pinned mirror
    float4* sp_xw[2] = {nullptr, nullptr};
    float4* sp_ps[2] = {nullptr, nullptr};
    uint4* sp_meta[2] = {nullptr, nullptr};
    unsigned long long* d_spn = nullptr;  // [2]
    long long sp_cap = 0;
    unsigned int* d_tile_cnt = nullptr;
    unsigned long long* d_tile_off = nullptr;
    unsigned long long* d_nnew = nullptr;
    long long tiles_cap = 0;
    double* d_mom = nullptr;
    void* d_scr = nullptr;                 // reusable scratch of the moment and roulette entry points
    size_t scr_bytes = 0;
    unsigned int* d_swcnt = nullptr;       // [3][256] live particles per swarm
    long long swarm_cap[3] = {0, 0, 0};    // pcl_set_swarm_cap, 0 = off
    // pcl_advance_host: copy streams and per-chunk events
    cudaStream_t s_h2d = nullptr, s_d2h = nullptr, s_cmp = nullptr;
    std::vector<cudaEvent_t> io_ev;        // [2 * chunks]: uploaded, stepped
    std::vector<cudaEvent_t> io_tev;       // [2 * chunks]: timing of each chunk's launch
    cudaEvent_t io_join = nullptr;
    unsigned long long* d_heads = nullptr; // [64] work counters of the chunk launches
    int host_io = PCL_HOST_IO_AUTO;        // pcl_set_host_io
    // host-direct mode, set for the duration of one pcl_advance_host call:
    // population launches read these host slots and every slot write is
    // repeated to hx_* (device-usable pointers of the caller's page-locked arrays)
    const float4* hin_xw[3] = {nullptr, nullptr, nullptr};
    const float4* hin_ps[3] = {nullptr, nullptr, nullptr};
    const uint4* hin_meta[3] = {nullptr, nullptr, nullptr};
    float4* hx_xw[3] = {nullptr, nullptr, nullptr};
    float4* hx_ps[3] = {nullptr, nullptr, nullptr};
    uint4* hx_meta[3] = {nullptr, nullptr, nullptr};
    long long hx_cap[3] = {0, 0, 0};
    // accumulated host state
    double t = 0.0;
    long long steps = 0;
    long long particle_steps = 0;
    long long live[3] = {0, 0, 0};
    long long steps_since_compact = 0;
    int sticky = PCL_OK;
    // learned sampler: network per (species, table position), suspended-collision queues
    void* learn_net[3][16] = {};
    int learn_kind[3][16] = {};
    uint32_t learn_ok[3][16][2] = {};
    std::vector<void*> nets;       // distinct attached networks
    LearnPick pick{};
    bool learn_on = false;
    float4* lq_xw[2] = {nullptr, nullptr};
    float4* lq_ps[2] = {nullptr, nullptr};
    uint4* lq_m1[2] = {nullptr, nullptr};
    float4* lq_m2[2] = {nullptr, nullptr};
    float* lq_x = nullptr;         // [cap][2] network inputs
    float* lq_yk = nullptr;        // [nets][cap] outputs per network
    float* lq_y = nullptr;         // [cap] output of each collision's network
    unsigned long long* d_lqn = nullptr;  // [2]
    long long lq_cap = 0, lq_nets_cap = 0;
    long long learn_rounds = 0, learn_suspended = 0;
    // WallCallback records (device) and the context time at each launch start
    float4* d_wall_xw = nullptr; float4* d_wall_pt = nullptr; uint4* d_wall_meta = nullptr;
    unsigned long long* d_wall_n = nullptr;
    long long wall_cap = 0;
    std::vector<double> launch_t0 = std::vector<double>(1, 0.0);   // index = device launch_seq
    // CUDA graphs of launch groups (use_graph), keyed by every launch parameter
    struct GraphEntry { std::vector<unsigned char> key; cudaGraphExec_t exec; };
    std::vector<GraphEntry> graphs;
    unsigned long long* h_spn = nullptr;  // pinned mirror of d_spn
    unsigned long long* h_lqn = nullptr;  // pinned mirror of d_lqn
    long long graph_launches = 0;
    // instrumentation
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr, ev_t0 = nullptr, ev_t1 = nullptr;
    double k_ms = 0.0, k_bytes = 0.0;
    long long k_launches = 0, launches = 0;
};


#define PCL_INTERNAL __attribute__((visibility("hidden")))

inline int fail(Ctx* c, int code, const std::string& msg) {
    if (c) c->last_error = msg;
    return code;
}


// Stream-ordered copies: every transfer goes through the context stream and
// waits for it, so kernels on the (non-blocking) stream never race a copy.
inline cudaError_t h2d(Ctx* c, void* dst, const void* src, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(c->stream);
}
inline cudaError_t d2h(Ctx* c, void* dst, const void* src, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(c->stream);
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t _e = (call);                                                          \
        if (_e != cudaSuccess)                                                            \
            return fail(c, PCL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)


// ---- helpers defined in ctx.cu
PCL_INTERNAL void free_species_buffers(SpeciesState& s);
PCL_INTERNAL int ensure_tiles(Ctx* c);
PCL_INTERNAL int ensure_spill(Ctx* c);
PCL_INTERNAL int build_blob(Ctx* c);
PCL_INTERNAL StepArgs make_args(Ctx* c, double dt, int nsteps, int spill_mode, int sp_in);
PCL_INTERNAL void set_lq(StepArgs& A, Ctx* c, int out, int in);
PCL_INTERNAL void free_lq(Ctx* c);
PCL_INTERNAL int ensure_lq(Ctx* c);
PCL_INTERNAL int blocks_per_sm(Ctx* c);
PCL_INTERNAL int grid_blocks(Ctx* c);
PCL_INTERNAL int block_threads(Ctx* c);
PCL_INTERNAL int readback(Ctx* c);
PCL_INTERNAL int ensure_scratch(Ctx* c, size_t bytes);
PCL_INTERNAL int apply_swarm_caps(Ctx* c);
PCL_INTERNAL CompactArgs make_compact_args(Ctx* c);
PCL_INTERNAL cudaError_t enqueue_compact(Ctx* c, const CompactArgs& C);
PCL_INTERNAL void flip_buffers(Ctx* c);
PCL_INTERNAL int compact_all(Ctx* c);
PCL_INTERNAL cudaError_t enqueue_learned_round(Ctx* c, double dt, int nsteps, int minb, int threads,
                                               size_t smem);
PCL_INTERNAL void count_learned(Ctx* c);
PCL_INTERNAL int run_group_graph(Ctx* c, const StepArgs& A, const StepArgs& P0, const StepArgs& P1,
                                 const CompactArgs* C, int minb, int grid, int threads, size_t smem);
PCL_INTERNAL int drain_spills(Ctx* c, double dt, int nsteps, int threads, size_t smem, int in, int lq_out, bool* ran,
                              const unsigned long long* known_pending);
PCL_INTERNAL int launch_steps(Ctx* c, double dt_si, int nsteps);
PCL_INTERNAL int check_species(Ctx* c, int s);
PCL_INTERNAL int get_n(Ctx* c, int species, long long& n);

}  // namespace pcl
