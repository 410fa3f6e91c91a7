// Host side of the C ABI: context, device memory, table packing, the step
// driver (advance! / run!) and the maintenance calls.  Every entry point
// returns a PCL_* status and records a message for pcl_last_error.
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
__global__ void k_split(float4* xw, float4* ps, uint4* meta, long long n, long long cap, float p, uint32_t k0,
                        uint32_t k1, unsigned long long* nslots, unsigned long long* lost);
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
namespace mlp {
cudaError_t infer_multi(void* const* handles, int nnets, const float* X, const unsigned long long* n_dev,
                        long long cap, float* Y, long long ystride, cudaStream_t stream);
}
__global__ void k_begin(Control* ctl, long long cap0, long long cap1, long long cap2);
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
static void philox_host(uint32_t c[4], uint32_t k0, uint32_t k1) {
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

static int fail(Ctx* c, int code, const std::string& msg) {
    if (c) c->last_error = msg;
    return code;
}


// Stream-ordered copies: every transfer goes through the context stream and
// waits for it, so kernels on the (non-blocking) stream never race a copy.
static cudaError_t h2d(Ctx* c, void* dst, const void* src, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(c->stream);
}
static cudaError_t d2h(Ctx* c, void* dst, const void* src, size_t bytes) {
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

static void free_species_buffers(SpeciesState& s) {
    for (int b = 0; b < 2; ++b) {
        cudaFree(s.xw[b]); cudaFree(s.ps[b]); cudaFree(s.meta[b]);
        s.xw[b] = nullptr; s.ps[b] = nullptr; s.meta[b] = nullptr;
    }
    cudaFree(s.hist_n); cudaFree(s.hist_w);
    s.hist_n = nullptr; s.hist_w = nullptr;
}

static int ensure_tiles(Ctx* c) {
    long long capmax = 0;
    for (auto& s : c->sp) capmax = std::max(capmax, s.cap);
    long long nt = (capmax + kTile - 1) / kTile;
    if (nt < 1) nt = 1;
    if (nt <= c->tiles_cap) return PCL_OK;
    cudaFree(c->d_tile_cnt); cudaFree(c->d_tile_off);
    CK(cudaMalloc(&c->d_tile_cnt, sizeof(unsigned int) * 3 * nt));
    CK(cudaMalloc(&c->d_tile_off, sizeof(unsigned long long) * 3 * nt));
    c->tiles_cap = nt;
    return PCL_OK;
}

static int ensure_spill(Ctx* c) {
    long long capmax = 0;
    for (auto& s : c->sp) capmax = std::max(capmax, s.cap);
    long long want = std::max<long long>(1 << 16, capmax / 16);
    if (want <= c->sp_cap) return PCL_OK;
    for (int b = 0; b < 2; ++b) {
        cudaFree(c->sp_xw[b]); cudaFree(c->sp_ps[b]); cudaFree(c->sp_meta[b]);
        CK(cudaMalloc(&c->sp_xw[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->sp_ps[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->sp_meta[b], sizeof(uint4) * want));
    }
    c->sp_cap = want;
    return PCL_OK;
}

// ------------------------------------------------------------ blob pack --
static void pack_proc(const pcl_process& P, int sbi, DevProc& D) {
    std::memset(&D, 0, sizeof(D));
    D.kind = P.kind;
    D.sb = -1;
    using namespace si;
    switch (P.kind) {
        case PCL_PROC_MOLLER:
        case PCL_PROC_BHABHA:
            D.p[0] = float(P.param[0] / mc2);
            break;
        case PCL_PROC_RBEB:
            D.p[0] = float(P.param[0] / mc2);
            D.p[1] = float(P.param[1] / mc2);
            D.p[2] = float(P.param[2]);
            break;
        case PCL_PROC_REL_COULOMB: {
            double Z = (P.Z == 0) ? P.param[0] : double(P.Z);
            double a = 1.3413 * std::pow(Z, -1.0 / 3.0) * a_0;     // relativistic_coulomb.jl:14
            double lam = hbar / (m_e * c * a);
            D.p[0] = float(lam * lam / 4.0);                       // alpha = p[0] / p^2
            break;
        }
        case PCL_PROC_SELTZER_BERGER:
            D.sb = sbi;
            D.p[0] = float(P.Z);
            break;
        case PCL_PROC_PHOTOELECTRIC:
            D.nbind = std::min(P.nparam, 8);
            for (int m = 0; m < D.nbind; ++m) D.p[m] = float(P.param[m] / mc2);
            break;
        case PCL_PROC_BETHE_HEITLER: {
            double Z = P.Z;
            double aZ = alpha, aZ2 = aZ * aZ, aZ4 = aZ2 * aZ2, aZ6 = aZ4 * aZ2;  // _fc (bethe_heitler.jl:153-161)
            double fc = (1 / (1 + aZ2) + 0.20206 - 0.0369 * aZ2 + 0.0083 * aZ4 - 0.0020 * aZ6) * aZ2;
            double FZ = 8 * std::log(Z) / 3;
            D.p[0] = float(Z);
            D.p[1] = float(std::pow(Z, 1.0 / 3.0));
            D.p[2] = float(FZ);
            D.p[3] = float(FZ + 8 * fc);
            D.p[4] = float(2e6 * eV / mc2);
            D.p[5] = float(50e6 * eV / mc2);
            break;
        }
        case PCL_PROC_ELASTIC:
            D.p[0] = float(P.param[0]);
            break;
        case PCL_PROC_EXCITATION:
        case PCL_PROC_IONIZATION:
        case PCL_PROC_ATTACHMENT:
            D.p[0] = float(P.param[0] / mc2);
            break;
        default:
            break;
    }
}

static int build_blob(Ctx* c) {
    if (!c->blob_dirty) return PCL_OK;
    using si::mc2;
    using si::e;
    using si::m_e;
    std::vector<float> data;
    auto off = [&]() { return int((sizeof(BlobHdr) / 4) + data.size()); };
    BlobHdr H;
    std::memset(&H, 0, sizeof(H));
    const float charge[3] = {-1.0f, 0.0f, 1.0f};
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        SpeciesHdr& h = H.sp[s];
        h.nproc = S.nproc;
        h.order = S.order;
        h.k = S.nint;
        h.tally_only = (S.flags & PCL_SPECIES_TALLY_ONLY) ? 1 : 0;
        h.xscale = float(1.0 / (S.xmax / mc2));
        h.cut = S.set ? float(S.cut / mc2) : INFINITY;
        h.charge = charge[s];
        h.table_kind = S.table_kind;
        h.wall_coord = (S.wall_coord >= 0 && c->wall_cap > 0) ? S.wall_coord : -1;
        h.wall_v = float(S.wall_v);
        h.wall_drop = S.wall_drop;
        if (S.table_kind == 1) {
            h.lin_n = S.lin_n;
            h.lin_e0 = float(S.lin_e0 / mc2);
            h.lin_inv_step = float(1.0 / ((S.lin_e1 - S.lin_e0) / (S.lin_n - 1) / mc2));
            h.rate_off = off();
            for (size_t q = 0; q < S.rate.size(); ++q) data.push_back(float(rate_to_dev(S.rate[q])));
            h.rb_off = off();
            for (int i = 0; i < S.lin_n; ++i) data.push_back(float(rate_to_dev(S.rb[i])));
        } else {
            const int nI = S.nint + 1;
            h.rate_off = off();
            for (int i = 0; i < nI; ++i)
                for (int j = 0; j < S.nproc; ++j)
                    for (int k = 0; k < S.order; ++k)
                        data.push_back(float(rate_to_dev(S.rate[k + S.order * (j + S.nproc * i)])));
            h.rb_off = off();
            for (int i = 0; i < nI; ++i)
                for (int k = 0; k < S.order; ++k)
                    data.push_back(S.rb.empty() ? 0.0f : float(rate_to_dev(S.rb[k + S.order * i])));
        }
        h.cl_off = -1;
        if (c->cl_order > 0 && s != PCL_PHOTON) {
            const std::vector<double>& cf = (s == PCL_ELECTRON) ? c->cl_ec : c->cl_pc;
            h.cl_off = off();
            h.cl_k = c->cl_k;
            h.cl_order = c->cl_order;
            h.cl_xscale = float(1.0 / (c->cl_xmax / mc2));
            for (int i = 0; i <= c->cl_k; ++i)
                for (int k = 0; k < c->cl_order; ++k) data.push_back(float(force_to_dev(cf[k + c->cl_order * i])));
        }
        h.rbB_off = -1;
        if (c->nswarm > 0 && S.table_kind == 0 && S.nproc > 0 && s != PCL_PHOTON) {
            // swarm mode: the rate bound of swarm k is A + Fdt_k B (compratebound is linear in Fdt)
            const int nI = S.nint + 1;
            std::vector<double> A(size_t(S.order) * nI), Bt(size_t(S.order) * nI);
            pcl_ratebound_split(s, S.order, S.nproc, S.nint, S.xmax, S.rate.data(), c->swarm_safety, A.data(),
                                Bt.data());
            h.rb_off = off();
            for (int i = 0; i < nI; ++i)
                for (int k = 0; k < S.order; ++k) data.push_back(float(rate_to_dev(A[k + S.order * i])));
            h.rbB_off = off();
            for (int i = 0; i < nI; ++i)
                for (int k = 0; k < S.order; ++k) data.push_back(float(rate_to_dev(Bt[k + S.order * i])));
        }
        for (int j = 0; j < S.nproc; ++j) {
            pack_proc(S.procs[j], S.sb_index[j], h.proc[j]);
            h.proc[j].learn = c->learn_net[s][j] ? c->learn_kind[s][j] : 0;
            h.proc[j].learn_ok[0] = c->learn_ok[s][j][0];
            h.proc[j].learn_ok[1] = c->learn_ok[s][j][1];
        }
        if (S.hist_bins > 0) {
            h.hist_bins = S.hist_bins;
            double lmin = std::log(S.hist_emin / mc2), lmax = std::log(S.hist_emax / mc2);
            h.hist_lmin = float(lmin);
            h.hist_linv = float(S.hist_bins / (lmax - lmin));
        }
    }
    H.nsb = int(c->sb.size());
    for (size_t b = 0; b < c->sb.size(); ++b) {
        SBHdr& h = H.sb[b];
        h.ne = c->sb[b].ne;
        h.ncum = c->sb[b].ncum;
        h.inv_dp = float(c->sb[b].ncum - 1);
        double ym = 0.0;
        for (int j = 0; j + 1 < h.ne; ++j)
            ym = std::max(ym, std::fabs(c->sb[b].data[size_t(j + 1) * h.ncum] - c->sb[b].data[size_t(j) * h.ncum]));
        h.ymargin = float(ym);
        h.le_off = off();
        for (int j = 0; j < h.ne; ++j) data.push_back(float(c->sb[b].log_energy[j] - std::log(mc2)));
    }
    for (int a = 0; a < 3; ++a) {
        H.E[a] = float(force_to_dev(e * c->E[a]));            // per unit charge
        H.B[a] = float(e * c->B[a] / m_e * NS);
    }
    H.field_kind = c->field_kind;
    {
        const double* q = c->field_p;
        auto fe = [&](double v) { return float(force_to_dev(e * v)); };
        switch (c->field_kind) {
            case 1: H.fp[0] = float(q[0]); H.fp[1] = float(q[1]);
                    for (int a = 0; a < 3; ++a) H.fp[2 + a] = fe(q[2 + a]);
                    break;
            case 2: H.fp[0] = float(q[0]);
                    for (int a = 0; a < 6; ++a) H.fp[1 + a] = fe(q[1 + a]);
                    break;
            case 3: for (int a = 0; a < 3; ++a) H.fp[a] = float(q[a]);
                    H.fp[3] = fe(q[3]);
                    break;
            default: break;
        }
    }
    H.nswarm = c->nswarm;
    H.swarm_off = off();
    if (c->nswarm > 0) {
        for (int k = 0; k < c->nswarm; ++k) {
            for (int a = 0; a < 3; ++a) data.push_back(float(force_to_dev(e * c->swarm_E[3 * k + a])));
            data.push_back(float(c->swarm_Fdt[k]));
        }
    } else {
        for (int a = 0; a < 3; ++a) data.push_back(H.E[a]);
        data.push_back(0.0f);
    }
    while (data.size() % 4) data.push_back(0.0f);
    size_t bytes = sizeof(BlobHdr) + data.size() * 4;
    bytes = (bytes + 15) & ~size_t(15);
    H.bytes = int(bytes);
    c->blob.assign(bytes, 0);
    std::memcpy(c->blob.data(), &H, sizeof(H));
    std::memcpy(c->blob.data() + sizeof(H), data.data(), data.size() * 4);
    if (bytes > c->d_blob_cap) {
        cudaFree(c->d_blob);
        CK(cudaMalloc(&c->d_blob, bytes));
        c->d_blob_cap = bytes;
    }
    CK(cudaMemcpyAsync(c->d_blob, c->blob.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->blob_dirty = false;
    return PCL_OK;
}

static StepArgs make_args(Ctx* c, double dt, int nsteps, int spill_mode, int sp_in) {
    StepArgs A;
    std::memset(&A, 0, sizeof(A));
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        A.xw[s] = S.xw[S.cur];
        A.ps[s] = S.ps[S.cur];
        A.meta[s] = S.meta[S.cur];
        A.cap[s] = S.cap;
        A.hist_n[s] = S.hist_n;
        A.hist_w[s] = S.hist_w;
    }
    int sp_out = 1 - sp_in;
    A.sp_in_xw = c->sp_xw[sp_in]; A.sp_in_ps = c->sp_ps[sp_in]; A.sp_in_meta = c->sp_meta[sp_in];
    A.sp_out_xw = c->sp_xw[sp_out]; A.sp_out_ps = c->sp_ps[sp_out]; A.sp_out_meta = c->sp_meta[sp_out];
    A.sp_cap = c->sp_cap;
    A.sp_in_n = c->d_spn + sp_in;
    A.sp_out_n = c->d_spn + sp_out;
    A.ctl = c->d_ctl;
    A.head = &c->d_ctl->head;
    A.blob = c->d_blob;
    for (size_t b = 0; b < c->sb.size(); ++b) A.sb_data[b] = c->sb[b].d_data;
    A.key0 = uint32_t(c->cfg.seed);
    A.key1 = uint32_t(c->cfg.seed >> 32);
    A.dt = dt;
    A.nsteps = nsteps;
    A.spill_mode = spill_mode;
    A.blob_bytes = int(c->blob.size());
    A.wall_xw = c->d_wall_xw; A.wall_pt = c->d_wall_pt; A.wall_meta = c->d_wall_meta;
    A.wall_n = c->d_wall_n; A.wall_cap = c->wall_cap;
    A.general = (c->field_kind != 0) ? 1 : 0;
    A.learn = c->learn_on ? 1 : 0;
    for (int s = 0; s < 3; ++s)
        if (c->sp[s].wall_coord >= 0 && c->wall_cap > 0) A.general = 1;
    A.event = (c->cfg.classic_step == 0) ? 1 : 0;
    if (c->learn_on) {  // suspended collisions go to queue 0 unless set_lq says otherwise
        A.lq_out_xw = c->lq_xw[0]; A.lq_out_ps = c->lq_ps[0]; A.lq_out_m1 = c->lq_m1[0]; A.lq_out_m2 = c->lq_m2[0];
        A.lq_out_n = c->d_lqn;
        A.lq_cap = c->lq_cap;
    }
    return A;
}

// Suspended-collision queues of a pass: output queue `out`, input queue `in` (-1: none).
static void set_lq(StepArgs& A, Ctx* c, int out, int in) {
    if (!c->learn_on) return;
    A.lq_out_xw = c->lq_xw[out]; A.lq_out_ps = c->lq_ps[out]; A.lq_out_m1 = c->lq_m1[out];
    A.lq_out_m2 = c->lq_m2[out]; A.lq_out_n = c->d_lqn + out;
    if (in >= 0) {
        A.lq_in_xw = c->lq_xw[in]; A.lq_in_ps = c->lq_ps[in]; A.lq_in_m1 = c->lq_m1[in]; A.lq_in_m2 = c->lq_m2[in];
        A.lq_in_n = c->d_lqn + in;
        A.lq_in_y = c->lq_y;
    }
    A.lq_cap = c->lq_cap;
}

static void free_lq(Ctx* c) {
    for (int b = 0; b < 2; ++b) {
        cudaFree(c->lq_xw[b]); cudaFree(c->lq_ps[b]); cudaFree(c->lq_m1[b]); cudaFree(c->lq_m2[b]);
        c->lq_xw[b] = c->lq_ps[b] = nullptr; c->lq_m1[b] = nullptr; c->lq_m2[b] = nullptr;
    }
    cudaFree(c->lq_x); cudaFree(c->lq_yk); cudaFree(c->lq_y); cudaFree(c->d_lqn);
    c->lq_x = c->lq_yk = c->lq_y = nullptr; c->d_lqn = nullptr;
    c->lq_cap = 0; c->lq_nets_cap = 0;
}

// Queues sized for 1/64 of the largest population (at least 64 Ki collisions);
// a full queue makes the step use the table sampler for the excess.
static int ensure_lq(Ctx* c) {
    if (!c->learn_on) return PCL_OK;
    long long capmax = 0;
    for (auto& s : c->sp) capmax = std::max(capmax, s.cap);
    long long want = std::max<long long>(1 << 16, capmax / 64);
    long long nn = std::max<long long>(1, (long long)c->nets.size());
    if (want <= c->lq_cap && nn <= c->lq_nets_cap) return PCL_OK;
    CK(cudaStreamSynchronize(c->stream));
    free_lq(c);
    for (int b = 0; b < 2; ++b) {
        CK(cudaMalloc(&c->lq_xw[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->lq_ps[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->lq_m1[b], sizeof(uint4) * want));
        CK(cudaMalloc(&c->lq_m2[b], sizeof(float4) * want));
    }
    CK(cudaMalloc(&c->lq_x, sizeof(float) * 2 * want));
    CK(cudaMalloc(&c->lq_yk, sizeof(float) * nn * want));
    CK(cudaMalloc(&c->lq_y, sizeof(float) * want));
    CK(cudaMalloc(&c->d_lqn, 2 * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
    c->lq_cap = want;
    c->lq_nets_cap = nn;
    return PCL_OK;
}

static int blocks_per_sm(Ctx* c) {
    if (c->cfg.classic_step == 0) return 3;   // the event kernel's stash leaves room for 3 blocks per SM
    int b = c->cfg.blocks_per_sm;
    return (b >= 2 && b <= 4) ? b : 4;
}

static int grid_blocks(Ctx* c) {
    if (c->cfg.grid_blocks > 0) return c->cfg.grid_blocks;
    return blocks_per_sm(c) * c->sm_count;
}

static int block_threads(Ctx* c) {
    int b = c->cfg.block_size > 0 ? c->cfg.block_size : 256;
    return std::min(256, std::max(32, (b / 32) * 32));
}

static int readback(Ctx* c) {
    CK(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PCL_OK;
}

// Device scratch of at least `bytes`, kept across calls (grown by doubling).
static int ensure_scratch(Ctx* c, size_t bytes) {
    if (bytes <= c->scr_bytes) return PCL_OK;
    const size_t nb = std::max(bytes, 2 * c->scr_bytes);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaFree(c->d_scr));
    c->d_scr = nullptr;
    c->scr_bytes = 0;
    CK(cudaMalloc(&c->d_scr, nb));
    c->scr_bytes = nb;
    return PCL_OK;
}

// The per-swarm population cap (pcl_set_swarm_cap) after a launch group:
// count the live particles of each swarm, then roulette the swarms above the
// cap, both on the context stream with the slot count read on the device.
// Removed particles stay as dead slots until the next compaction.
static int apply_swarm_caps(Ctx* c) {
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        if (c->swarm_cap[s] <= 0 || S.cap <= 0) continue;
        const int ns = std::max(1, c->nswarm);
        unsigned int* cnt = c->d_swcnt + 256 * s;
        const int grid = int(std::min<long long>((S.cap + 255) / 256, 4ll * c->sm_count));
        CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned int) * ns, c->stream));
        k_swarm_count<<<grid, 256, 0, c->stream>>>(S.meta[S.cur], &c->d_ctl->n[s], S.cap, ns, cnt);
        CK(cudaGetLastError());
        k_roulette_cap<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.meta[S.cur], &c->d_ctl->n[s], S.cap, cnt, ns,
                                                    (unsigned long long)c->swarm_cap[s], uint32_t(c->cfg.seed),
                                                    uint32_t(c->cfg.seed >> 32));
        CK(cudaGetLastError());
        c->launches += 2;
    }
    return PCL_OK;
}

static CompactArgs make_compact_args(Ctx* c) {
    CompactArgs C;
    std::memset(&C, 0, sizeof(C));
    long long capmax = 0;
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        int o = 1 - S.cur;
        C.sxw[s] = S.xw[S.cur]; C.sps[s] = S.ps[S.cur]; C.smeta[s] = S.meta[S.cur];
        C.dxw[s] = S.xw[o]; C.dps[s] = S.ps[o]; C.dmeta[s] = S.meta[o];
        C.tile_cnt[s] = c->d_tile_cnt + s * c->tiles_cap;
        C.tile_off[s] = c->d_tile_off + s * c->tiles_cap;
        capmax = std::max(capmax, S.cap);
    }
    C.n = c->d_ctl->n;
    C.n_out = c->d_nnew;
    C.ntiles_max = int(std::max<long long>(1, (capmax + kTile - 1) / kTile));
    return C;
}

// Enqueue the compaction (no host state change: the caller flips buffers).
static cudaError_t enqueue_compact(Ctx* c, const CompactArgs& C) {
    dim3 g(C.ntiles_max, 3);
    k_compact_count<<<g, 256, 0, c->stream>>>(C);
    k_compact_scan<<<3, 1024, 0, c->stream>>>(C);
    k_compact_scatter<<<g, 256, 0, c->stream>>>(C);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(c->d_ctl->n, c->d_nnew, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToDevice,
                           c->stream);
}

static void flip_buffers(Ctx* c) {
    for (int s = 0; s < 3; ++s)
        if (c->sp[s].cap > 0) c->sp[s].cur = 1 - c->sp[s].cur;
    c->steps_since_compact = 0;
}

static int compact_all(Ctx* c) {
    int rc = ensure_tiles(c);
    if (rc) return rc;
    CK(enqueue_compact(c, make_compact_args(c)));
    c->launches += 3;
    flip_buffers(c);
    return PCL_OK;
}

// The learned-sampler round, enqueued with no host read-back (so that it can
// be captured): the networks answer every collision suspended in queue 0 by
// the step and its two spill passes (network inputs, one batched tensor-core
// forward pass per attached network, the pick of each collision's network),
// then a resume pass finishes those collisions and carries the particles to
// the end of the launch, appending its overflow children to spill queue 1
// after what the spill passes left there, and two more spill passes drain
// it.  Every count is read on the device; the resume pass and the passes
// after it use the table sampler for any further collision (no suspension).
static cudaError_t enqueue_learned_round(Ctx* c, double dt, int nsteps, int minb, int threads, size_t smem) {
    const int g = int(std::max<long long>(1, std::min<long long>((c->lq_cap + 255) / 256, 2ll * c->sm_count)));
    const unsigned long long* nq = c->d_lqn;   // queue 0
    k_learn_x<<<g, 256, 0, c->stream>>>(c->lq_ps[0], c->lq_m2[0], nq, c->lq_cap, c->lq_x);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = mlp::infer_multi(c->nets.data(), int(c->nets.size()), c->lq_x, nq, c->lq_cap, c->lq_yk, c->lq_cap,
                             c->stream);
    if (e != cudaSuccess) return e;
    k_learn_pick<<<g, 256, 0, c->stream>>>(c->lq_m2[0], nq, c->lq_cap, c->lq_yk, c->lq_cap, c->pick, c->lq_y);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, nullptr, nullptr);   // work head only
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    StepArgs R = make_args(c, dt, nsteps, 2, 0);   // spill output: queue 1
    set_lq(R, c, 1, 0);
    R.lq_out_n = nullptr;
    // queue-driven passes take any grid: one block per SM
    if ((e = launch_step(minb, c->sm_count, threads, smem, c->stream, R)) != cudaSuccess) return e;
    for (int in = 1, pass = 0; pass < 2; ++pass, in = 1 - in) {
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + in, c->d_spn + (1 - in));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        StepArgs P = make_args(c, dt, nsteps, 1, in);
        P.lq_out_n = nullptr;
        if ((e = launch_step(minb, c->sm_count, threads, smem, c->stream, P)) != cudaSuccess) return e;
    }
    c->launches += 8 + ((long long)c->nets.size() + mlp::kMaxNets - 1) / mlp::kMaxNets;
    return cudaSuccess;
}

// Statistics of the learned round of the last launch group (queue 0's count
// read back with the control block).
static void count_learned(Ctx* c) {
    const long long m = std::min<long long>((long long)c->h_lqn[0], c->lq_cap);
    if (m > 0) {
        c->learn_rounds += 1;
        c->learn_suspended += m;
    }
}

// One launch group as a CUDA graph: prologue, step kernel, two spill passes
// (each a no-op when its queue is empty), the compaction when due, and the
// read-back of the control block and spill counts.  Graphs are cached by the
// bytes of every launch parameter, so a replay is identical to a fresh capture.
static int run_group_graph(Ctx* c, const StepArgs& A, const StepArgs& P0, const StepArgs& P1,
                           const CompactArgs* C, int minb, int grid, int threads, size_t smem) {
    std::vector<unsigned char> key;
    auto put = [&key](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        key.insert(key.end(), b, b + n);
    };
    put(&A, sizeof(A)); put(&P0, sizeof(P0)); put(&P1, sizeof(P1));
    int hdr[4] = {minb, grid, threads, (C ? 1 : 0) | (c->learn_on ? 2 : 0)};
    if (c->learn_on) {   // the learned round's networks and their pick table
        put(c->nets.data(), c->nets.size() * sizeof(void*));
        put(&c->pick, sizeof(c->pick));
        put(&c->lq_cap, sizeof(c->lq_cap));
    }
    put(hdr, sizeof(hdr)); put(&smem, sizeof(smem));
    if (C) put(C, sizeof(*C));
    long long caps[3] = {c->sp[0].cap, c->sp[1].cap, c->sp[2].cap};
    put(caps, sizeof(caps));
    cudaGraphExec_t exec = nullptr;
    for (auto& g : c->graphs)
        if (g.key == key) { exec = g.exec; break; }
    if (!exec) {
        CK(prepare_step(minb, smem, A.general != 0, A.event != 0, A.learn != 0));
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        auto q = [&e](cudaError_t r) { if (e == cudaSuccess) e = r; };
        k_begin<<<1, 64, 0, c->stream>>>(c->d_ctl, caps[0], caps[1], caps[2]);
        q(cudaGetLastError());
        q(cudaMemsetAsync(c->d_spn, 0, 2 * sizeof(unsigned long long), c->stream));
        if (c->learn_on) q(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
        // external records: event-record nodes that fire on every replay, so
        // the step kernel stays timed by events on its own stream
        q(cudaEventRecordWithFlags(c->ev_k0, c->stream, cudaEventRecordExternal));
        q(launch_step(minb, grid, threads, smem, c->stream, A));
        q(cudaEventRecordWithFlags(c->ev_k1, c->stream, cudaEventRecordExternal));
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 1, c->d_spn + 0);
        q(cudaGetLastError());
        q(launch_step(minb, grid, threads, smem, c->stream, P0));
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 0, c->d_spn + 1);
        q(cudaGetLastError());
        q(launch_step(minb, grid, threads, smem, c->stream, P1));
        const long long l0 = c->launches;
        if (c->learn_on) q(enqueue_learned_round(c, A.dt, A.nsteps, minb, threads, smem));
        c->launches = l0;   // counted per replay below
        if (C) q(enqueue_compact(c, *C));
        q(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
        q(cudaMemcpyAsync(c->h_spn, c->d_spn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
        if (c->learn_on)
            q(cudaMemcpyAsync(c->h_lqn, c->d_lqn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              c->stream));
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        CK(e);
        if (c->graphs.size() >= 8) {
            cudaGraphExecDestroy(c->graphs.front().exec);
            c->graphs.erase(c->graphs.begin());
        }
        c->graphs.push_back({std::move(key), exec});
    }
    CK(cudaGraphLaunch(exec, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->graph_launches += 1;
    c->launches += (C ? 11 : 8) +
                   (c->learn_on ? 8 + ((long long)c->nets.size() + mlp::kMaxNets - 1) / mlp::kMaxNets : 0);
    return PCL_OK;
}

// Spill passes: the queue written by the previous pass is the next pass's
// input, starting from spill queue `in`; suspended collisions of these passes
// go to learned queue `lq_out` (-1: none suspended).  *ran = whether any pass ran.
static int drain_spills(Ctx* c, double dt, int nsteps, int threads, size_t smem, int in, int lq_out, bool* ran,
                        const unsigned long long* known_pending) {
    for (int pass = 0; pass < 64; ++pass) {
        unsigned long long pending = 0;
        if (pass == 0 && known_pending) pending = *known_pending;
        else CK(d2h(c, &pending, c->d_spn + in, sizeof(pending)));
        if (pending == 0) return PCL_OK;
        *ran = true;
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + in, c->d_spn + (1 - in));
        StepArgs S = make_args(c, dt, nsteps, 1, in);
        if (lq_out >= 0) set_lq(S, c, lq_out, -1);
        else S.lq_out_n = nullptr;   // no suspension in these passes
        CK(launch_step(blocks_per_sm(c), grid_blocks(c), threads, smem, c->stream, S));
        c->launches += 2;
        in = 1 - in;
    }
    return fail(c, PCL_ERR_TIMEOUT, "spill passes did not drain");
}

// One launch of `nsteps` steps of length dt (seconds), plus spill passes and,
// with a learned sampler attached, the learned round.
static int launch_steps(Ctx* c, double dt_si, int nsteps) {
    int rc = build_blob(c);
    if (rc) return rc;
    if ((rc = ensure_spill(c))) return rc;
    if ((rc = ensure_lq(c))) return rc;
    const double dt = t_to_dev(dt_si);
    const int threads = block_threads(c);
    const size_t smem = step_smem_bytes(int(c->blob.size()), threads, c->cfg.classic_step == 0);
    const int period = c->cfg.compaction_period > 0 ? c->cfg.compaction_period : 8;
    const bool graph = c->cfg.use_graph != 0;
    bool compacted = false, host_passes = false;
    StepArgs A = make_args(c, dt, nsteps, 0, 0);
    c->launch_t0.push_back(c->t);   // k_begin advances the device launch counter to match
    unsigned long long pending0 = 0;
    if (graph) {
        const bool due = c->steps_since_compact + nsteps >= period;
        if (due && (rc = ensure_tiles(c))) return rc;
        CompactArgs C;
        if (due) C = make_compact_args(c);
        StepArgs P0 = make_args(c, dt, nsteps, 1, 1), P1 = make_args(c, dt, nsteps, 1, 0);
        if ((rc = run_group_graph(c, A, P0, P1, due ? &C : nullptr, blocks_per_sm(c), grid_blocks(c), threads,
                                  smem)))
            return rc;
        if (due) { flip_buffers(c); compacted = true; }
        pending0 = c->h_spn[1];  // the two in-graph passes leave the last queue written in 1
    } else {
        const int minb = blocks_per_sm(c);
        k_begin<<<1, 64, 0, c->stream>>>(c->d_ctl, c->sp[0].cap, c->sp[1].cap, c->sp[2].cap);
        CK(cudaMemsetAsync(c->d_spn, 0, 2 * sizeof(unsigned long long), c->stream));
        if (c->learn_on) CK(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
        CK(cudaEventRecord(c->ev_k0, c->stream));
        CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, A));
        CK(cudaEventRecord(c->ev_k1, c->stream));
        c->launches += 2;
        if (c->learn_on) {   // the graph's sequence: two spill passes, then the learned round
            StepArgs P0 = make_args(c, dt, nsteps, 1, 1), P1 = make_args(c, dt, nsteps, 1, 0);
            k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 1, c->d_spn + 0);
            CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P0));
            k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 0, c->d_spn + 1);
            CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P1));
            c->launches += 4;
            CK(enqueue_learned_round(c, dt, nsteps, minb, threads, smem));
            CK(cudaMemcpyAsync(c->h_lqn, c->d_lqn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c->stream));
        }
        CK(cudaMemcpyAsync(c->h_spn, c->d_spn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
        if ((rc = readback(c))) return rc;   // the one synchronisation of the group
        pending0 = c->h_spn[1];
    }
    if (c->learn_on) count_learned(c);
    {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, c->ev_k0, c->ev_k1));
        c->k_ms += ms;
        c->k_launches += 1;
        double nstart = 0, nout = 0, ndead = 0;
        for (int s = 0; s < 3; ++s) {
            nstart += double(c->h_ctl->n_start[s]);
            nout += double(c->h_ctl->live_end[nsteps - 1][s]);
            ndead += double(c->h_ctl->dead[s]);
        }
        c->k_bytes += 48.0 * nstart + 48.0 * nout + 4.0 * ndead;
    }
    // leftovers of the in-group passes (rare): host-driven passes, table sampler only
    if ((rc = drain_spills(c, dt, nsteps, threads, smem, 1, -1, &host_passes, &pending0))) return rc;
    // the last read-back holds the final counters unless host passes ran after it
    if (host_passes && (rc = readback(c))) return rc;
    if (c->h_ctl->timeout) return fail(c, PCL_ERR_TIMEOUT, "table staging wait timed out");
    c->t += dt_si * nsteps;
    c->steps += nsteps;
    for (int k = 0; k < nsteps; ++k) c->particle_steps += (long long)c->h_ctl->live_start[k];
    for (int s = 0; s < 3; ++s) c->live[s] = (long long)c->h_ctl->live_end[nsteps - 1][s];
    if (!compacted) {
        c->steps_since_compact += nsteps;
        if (c->steps_since_compact >= period) {
            if ((rc = compact_all(c))) return rc;
        }
    }
    if (c->h_ctl->err[PCL_E_CAPACITY] > 0) return fail(c, PCL_ERR_CAPACITY, "population capacity exceeded");
    return PCL_OK;
}

static int check_species(Ctx* c, int s) {
    if (s < 0 || s >= 3) return fail(c, PCL_ERR_INVALID, "species out of range");
    return PCL_OK;
}

}  // namespace pcl

using namespace pcl;

// =============================================================== C ABI ===
extern "C" {

const char* pcl_version(void) { return "particulator_gb300 0.1 (sm_103a)"; }

int pcl_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

const char* pcl_last_error(void* ctx) {
    if (!ctx) return noalloc_last_error();
    return static_cast<Ctx*>(ctx)->last_error.c_str();
}

int pcl_create(const pcl_config* cfg, void** out) {
    if (!cfg || !out) return PCL_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PCL_ERR_CUDA;
    if (cfg->device < 0 || cfg->device >= ndev) return PCL_ERR_INVALID;
    if (cfg->steps_per_launch > PCL_MAX_STEPS_PER_LAUNCH) return PCL_ERR_INVALID;
    Ctx* c = new Ctx();
    c->cfg = *cfg;
    c->device = cfg->device;
    if (cudaSetDevice(c->device) != cudaSuccess) { delete c; return PCL_ERR_CUDA; }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_ctl, sizeof(Control)) != cudaSuccess ||
        cudaMallocHost(&c->h_ctl, sizeof(Control)) != cudaSuccess ||
        cudaMallocHost(&c->h_spn, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost(&c->h_lqn, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&c->d_spn, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&c->d_nnew, 3 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&c->d_mom, 16 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c->d_swcnt, 3 * 256 * sizeof(unsigned int)) != cudaSuccess ||
        cudaEventCreate(&c->ev_k0) != cudaSuccess || cudaEventCreate(&c->ev_k1) != cudaSuccess ||
        cudaEventCreate(&c->ev_t0) != cudaSuccess || cudaEventCreate(&c->ev_t1) != cudaSuccess) {
        pcl_destroy(c);
        return PCL_ERR_CUDA;
    }
    cudaMemset(c->d_ctl, 0, sizeof(Control));
    cudaMemset(c->d_spn, 0, 2 * sizeof(unsigned long long));
    std::memset(c->h_ctl, 0, sizeof(Control));
    cudaDeviceSynchronize();
    *out = c;
    return PCL_OK;
}

void pcl_destroy(void* ctx) {
    if (!ctx) return;
    Ctx* c = static_cast<Ctx*>(ctx);
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& s : c->sp) free_species_buffers(s);
    for (auto& t : c->sb) cudaFree(t.d_data);
    for (int b = 0; b < 2; ++b) { cudaFree(c->sp_xw[b]); cudaFree(c->sp_ps[b]); cudaFree(c->sp_meta[b]); }
    cudaFree(c->d_spn); cudaFree(c->d_blob); cudaFree(c->d_ctl); cudaFree(c->d_tile_cnt);
    cudaFree(c->d_tile_off); cudaFree(c->d_nnew); cudaFree(c->d_mom); cudaFree(c->d_scr); cudaFree(c->d_swcnt);
    if (c->h_ctl) cudaFreeHost(c->h_ctl);
    if (c->h_spn) cudaFreeHost(c->h_spn);
    if (c->h_lqn) cudaFreeHost(c->h_lqn);
    for (cudaEvent_t e : c->io_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : c->io_tev) cudaEventDestroy(e);
    if (c->io_join) cudaEventDestroy(c->io_join);
    if (c->s_h2d) cudaStreamDestroy(c->s_h2d);
    if (c->s_d2h) cudaStreamDestroy(c->s_d2h);
    if (c->s_cmp) cudaStreamDestroy(c->s_cmp);
    cudaFree(c->d_heads);
    free_lq(c);
    cudaFree(c->d_wall_xw); cudaFree(c->d_wall_pt); cudaFree(c->d_wall_meta); cudaFree(c->d_wall_n);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    for (cudaEvent_t ev : {c->ev_k0, c->ev_k1, c->ev_t0, c->ev_t1})
        if (ev) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int pcl_set_species(void* ctx, int species, double energy_cut, int64_t capacity, int flags) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (capacity < 0 || capacity >= (1ll << 31)) return fail(c, PCL_ERR_INVALID, "capacity out of range");
    if (!(energy_cut >= 0)) return fail(c, PCL_ERR_INVALID, "energy cut must be >= 0");
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    CK(cudaStreamSynchronize(c->stream));
    free_species_buffers(S);
    S.set = true;
    S.cut = energy_cut;
    S.flags = flags;
    S.cap = (flags & PCL_SPECIES_TALLY_ONLY) ? 0 : capacity;
    S.cur = 0;
    if (S.cap > 0) {
        for (int b = 0; b < 2; ++b) {
            CK(cudaMalloc(&S.xw[b], sizeof(float4) * S.cap));
            CK(cudaMalloc(&S.ps[b], sizeof(float4) * S.cap));
            CK(cudaMalloc(&S.meta[b], sizeof(uint4) * S.cap));
        }
    }
    unsigned long long zero = 0;
    CK(h2d(c, &c->d_ctl->n[species], &zero, sizeof(zero)));
    c->live[species] = 0;
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_collision_table(void* ctx, int species, int order, int nproc, int nintervals, double xmax,
                            const double* rate, const double* ratebound, const pcl_process* procs) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (order < 1 || order > PCL_MAX_ORDER || nproc < 0 || nproc > PCL_MAX_PROC || nintervals < 1 ||
        nintervals > PCL_MAX_INTERVALS || !(xmax > 0) || !ratebound || (nproc > 0 && (!rate || !procs)))
        return fail(c, PCL_ERR_INVALID, "bad collision table");
    SpeciesState& S = c->sp[species];
    const int nI = nintervals + 1;
    S.table_kind = 0;
    S.order = order; S.nproc = nproc; S.nint = nintervals; S.xmax = xmax;
    S.rate.assign(rate, rate + size_t(order) * nproc * nI);
    if (nproc == 0) S.rate.clear();
    S.rb.assign(ratebound, ratebound + size_t(order) * nI);
    S.procs.assign(procs, procs + nproc);
    S.sb_index.assign(nproc, -1);
    CK(cudaSetDevice(c->device));
    for (int j = 0; j < nproc; ++j) {
        const pcl_process& P = procs[j];
        if (P.kind < PCL_PROC_MOLLER || P.kind > PCL_PROC_ATTACHMENT)
            return fail(c, PCL_ERR_UNSUPPORTED, "unsupported process kind");
        if (P.kind == PCL_PROC_SELTZER_BERGER) {
            if (!P.aux0 || !P.aux2 || P.naux < 2 || P.naux2 < 2)
                return fail(c, PCL_ERR_INVALID, "Seltzer-Berger process needs log_energy and data");
            int found = -1;
            // one device table per distinct inverse-CDF content (the reference's
            // SeltzerBerger struct carries no Z, and every Z shares one energy grid)
            for (size_t b = 0; b < c->sb.size(); ++b)
                if (c->sb[b].ne == P.naux && c->sb[b].ncum == P.naux2 &&
                    c->sb[b].log_energy == std::vector<double>(P.aux0, P.aux0 + P.naux) &&
                    c->sb[b].data == std::vector<double>(P.aux2, P.aux2 + size_t(P.naux) * P.naux2))
                    found = int(b);
            if (found < 0) {
                if (c->sb.size() >= PCL_MAX_SB) return fail(c, PCL_ERR_UNSUPPORTED, "too many SB tables");
                SBTable T;
                T.Z = P.Z; T.ne = P.naux; T.ncum = P.naux2;
                T.log_energy.assign(P.aux0, P.aux0 + P.naux);
                T.data.assign(P.aux2, P.aux2 + size_t(P.naux) * P.naux2);
                std::vector<float> f(size_t(T.ne) * T.ncum);
                for (size_t q = 0; q < f.size(); ++q) f[q] = float(P.aux2[q]);
                CK(cudaMalloc(&T.d_data, f.size() * sizeof(float)));
                CK(h2d(c, T.d_data, f.data(), f.size() * sizeof(float)));
                c->sb.push_back(T);
                found = int(c->sb.size()) - 1;
            }
            S.sb_index[j] = found;
        }
        if (P.kind == PCL_PROC_PHOTOELECTRIC && P.nparam < 1)
            return fail(c, PCL_ERR_INVALID, "photoelectric process needs binding energies");
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_linear_table(void* ctx, int species, int nproc, int n, double e0, double e1, const double* rate,
                         const double* ratebound, int nrb, const pcl_process* procs) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nproc < 0 || nproc > PCL_MAX_PROC || n < 2 || !(e1 > e0) || !ratebound || (nrb != 1 && nrb != n) ||
        (nproc > 0 && (!rate || !procs)))
        return fail(c, PCL_ERR_INVALID, "bad linear collision table");
    for (int j = 0; j < nproc; ++j)
        if (procs[j].kind != PCL_PROC_ELASTIC && procs[j].kind != PCL_PROC_EXCITATION &&
            procs[j].kind != PCL_PROC_NULL_COLLISION && procs[j].kind != PCL_PROC_REL_COULOMB &&
            procs[j].kind != PCL_PROC_IONIZATION && procs[j].kind != PCL_PROC_ATTACHMENT)
            return fail(c, PCL_ERR_UNSUPPORTED, "process kind not supported on a linear-grid table");
    SpeciesState& S = c->sp[species];
    S.table_kind = 1;
    S.nproc = nproc; S.order = 1; S.nint = 1; S.xmax = e1;
    S.lin_n = n; S.lin_e0 = e0; S.lin_e1 = e1;
    S.rate.assign(rate, rate + size_t(nproc) * n);
    S.rb.resize(n);
    for (int i = 0; i < n; ++i) S.rb[i] = ratebound[nrb == 1 ? 0 : i];
    S.procs.assign(procs, procs + nproc);
    S.sb_index.assign(nproc, -1);
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_forcing(void* ctx, const double E[3], const double B[3], int cl_order, int cl_k, double cl_xmax,
                    const double* cl_ec, const double* cl_pc) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !E || !B) return PCL_ERR_INVALID;
    if (cl_order < 0 || cl_order > PCL_MAX_ORDER) return fail(c, PCL_ERR_INVALID, "bad continuum order");
    for (int a = 0; a < 3; ++a) { c->E[a] = E[a]; c->B[a] = B[a]; }
    c->cl_order = cl_order;
    if (cl_order > 0) {
        if (cl_k < 1 || cl_k > PCL_MAX_INTERVALS || !(cl_xmax > 0) || !cl_ec || !cl_pc)
            return fail(c, PCL_ERR_INVALID, "bad continuum-loss table");
        c->cl_k = cl_k;
        c->cl_xmax = cl_xmax;
        c->cl_ec.assign(cl_ec, cl_ec + size_t(cl_order) * (cl_k + 1));
        c->cl_pc.assign(cl_pc, cl_pc + size_t(cl_order) * (cl_k + 1));
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_field(void* ctx, int kind, const double* params, int nparams) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    static const int need[4] = {0, 5, 7, 4};
    if (kind < 0 || kind > 3 || nparams < need[kind] || (need[kind] > 0 && !params))
        return fail(c, PCL_ERR_INVALID, "field kind or parameters");
    if (kind == 3 && !(params[0] > 0 && params[1] > 0 && params[2] > 0))
        return fail(c, PCL_ERR_INVALID, "confined double layer widths must be > 0");
    c->field_kind = kind;
    for (int i = 0; i < 8; ++i) c->field_p[i] = (i < need[kind]) ? params[i] : 0.0;
    c->blob_dirty = true;
    return PCL_OK;
}

static int get_n(Ctx* c, int species, long long& n);

int pcl_roulette(void* ctx, int species, double pkeep) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (!(pkeep > 0.0 && pkeep <= 1.0)) return fail(c, PCL_ERR_INVALID, "keep probability must be in (0, 1]");
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long n = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, n)) || n == 0) return rc;
    unsigned long long* killed = nullptr;
    CK(cudaMallocAsync(&killed, sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(killed, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((n + 255) / 256, 8ll * c->sm_count));
    k_roulette<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.meta[S.cur], n, float(pkeep), uint32_t(c->cfg.seed),
                                            uint32_t(c->cfg.seed >> 32), killed);
    CK(cudaGetLastError());
    unsigned long long hk = 0;
    CK(cudaMemcpyAsync(&hk, killed, sizeof(hk), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaFreeAsync(killed, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->live[species] = std::max<long long>(0, c->live[species] - (long long)hk);
    return PCL_OK;
}

int pcl_roulette_swarms(void* ctx, int species, int nswarm, const double* pkeep) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !pkeep || nswarm < 1 || nswarm > 256) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    std::vector<float> q(nswarm);
    for (int i = 0; i < nswarm; ++i) {
        if (!(pkeep[i] > 0.0)) return fail(c, PCL_ERR_INVALID, "keep probabilities must be > 0");
        q[i] = float(std::min(1.0, pkeep[i]));
    }
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long n = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, n)) || n == 0) return rc;
    if ((rc = ensure_scratch(c, 256 + sizeof(float) * nswarm))) return rc;
    unsigned long long* killed = static_cast<unsigned long long*>(c->d_scr);
    float* dq = reinterpret_cast<float*>(static_cast<char*>(c->d_scr) + 256);
    CK(cudaMemcpyAsync(dq, q.data(), sizeof(float) * nswarm, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(killed, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((n + 255) / 256, 8ll * c->sm_count));
    k_roulette_swarms<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.meta[S.cur], n, dq, nswarm,
                                                   uint32_t(c->cfg.seed), uint32_t(c->cfg.seed >> 32), killed);
    CK(cudaGetLastError());
    unsigned long long hk = 0;
    CK(cudaMemcpyAsync(&hk, killed, sizeof(hk), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->live[species] = std::max<long long>(0, c->live[species] - (long long)hk);
    return PCL_OK;
}

int pcl_split(void* ctx, int species, double p) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (!(p >= 0.0 && p <= 64.0)) return fail(c, PCL_ERR_INVALID, "mean number of copies must be in [0, 64]");
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long n = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, n)) || n == 0) return rc;
    unsigned long long* lost = nullptr;
    CK(cudaMallocAsync(&lost, sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(lost, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((n + 255) / 256, 8ll * c->sm_count));
    k_split<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], n, S.cap, float(p),
                                         uint32_t(c->cfg.seed), uint32_t(c->cfg.seed >> 32), &c->d_ctl->n[species],
                                         lost);
    CK(cudaGetLastError());
    unsigned long long hl = 0;
    CK(cudaMemcpyAsync(&hl, lost, sizeof(hl), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaFreeAsync(lost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    long long nn = 0;
    if ((rc = get_n(c, species, nn))) return rc;
    c->live[species] += nn - n;
    if (hl) return fail(c, PCL_ERR_CAPACITY, "split copies beyond the population capacity were lost");
    return PCL_OK;
}

int pcl_set_wall(void* ctx, int species, int coord, double v, int drop, int64_t capacity) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (coord < -1 || coord > 2 || capacity < 0 || capacity > (1ll << 30))
        return fail(c, PCL_ERR_INVALID, "wall axis or capacity");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    SpeciesState& S = c->sp[species];
    S.wall_coord = coord;
    S.wall_v = v;
    S.wall_drop = drop ? 1 : 0;
    if (coord >= 0 && capacity > c->wall_cap) {
        cudaFree(c->d_wall_xw); cudaFree(c->d_wall_pt); cudaFree(c->d_wall_meta); cudaFree(c->d_wall_n);
        c->d_wall_xw = c->d_wall_pt = nullptr; c->d_wall_meta = nullptr; c->d_wall_n = nullptr; c->wall_cap = 0;
        CK(cudaMalloc(&c->d_wall_xw, sizeof(float4) * capacity));
        CK(cudaMalloc(&c->d_wall_pt, sizeof(float4) * capacity));
        CK(cudaMalloc(&c->d_wall_meta, sizeof(uint4) * capacity));
        CK(cudaMalloc(&c->d_wall_n, sizeof(unsigned long long)));
        CK(cudaMemset(c->d_wall_n, 0, sizeof(unsigned long long)));
        c->wall_cap = capacity;
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_get_wall(void* ctx, int64_t* n, int32_t* species, uint64_t* sid, double* x, double* p, double* w, double* t) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !n) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    if (!c->d_wall_n) { *n = 0; return PCL_OK; }
    unsigned long long cnt = 0;
    CK(d2h(c, &cnt, c->d_wall_n, sizeof(cnt)));
    const long long m = std::min<long long>((long long)cnt, c->wall_cap);
    if (!species) { *n = m; return PCL_OK; }   // query
    if (*n < m) { *n = m; return fail(c, PCL_ERR_INVALID, "output arrays too short for the wall records"); }
    std::vector<float4> xw(m), pt(m);
    std::vector<uint4> meta(m);
    if (m > 0) {
        CK(d2h(c, xw.data(), c->d_wall_xw, sizeof(float4) * m));
        CK(d2h(c, pt.data(), c->d_wall_pt, sizeof(float4) * m));
        CK(d2h(c, meta.data(), c->d_wall_meta, sizeof(uint4) * m));
    }
    for (long long i = 0; i < m; ++i) {
        species[i] = int32_t(meta[i].z);
        sid[i] = uint64_t(meta[i].x) | (uint64_t(meta[i].y) << 32);
        x[3 * i] = xw[i].x; x[3 * i + 1] = xw[i].y; x[3 * i + 2] = xw[i].z;
        w[i] = xw[i].w;
        p[3 * i] = p_to_si(pt[i].x); p[3 * i + 1] = p_to_si(pt[i].y); p[3 * i + 2] = p_to_si(pt[i].z);
        const size_t li = std::min<size_t>(meta[i].w, c->launch_t0.size() - 1);
        t[i] = c->launch_t0[li] + double(pt[i].w) * NS;
    }
    *n = m;
    const unsigned long long zero = 0;
    CK(h2d(c, c->d_wall_n, &zero, sizeof(zero)));
    return (long long)cnt > c->wall_cap ? fail(c, PCL_ERR_CAPACITY, "wall records beyond capacity were lost")
                                         : PCL_OK;
}

static int get_n(Ctx* c, int species, long long& n) {
    unsigned long long nn = 0;
    CK(d2h(c, &nn, &c->d_ctl->n[species], sizeof(nn)));
    n = std::min<long long>((long long)nn, c->sp[species].cap);
    return PCL_OK;
}

int pcl_set_swarms(void* ctx, int nswarm, const double* E, const double* Fdt, double safety) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (nswarm < 0 || nswarm > 256 || (nswarm > 0 && (!E || !Fdt)) || !(safety >= 0))
        return fail(c, PCL_ERR_INVALID, "bad swarm description");
    c->nswarm = nswarm;
    c->swarm_safety = safety;
    if (nswarm > 0) {
        c->swarm_E.assign(E, E + 3 * size_t(nswarm));
        c->swarm_Fdt.assign(Fdt, Fdt + nswarm);
    } else {
        c->swarm_E.clear();
        c->swarm_Fdt.clear();
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_swarm_moments(void* ctx, int species, int nswarm, double* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nswarm < 1 || nswarm > 256) return fail(c, PCL_ERR_INVALID, "nswarm out of range");
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    const int len = 6 * nswarm;
    const int blocks = int(std::max<long long>(1, std::min<long long>(2ll * c->sm_count, (slots + 255) / 256)));
    if ((rc = ensure_scratch(c, sizeof(double) * len * (blocks + 1)))) return rc;
    double* d = static_cast<double*>(c->d_scr);
    double* part = d + len;
    if (slots > 0) {
        k_swarm_moments<<<blocks, 256, sizeof(double) * len, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur],
                                                                          slots, species, nswarm, part);
        CK(cudaGetLastError());
    } else {
        CK(cudaMemsetAsync(part, 0, sizeof(double) * len * blocks, c->stream));
    }
    k_swarm_reduce<<<(len + 255) / 256, 256, 0, c->stream>>>(part, blocks, len, d);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d, sizeof(double) * len, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < nswarm; ++k) out[6 * k + 2] = e_to_si(out[6 * k + 2]);
    return PCL_OK;
}

int pcl_energy_histogram(void* ctx, int species, int swarm, int nedges, const double* edges, int64_t* counts,
                         double* weights) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !edges || !counts || !weights) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nedges < 2 || nedges > PCL_MAX_HIST_EDGES) return fail(c, PCL_ERR_INVALID, "nedges out of range");
    if (swarm < -1 || swarm >= std::max(1, c->nswarm) || (swarm >= 0 && c->nswarm == 0))
        return fail(c, PCL_ERR_INVALID, "swarm out of range");
    std::vector<double> ed(nedges);
    for (int i = 0; i < nedges; ++i) {
        if (!(std::isfinite(edges[i]) && edges[i] >= 0.0) || (i > 0 && !(edges[i] > edges[i - 1])))
            return fail(c, PCL_ERR_INVALID, "edges must be finite, >= 0 and strictly increasing");
        ed[i] = e_to_dev(edges[i]);
    }
    const int nb = nedges - 1;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    std::vector<unsigned long long> hc(nb, 0ull);
    std::vector<double> hw(nb, 0.0);
    if (S.cap > 0) {
        // scratch: counts [nb] (u64), weights [nb], edges [nb + 1]
        if ((rc = ensure_scratch(c, sizeof(double) * (3 * size_t(nb) + 1)))) return rc;
        unsigned long long* dc = static_cast<unsigned long long*>(c->d_scr);
        double* dw = reinterpret_cast<double*>(dc + nb);
        double* de = dw + nb;
        CK(cudaMemcpyAsync(de, ed.data(), sizeof(double) * nedges, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemsetAsync(dc, 0, 2 * sizeof(double) * nb, c->stream));
        const size_t smem = sizeof(double) * (2 * size_t(nb) + 1) + sizeof(unsigned int) * nb;
        CK(cudaFuncSetAttribute(k_energy_hist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(sizeof(double) * (2 * PCL_MAX_HIST_EDGES) + 4 * PCL_MAX_HIST_EDGES)));
        const int grid = int(std::min<long long>((S.cap + 255) / 256, 2ll * c->sm_count));
        k_energy_hist<<<grid, 256, smem, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], &c->d_ctl->n[species],
                                                      S.cap, species, swarm, de, nb, dc, dw);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(hc.data(), dc, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(hw.data(), dw, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    for (int i = 0; i < nb; ++i) {
        counts[i] = (int64_t)hc[i];
        weights[i] = hw[i];
    }
    return PCL_OK;
}

int pcl_swarm_counts(void* ctx, int species, int nswarm, int64_t* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nswarm < 1 || nswarm > 256) return fail(c, PCL_ERR_INVALID, "nswarm out of range");
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    std::vector<unsigned int> h(nswarm, 0u);
    if (S.cap > 0) {
        unsigned int* cnt = c->d_swcnt + 256 * species;
        const int grid = int(std::min<long long>((S.cap + 255) / 256, 4ll * c->sm_count));
        CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned int) * nswarm, c->stream));
        k_swarm_count<<<grid, 256, 0, c->stream>>>(S.meta[S.cur], &c->d_ctl->n[species], S.cap, nswarm, cnt);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h.data(), cnt, sizeof(unsigned int) * nswarm, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    for (int k = 0; k < nswarm; ++k) out[k] = (int64_t)h[k];
    return PCL_OK;
}

int pcl_set_swarm_cap(void* ctx, int species, int64_t cap) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (cap < 0 || cap > (int64_t)0xffffffffll) return fail(c, PCL_ERR_INVALID, "cap out of range");
    c->swarm_cap[species] = (long long)cap;
    return PCL_OK;
}

int pcl_upload(void* ctx, int species, int64_t n, const double* x, const double* p, const double* w,
               const double* t, const double* s, const uint64_t* sid, uint64_t sid_base) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (!S.set || S.cap == 0) return fail(c, PCL_ERR_STATE, "species not set or tally-only");
    if (n < 0 || n > S.cap) return fail(c, PCL_ERR_CAPACITY, "upload exceeds capacity");
    if (n > 0 && (!x || !p || !w || !t)) return fail(c, PCL_ERR_INVALID, "null particle arrays");
    std::vector<float4> hx(n), hp(n);
    std::vector<uint4> hm(n);
    const uint32_t k0 = uint32_t(c->cfg.seed), k1 = uint32_t(c->cfg.seed >> 32);
    for (int64_t i = 0; i < n; ++i) {
        uint64_t id = sid ? sid[i] : sid_base + uint64_t(i);
        uint32_t ctr = 0;
        double sv;
        if (s) {
            sv = s[i];
        } else {  // s = nextcoll() drawn from the particle's own stream (electron.jl:30-33)
            uint32_t cc[4] = {0u, uint32_t(id), uint32_t(id >> 32), 0u};
            philox_host(cc, k0, k1);
            double u = double(((cc[0] >> 9) << 1) | 1u) * 5.9604644775390625e-8;
            sv = -std::log(u);
            ctr = 1;
        }
        hx[i] = make_float4(float(x[3 * i]), float(x[3 * i + 1]), float(x[3 * i + 2]), float(w[i]));
        hp[i] = make_float4(float(p_to_dev(p[3 * i])), float(p_to_dev(p[3 * i + 1])),
                            float(p_to_dev(p[3 * i + 2])), float(sv));
        float toff = float(t_to_dev(t[i] - c->t));
        uint32_t tb;
        std::memcpy(&tb, &toff, 4);
        hm[i] = make_uint4(uint32_t(id), uint32_t(id >> 32), ctr, tb);
    }
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (n > 0) {
        CK(h2d(c, S.xw[S.cur], hx.data(), sizeof(float4) * n));
        CK(h2d(c, S.ps[S.cur], hp.data(), sizeof(float4) * n));
        CK(h2d(c, S.meta[S.cur], hm.data(), sizeof(uint4) * n));
    }
    unsigned long long nn = (unsigned long long)n;
    CK(h2d(c, &c->d_ctl->n[species], &nn, sizeof(nn)));
    c->live[species] = n;
    return PCL_OK;
}


int pcl_download(void* ctx, int species, int64_t* n, double* x, double* p, double* w, double* t, double* s,
                 uint64_t* sid, uint32_t* ctr) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !n) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    std::vector<float4> hx(slots), hp(slots);
    std::vector<uint4> hm(slots);
    if (slots > 0) {
        CK(d2h(c, hx.data(), S.xw[S.cur], sizeof(float4) * slots));
        CK(d2h(c, hp.data(), S.ps[S.cur], sizeof(float4) * slots));
        CK(d2h(c, hm.data(), S.meta[S.cur], sizeof(uint4) * slots));
    }
    int64_t capn = *n, m = 0;
    for (long long i = 0; i < slots; ++i) {
        if (hm[i].z == PCL_DEAD_CTR) continue;
        if (m >= capn) return fail(c, PCL_ERR_CAPACITY, "download arrays too small");
        if (x) { x[3 * m] = hx[i].x; x[3 * m + 1] = hx[i].y; x[3 * m + 2] = hx[i].z; }
        if (p) {
            p[3 * m] = p_to_si(hp[i].x); p[3 * m + 1] = p_to_si(hp[i].y); p[3 * m + 2] = p_to_si(hp[i].z);
        }
        if (w) w[m] = hx[i].w;
        if (s) s[m] = hp[i].w;
        float toff;
        std::memcpy(&toff, &hm[i].w, 4);
        if (t) t[m] = c->t + t_to_si(toff);
        if (sid) sid[m] = uint64_t(hm[i].x) | (uint64_t(hm[i].y) << 32);
        if (ctr) ctr[m] = hm[i].z;
        ++m;
    }
    *n = m;
    return PCL_OK;
}

int pcl_upload_packed(void* ctx, int species, int64_t n, const pcl_packed* host) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !host) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (!S.set || S.cap == 0) return fail(c, PCL_ERR_STATE, "species not set or tally-only");
    if (n < 0 || n > S.cap) return fail(c, PCL_ERR_CAPACITY, "upload exceeds capacity");
    CK(cudaSetDevice(c->device));
    if (n > 0) {
        CK(cudaMemcpyAsync(S.xw[S.cur], host->xw, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(S.ps[S.cur], host->ps, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(S.meta[S.cur], host->meta, sizeof(uint4) * n, cudaMemcpyHostToDevice, c->stream));
    }
    unsigned long long nn = (unsigned long long)n;
    CK(cudaMemcpyAsync(&c->d_ctl->n[species], &nn, sizeof(nn), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->live[species] = n;
    return PCL_OK;
}

int pcl_download_packed(void* ctx, int species, int64_t* n, pcl_packed* host) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !host || !n) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    if (slots > *n) return fail(c, PCL_ERR_CAPACITY, "download arrays too small");
    if (slots > 0) {
        CK(cudaMemcpyAsync(host->xw, S.xw[S.cur], sizeof(float4) * slots, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(host->ps, S.ps[S.cur], sizeof(float4) * slots, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(host->meta, S.meta[S.cur], sizeof(uint4) * slots, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    *n = slots;
    return PCL_OK;
}

// Slots [a, b) of each species covered by concatenated indices [g0, g1) of
// the species ranges n[0], n[1], n[2] (the step kernel's work order).
static void chunk_ranges(const long long n[3], long long g0, long long g1, long long a[3], long long b[3]) {
    long long base = 0;
    for (int s = 0; s < 3; ++s) {
        a[s] = std::min(std::max(g0 - base, 0ll), n[s]);
        b[s] = std::min(std::max(g1 - base, 0ll), n[s]);
        base += n[s];
    }
}

static cudaError_t copy_slots(const SpeciesState& S, const pcl_packed& h, long long a, long long b, bool up,
                              cudaStream_t st) {
    if (b <= a) return cudaSuccess;
    const size_t n = size_t(b - a);
    cudaError_t e;
    if (up) {
        e = cudaMemcpyAsync(S.xw[S.cur] + a, reinterpret_cast<const float4*>(h.xw) + a, 16 * n,
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(S.ps[S.cur] + a, reinterpret_cast<const float4*>(h.ps) + a, 16 * n,
                                cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(S.meta[S.cur] + a, reinterpret_cast<const uint4*>(h.meta) + a, 16 * n,
                                cudaMemcpyHostToDevice, st);
    } else {
        e = cudaMemcpyAsync(reinterpret_cast<float4*>(h.xw) + a, S.xw[S.cur] + a, 16 * n, cudaMemcpyDeviceToHost,
                            st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(reinterpret_cast<float4*>(h.ps) + a, S.ps[S.cur] + a, 16 * n,
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(reinterpret_cast<uint4*>(h.meta) + a, S.meta[S.cur] + a, 16 * n,
                                cudaMemcpyDeviceToHost, st);
    }
    return e;
}

int pcl_advance_host(void* ctx, double tfinal, const int64_t* n_in, const pcl_packed* in, int64_t* n_out,
                     pcl_packed* out, const int64_t* out_cap, int nchunks, int compact) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !n_in || !in || !n_out || !out || !out_cap) return PCL_ERR_INVALID;
    if (!(tfinal > c->t)) return fail(c, PCL_ERR_INVALID, "tfinal must exceed the current time");
    if (nchunks < 1 || nchunks > 64) return fail(c, PCL_ERR_INVALID, "nchunks must be in [1, 64]");
    bool any = false;
    long long n[3];
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        any = any || S.set;
        n[s] = (S.set && S.cap > 0) ? (long long)n_in[s] : 0;
        if (n[s] < 0 || n[s] > S.cap) return fail(c, PCL_ERR_CAPACITY, "input exceeds capacity");
        if (n[s] > 0 && (!in[s].xw || !in[s].ps || !in[s].meta || !out[s].xw || !out[s].ps || !out[s].meta))
            return fail(c, PCL_ERR_INVALID, "null particle arrays");
    }
    if (!any) return fail(c, PCL_ERR_STATE, "no species set");
    CK(cudaSetDevice(c->device));
    // every return, error or not, leaves no copy into or out of the caller's
    // buffers in flight
    struct Drain {
        Ctx* c;
        ~Drain() {
            if (c->s_h2d) cudaStreamSynchronize(c->s_h2d);
            if (c->s_d2h) cudaStreamSynchronize(c->s_d2h);
            if (c->s_cmp) cudaStreamSynchronize(c->s_cmp);
            cudaStreamSynchronize(c->stream);
        }
    } drain{c};
    int rc = build_blob(c);
    if (rc || (rc = ensure_spill(c)) || (rc = ensure_lq(c))) return rc;
    if (!c->s_h2d) CK(cudaStreamCreateWithFlags(&c->s_h2d, cudaStreamNonBlocking));
    if (!c->s_d2h) CK(cudaStreamCreateWithFlags(&c->s_d2h, cudaStreamNonBlocking));
    if (!c->s_cmp) CK(cudaStreamCreateWithFlags(&c->s_cmp, cudaStreamNonBlocking));
    if (!c->io_join) CK(cudaEventCreateWithFlags(&c->io_join, cudaEventDisableTiming));
    if (!c->d_heads) CK(cudaMalloc(&c->d_heads, 64 * sizeof(unsigned long long)));
    while ((int)c->io_ev.size() < 2 * nchunks) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->io_ev.push_back(e);
        CK(cudaEventCreate(&e));
        c->io_tev.push_back(e);
    }
    const double dt_si = tfinal - c->t;
    const double dt = t_to_dev(dt_si);
    const int threads = block_threads(c);
    const size_t smem = step_smem_bytes(int(c->blob.size()), threads, c->cfg.classic_step == 0);
    const int minb = blocks_per_sm(c);
    // slot counts, then the step prologue (k_begin takes n_start from them)
    unsigned long long nn[3] = {(unsigned long long)n[0], (unsigned long long)n[1], (unsigned long long)n[2]};
    for (int s = 0; s < 3; ++s)
        CK(cudaMemcpyAsync(&c->d_ctl->n[s], &nn[s], sizeof(nn[s]), cudaMemcpyHostToDevice, c->stream));
    c->launch_t0.push_back(c->t);
    k_begin<<<1, 64, 0, c->stream>>>(c->d_ctl, c->sp[0].cap, c->sp[1].cap, c->sp[2].cap);
    CK(cudaMemsetAsync(c->d_spn, 0, 2 * sizeof(unsigned long long), c->stream));
    if (c->learn_on) CK(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->d_heads, 0, 64 * sizeof(unsigned long long), c->stream));
    CK(cudaStreamSynchronize(c->stream));   // the host counts above are stack memory
    // pipeline: upload chunk i (copy stream) -> step chunk i (a launch over its
    // range with its own work counter, on two alternating compute streams, so
    // that the tail of one launch overlaps the next) -> download chunk i's
    // slots, updated in place (copy stream), unless the population is
    // compacted afterwards.  Launches of different chunks touch disjoint
    // slots; appends, spills and tallies are atomic.
    {
        const StepArgs A0 = make_args(c, dt, 1, 0, 0);
        CK(prepare_step(minb, smem, A0.general != 0, A0.event != 0, A0.learn != 0));
    }
    const long long G = n[0] + n[1] + n[2];
    const long long cs = std::max<long long>(1, (G + nchunks - 1) / nchunks);
    int nch = int((G + cs - 1) / cs);
    for (int i = 0; i < nch; ++i) {
        const long long g0 = i * cs, g1 = std::min(G, g0 + cs);
        long long a[3], b[3];
        chunk_ranges(n, g0, g1, a, b);
        cudaEvent_t up = c->io_ev[2 * i], done = c->io_ev[2 * i + 1];
        for (int s = 0; s < 3; ++s) CK(copy_slots(c->sp[s], in[s], a[s], b[s], true, c->s_h2d));
        CK(cudaEventRecord(up, c->s_h2d));
        cudaStream_t cs_i = (i & 1) ? c->s_cmp : c->stream;
        CK(cudaStreamWaitEvent(cs_i, up, 0));
        StepArgs A = make_args(c, dt, 1, 0, 0);
        A.g_lo = g0;
        A.g_hi = g1;
        A.head = c->d_heads + i;
        CK(cudaEventRecord(c->io_tev[2 * i], cs_i));
        CK(launch_step_prepared(minb, grid_blocks(c), threads, smem, cs_i, A));
        CK(cudaEventRecord(c->io_tev[2 * i + 1], cs_i));
        c->launches += 1;
        CK(cudaEventRecord(done, cs_i));
        if (!compact) {
            CK(cudaStreamWaitEvent(c->s_d2h, done, 0));
            for (int s = 0; s < 3; ++s) CK(copy_slots(c->sp[s], out[s], a[s], b[s], false, c->s_d2h));
        }
    }
    // both compute streams joined, then the spill passes and the learned
    // round, as in a launch group
    CK(cudaEventRecord(c->io_join, c->s_cmp));
    CK(cudaStreamWaitEvent(c->stream, c->io_join, 0));
    {
        StepArgs P0 = make_args(c, dt, 1, 1, 1), P1 = make_args(c, dt, 1, 1, 0);
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 1, c->d_spn + 0);
        CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P0));
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 0, c->d_spn + 1);
        CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P1));
        c->launches += 4;
        if (c->learn_on) {
            CK(enqueue_learned_round(c, dt, 1, minb, threads, smem));
            CK(cudaMemcpyAsync(c->h_lqn, c->d_lqn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c->stream));
        }
        CK(cudaMemcpyAsync(c->h_spn, c->d_spn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           c->stream));
        if ((rc = readback(c))) return rc;
        if (c->learn_on) count_learned(c);
        for (int i = 0; i < nch; ++i) {   // step-kernel time of the chunk launches
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, c->io_tev[2 * i], c->io_tev[2 * i + 1]));
            c->k_ms += ms;
            c->k_launches += 1;
        }
        unsigned long long pending = c->h_spn[1];
        bool host_passes = false;
        if ((rc = drain_spills(c, dt, 1, threads, smem, 1, -1, &host_passes, &pending))) return rc;
        if (host_passes && (rc = readback(c))) return rc;
    }
    if (c->h_ctl->timeout) return fail(c, PCL_ERR_TIMEOUT, "table staging wait timed out");
    c->t = tfinal;
    c->steps += 1;
    c->particle_steps += (long long)c->h_ctl->live_start[0];
    for (int s = 0; s < 3; ++s) c->live[s] = (long long)c->h_ctl->live_end[0][s];
    if (c->h_ctl->err[PCL_E_CAPACITY] > 0) return fail(c, PCL_ERR_CAPACITY, "population capacity exceeded");
    if (compact) {
        if ((rc = compact_all(c)) || (rc = readback(c))) return rc;
        for (int s = 0; s < 3; ++s) n[s] = 0;   // everything is downloaded below
    } else {
        c->steps_since_compact += 1;
    }
    // the rest: appended secondaries (or the whole compacted population)
    long long nf[3];
    for (int s = 0; s < 3; ++s) {
        nf[s] = (c->sp[s].set && c->sp[s].cap > 0) ? std::min<long long>((long long)c->h_ctl->n[s], c->sp[s].cap) : 0;
        if (nf[s] > out_cap[s]) return fail(c, PCL_ERR_CAPACITY, "output arrays too small");
    }
    for (int s = 0; s < 3; ++s) CK(copy_slots(c->sp[s], out[s], n[s], nf[s], false, c->s_d2h));
    CK(cudaStreamSynchronize(c->s_d2h));
    for (int s = 0; s < 3; ++s) n_out[s] = nf[s];
    return PCL_OK;
}

int pcl_host_register(void* ptr, size_t bytes) {
    if (!ptr || bytes == 0) return PCL_ERR_INVALID;
    return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? PCL_OK : PCL_ERR_CUDA;
}

int pcl_host_unregister(void* ptr) {
    if (!ptr) return PCL_ERR_INVALID;
    return cudaHostUnregister(ptr) == cudaSuccess ? PCL_OK : PCL_ERR_CUDA;
}

int pcl_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return PCL_ERR_INVALID;
    *ptr = nullptr;
    if (bytes == 0) return PCL_ERR_INVALID;
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) return PCL_ERR_CUDA;
    *ptr = p;
    return PCL_OK;
}

int pcl_host_free(void* ptr) {
    if (!ptr) return PCL_ERR_INVALID;
    return cudaFreeHost(ptr) == cudaSuccess ? PCL_OK : PCL_ERR_CUDA;
}

int pcl_advance(void* ctx, double tfinal) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (!(tfinal > c->t)) return fail(c, PCL_ERR_INVALID, "tfinal must exceed the current time");
    bool any = false;
    for (auto& s : c->sp) any = any || s.set;
    if (!any) return fail(c, PCL_ERR_STATE, "no species set");
    CK(cudaSetDevice(c->device));
    return launch_steps(c, tfinal - c->t, 1);
}

int pcl_run(void* ctx, double tfinal, double dt, const pcl_run_opts* opts, pcl_tallies* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (!(dt > 0)) return fail(c, PCL_ERR_INVALID, "dt must be > 0");
    CK(cudaSetDevice(c->device));
    const int K = std::max(1, c->cfg.steps_per_launch);
    // run.jl:6-27 steps while t < tfinal; the step count is fixed once, with a
    // tolerance, so that accumulated rounding of the clock never adds a step
    const long long total = (long long)std::ceil((tfinal - c->t) / dt - 1e-6);
    long long done = 0;
    while (done < total) {
        // advance!, droplow!, onstep (population target)
        int ns = int(std::min<long long>(K, total - done));
        if (opts && opts->max_steps > 0) ns = int(std::min<long long>(ns, opts->max_steps - done));
        if (ns <= 0) break;
        int rc = launch_steps(c, dt, ns);
        if (rc || (rc = apply_swarm_caps(c))) return rc;
        done += ns;
        if (done == total && std::fabs(c->t - tfinal) < 1e-6 * dt) c->t = tfinal;
        if (opts && opts->target_species >= 0 && opts->target_species < 3) {
            long long live = c->live[opts->target_species];
            bool cont = opts->target_ismax ? (live < opts->target_n) : (live > opts->target_n);
            if (!cont) break;
        }
        if (opts && opts->max_steps > 0 && done >= opts->max_steps) break;
    }
    if (out) return pcl_get_tallies(ctx, out);
    return PCL_OK;
}

int pcl_get_tallies(void* ctx, pcl_tallies* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    int rc = readback(c);
    if (rc) return rc;
    std::memset(out, 0, sizeof(*out));
    const Control& C = *c->h_ctl;
    out->t = c->t;
    out->steps = c->steps;
    out->particle_steps = c->particle_steps;
    for (int s = 0; s < 3; ++s) {
        out->n[s] = std::min<long long>((long long)C.n[s], c->sp[s].cap);
        out->live[s] = c->live[s];
        for (int j = 0; j < PCL_MAX_PROC; ++j) out->collisions[s][j] = (long long)C.coll[s][j];
        out->nulls[s] = (long long)C.nulls[s];
        out->spawned[s] = (long long)C.spawned[s];
        out->tally_count[s] = (long long)C.tally_count[s];
        out->tally_w[s] = C.tally_w[s];
        out->tally_wE[s] = e_to_si(C.tally_wE[s]);
    }
    for (int e = 0; e < PCL_NERR; ++e) out->errors[e] = (long long)C.err[e];
    return PCL_OK;
}

int pcl_reset_tallies(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    int rc = readback(c);
    if (rc) return rc;
    Control keep = *c->h_ctl;
    Control z;
    std::memset(&z, 0, sizeof(z));
    for (int s = 0; s < 3; ++s) z.n[s] = keep.n[s];
    CK(h2d(c, c->d_ctl, &z, sizeof(z)));
    c->particle_steps = 0;
    for (auto& S : c->sp) {
        if (S.hist_bins > 0) {
            CK(cudaMemsetAsync(S.hist_n, 0, sizeof(unsigned long long) * S.hist_bins, c->stream));
            CK(cudaMemsetAsync(S.hist_w, 0, sizeof(double) * S.hist_bins, c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
    }
    return PCL_OK;
}

int pcl_moments(void* ctx, int species, double out[10]) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    CK(cudaMemsetAsync(c->d_mom, 0, 10 * sizeof(double), c->stream));
    if (slots > 0) {
        int blocks = int(std::min<long long>(4 * c->sm_count, (slots + 255) / 256));
        k_moments<<<blocks, 256, 0, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], slots, species,
                                                   c->d_mom);
        CK(cudaGetLastError());
    }
    double h[10];
    CK(cudaMemcpyAsync(h, c->d_mom, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < 8; ++q) out[q] = h[q];
    out[1] = e_to_si(h[1]);
    out[8] = e_to_si(h[8]);
    unsigned long long live;
    std::memcpy(&live, &h[9], 8);
    out[9] = double(live);
    return PCL_OK;
}

int pcl_compact(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    int rc = compact_all(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return PCL_OK;
}

int pcl_set_tally_histogram(void* ctx, int species, int nbins, double emin, double emax) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nbins < 0 || nbins > (1 << 16) || (nbins > 0 && !(emin > 0 && emax > emin)))
        return fail(c, PCL_ERR_INVALID, "bad histogram");
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    cudaFree(S.hist_n); cudaFree(S.hist_w);
    S.hist_n = nullptr; S.hist_w = nullptr;
    S.hist_bins = nbins; S.hist_emin = emin; S.hist_emax = emax;
    if (nbins > 0) {
        CK(cudaMalloc(&S.hist_n, sizeof(unsigned long long) * nbins));
        CK(cudaMalloc(&S.hist_w, sizeof(double) * nbins));
        CK(cudaMemsetAsync(S.hist_n, 0, sizeof(unsigned long long) * nbins, c->stream));
        CK(cudaMemsetAsync(S.hist_w, 0, sizeof(double) * nbins, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_get_tally_histogram(void* ctx, int species, int nbins, int64_t* counts, double* weights) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (nbins != S.hist_bins) return fail(c, PCL_ERR_INVALID, "bin count mismatch");
    if (nbins == 0) return PCL_OK;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (counts) CK(d2h(c, counts, S.hist_n, sizeof(int64_t) * nbins));
    if (weights) CK(d2h(c, weights, S.hist_w, sizeof(double) * nbins));
    return PCL_OK;
}

int pcl_sync(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return PCL_OK;
}

int pcl_timer_start(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaEventRecord(c->ev_t0, c->stream));
    return PCL_OK;
}

int pcl_timer_stop(void* ctx, double* ms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !ms) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaEventRecord(c->ev_t1, c->stream));
    CK(cudaEventSynchronize(c->ev_t1));
    float f = 0.0f;
    CK(cudaEventElapsedTime(&f, c->ev_t0, c->ev_t1));
    *ms = f;
    return PCL_OK;
}

int pcl_kernel_stats(void* ctx, double* step_kernel_ms, int64_t* step_launches, int64_t* launches,
                     double* step_bytes, int reset) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (step_kernel_ms) *step_kernel_ms = c->k_ms;
    if (step_launches) *step_launches = c->k_launches;
    if (launches) *launches = c->launches;
    if (step_bytes) *step_bytes = c->k_bytes;
    if (reset) { c->k_ms = 0; c->k_launches = 0; c->launches = 0; c->k_bytes = 0; }
    return PCL_OK;
}

static int learn_kind_ok(const pcl_process& P, int kind) {
    return (kind == PCL_LEARN_SB && P.kind == PCL_PROC_SELTZER_BERGER) ||
           (kind == PCL_LEARN_MOLLER && P.kind == PCL_PROC_MOLLER);
}

int pcl_set_learned(void* ctx, int species, int proc_index, int kind, void* mlp) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (proc_index < 0 || proc_index >= S.nproc || proc_index >= 16) return fail(c, PCL_ERR_INVALID, "process index");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (!mlp) {
        c->learn_net[species][proc_index] = nullptr;
        c->learn_kind[species][proc_index] = 0;
        c->learn_ok[species][proc_index][0] = c->learn_ok[species][proc_index][1] = 0u;
    } else {
        if (!learn_kind_ok(S.procs[proc_index], kind))
            return fail(c, PCL_ERR_UNSUPPORTED, "learned sampler kind does not match the process");
        // where the network is monotone in u: 64 bins of a, 4 energies each, 257 values of u
        const int nb = 64, ne = 4, nu = 257;
        std::vector<float> x(2 * nb * ne * nu), y(nb * ne * nu);
        for (int b = 0; b < nb; ++b)
            for (int e = 0; e < ne; ++e)
                for (int i = 0; i < nu; ++i) {
                    size_t r = (size_t(b) * ne + e) * nu + i;
                    x[2 * r] = -1.0f + (float(b) + (float(e) + 0.5f) / ne) * (2.0f / nb);
                    x[2 * r + 1] = 2.0f * (float(i) + 0.5f) / nu - 1.0f;
                }
        rc = pcl_mlp_forward(mlp, int64_t(y.size()), x.data(), y.data());
        if (rc) return fail(c, rc, std::string("network evaluation: ") + pcl_mlp_last_error(mlp));
        uint32_t ok[2] = {0u, 0u};
        for (int b = 0; b < nb; ++b) {
            bool mono = true;
            for (int e = 0; e < ne && mono; ++e)
                for (int i = 1; i < nu && mono; ++i) {
                    size_t r = (size_t(b) * ne + e) * nu + i;
                    if (!(y[r] >= y[r - 1]) || !std::isfinite(y[r])) mono = false;
                }
            if (mono) ok[b >> 5] |= 1u << (b & 31);
        }
        c->learn_net[species][proc_index] = mlp;
        c->learn_kind[species][proc_index] = kind;
        c->learn_ok[species][proc_index][0] = ok[0];
        c->learn_ok[species][proc_index][1] = ok[1];
    }
    // distinct networks and the pick table
    c->nets.clear();
    for (int k = 0; k < 48; ++k) c->pick.net[k] = -1;
    for (int sp = 0; sp < 3; ++sp)
        for (int j = 0; j < 16; ++j) {
            void* n = c->learn_net[sp][j];
            if (!n) continue;
            int idx = -1;
            for (size_t q = 0; q < c->nets.size(); ++q)
                if (c->nets[q] == n) idx = int(q);
            if (idx < 0) { idx = int(c->nets.size()); c->nets.push_back(n); }
            c->pick.net[sp * 16 + j] = int8_t(idx);
        }
    c->learn_on = !c->nets.empty();
    c->blob_dirty = true;
    return ensure_lq(c);
}

int pcl_learn_data(void* ctx, int species, int proc_index, int kind, int nT, int64_t per_T, int Q, uint64_t seed,
                   float* x_out, float* t_out, int64_t* nrows) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (proc_index < 0 || proc_index >= S.nproc) return fail(c, PCL_ERR_INVALID, "process index");
    if (nT < 2 || nT > 65536 || per_T < 1 || Q < 2 || !x_out || !t_out || !nrows)
        return fail(c, PCL_ERR_INVALID, "learn_data sizes");
    const pcl_process& P = S.procs[proc_index];
    if (!learn_kind_ok(P, kind)) return fail(c, PCL_ERR_UNSUPPORTED, "learned sampler kind does not match the process");
    CK(cudaSetDevice(c->device));
    if ((rc = build_blob(c))) return rc;
    const int nbins = 4096;
    const float hmin = 0.0f, hmax = 1.0f;   // both output variables lie in [0, 1]
    unsigned int* hist = nullptr;
    const size_t hn = size_t(nT) * nbins;
    CK(cudaMallocAsync(&hist, sizeof(unsigned int) * hn, c->stream));
    CK(cudaMemsetAsync(hist, 0, sizeof(unsigned int) * hn, c->stream));
    StepArgs A = make_args(c, 0.0, 1, 0, 0);
    const size_t smem = c->blob.size() + 16;
    CK(cudaFuncSetAttribute(k_learn_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const long long total = (long long)nT * per_T;
    const int grid = int(std::max<long long>(1, std::min<long long>((total + 255) / 256, 8ll * c->sm_count)));
    const unsigned long long sid_base = (0xA5ull << 56) | ((seed & 0xFFFFull) << 40);
    k_learn_hist<<<grid, 256, smem, c->stream>>>(A, species, proc_index, kind, nT, (long long)per_T, nbins, hmin, hmax,
                                                  sid_base, hist);
    CK(cudaGetLastError());
    std::vector<unsigned int> h(hn);
    CK(cudaMemcpyAsync(h.data(), hist, sizeof(unsigned int) * hn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaFreeAsync(hist, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const double dh = double(hmax - hmin) / nbins;
    int64_t r = 0;
    std::vector<double> cum(nbins + 1);
    for (int g = 0; g < nT; ++g) {
        const double a = -1.0 + 2.0 * g / double(nT - 1);
        if (kind == PCL_LEARN_MOLLER) {
            const double T = std::pow(10.0, 6.0 + 2.0 * a) * si::e;
            if (!(P.param[0] < 0.45 * T)) continue;   // degenerate kinematic range: no rows
        }
        const unsigned int* hg = h.data() + size_t(g) * nbins;
        cum[0] = 0.0;
        for (int b = 0; b < nbins; ++b) cum[b + 1] = cum[b] + hg[b];
        const double N = cum[nbins];
        if (N <= 0) continue;
        int b = 0;
        for (int i = 0; i < Q; ++i) {
            const double u = (i + 0.5) / Q;
            const double target = u * N;
            while (b < nbins - 1 && cum[b + 1] < target) ++b;
            const double f = hg[b] ? (target - cum[b]) / hg[b] : 0.5;
            x_out[2 * r] = float(a);
            x_out[2 * r + 1] = float(2.0 * u - 1.0);
            t_out[r] = float(hmin + (b + std::min(1.0, std::max(0.0, f))) * dh);
            ++r;
        }
    }
    *nrows = r;
    return PCL_OK;
}

int pcl_autotune(void* ctx, double dt, int32_t steps_budget, pcl_tune_result* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !(dt > 0) || steps_budget < 16) return PCL_ERR_INVALID;
    bool any = false;
    for (auto& sp : c->sp) any = any || sp.set;
    if (!any) return fail(c, PCL_ERR_STATE, "no species set");
    CK(cudaSetDevice(c->device));
    // step kernel: 0 = event, 2-4 = classic with that many blocks per SM
    const int bps_c[] = {0, 2, 3, 4}, k_c[] = {1, 2, 4, 8, 16}, per_c[] = {2, 4, 8, 16, 32}, g_c[] = {0, 1};
    const int ntrials = 4 + 5 + 5 + 2;
    // steps per trial: a multiple of the largest steps-per-launch and period tried
    int len = std::max(32, (steps_budget / ntrials) / 32 * 32);
    pcl_config best = c->cfg;
    best.blocks_per_sm = (c->cfg.classic_step == 0) ? 4 : blocks_per_sm(c);
    if (best.steps_per_launch < 1) best.steps_per_launch = 1;
    if (best.compaction_period < 1) best.compaction_period = 8;
    double best_rate = -1.0;
    int trials = 0, done = 0;
    auto trial = [&](const pcl_config& cfg, double& rate) -> int {
        c->cfg = cfg;
        int rc = compact_all(c);   // every trial starts from a compacted population
        if (rc) return rc;
        const long long ps0 = c->particle_steps;
        CK(cudaEventRecord(c->ev_t0, c->stream));
        int left = len;
        while (left > 0) {
            int ns = std::min(left, std::max(1, cfg.steps_per_launch));
            if ((rc = launch_steps(c, dt, ns))) return rc;
            left -= ns;
        }
        CK(cudaEventRecord(c->ev_t1, c->stream));
        CK(cudaEventSynchronize(c->ev_t1));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, c->ev_t0, c->ev_t1));
        rate = double(c->particle_steps - ps0) / (double(ms) * 1e-3);
        done += len;
        ++trials;
        return PCL_OK;
    };
    auto consider = [&](pcl_config cfg) -> int {
        if (done + len > steps_budget) return PCL_OK;
        double r = 0.0;
        int rc = trial(cfg, r);
        if (rc) return rc;
        if (r > best_rate) { best_rate = r; best = cfg; }
        return PCL_OK;
    };
    int rc = PCL_OK;
    for (int v : bps_c) {
        pcl_config q = best;
        q.classic_step = (v == 0) ? 0 : 1;
        q.blocks_per_sm = (v == 0) ? 4 : v;
        if ((rc = consider(q))) return rc;
    }
    const pcl_config after_bps = best;
    for (int v : k_c) { pcl_config q = after_bps; q.steps_per_launch = v; if ((rc = consider(q))) return rc; }
    const pcl_config after_k = best;
    for (int v : per_c) { pcl_config q = after_k; q.compaction_period = v; if ((rc = consider(q))) return rc; }
    const pcl_config after_p = best;
    for (int v : g_c) { pcl_config q = after_p; q.use_graph = v; if ((rc = consider(q))) return rc; }
    c->cfg = best;
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->blocks_per_sm = best.classic_step ? best.blocks_per_sm : 0;
        out->steps_per_launch = best.steps_per_launch;
        out->compaction_period = best.compaction_period;
        out->use_graph = best.use_graph;
        out->rate = best_rate;
        out->trials = trials;
        out->steps = done;
    }
    return PCL_OK;
}

int pcl_set_launch(void* ctx, int32_t bps, int32_t spl, int32_t period, int32_t use_graph) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !(bps == 0 || (bps >= 2 && bps <= 4)) || spl < 1 || spl > PCL_MAX_STEPS_PER_LAUNCH || period < 1 ||
        (use_graph != 0 && use_graph != 1))
        return PCL_ERR_INVALID;
    c->cfg.classic_step = (bps == 0) ? 0 : 1;
    c->cfg.blocks_per_sm = (bps == 0) ? 4 : bps;
    c->cfg.steps_per_launch = spl;
    c->cfg.compaction_period = period;
    c->cfg.use_graph = use_graph;
    return PCL_OK;
}

int pcl_learn_stats(void* ctx, int64_t* suspended, int64_t* rounds) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (suspended) *suspended = c->learn_suspended;
    if (rounds) *rounds = c->learn_rounds;
    return PCL_OK;
}

int pcl_test_sampler(void* ctx, int species, int proc_index, int64_t n, const double* p, const uint64_t* sid,
                     double* out_p, double* out_s, int32_t* out_kind, uint32_t* out_ctr) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (proc_index < 0 || proc_index >= S.nproc) return fail(c, PCL_ERR_INVALID, "process index");
    if (n <= 0 || !p || !sid || !out_p || !out_s || !out_kind || !out_ctr) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    if ((rc = build_blob(c))) return rc;
    std::vector<float> hp(3 * n);
    std::vector<uint32_t> hs(2 * n);
    for (int64_t i = 0; i < 3 * n; ++i) hp[i] = float(p_to_dev(p[i]));
    for (int64_t i = 0; i < n; ++i) { hs[2 * i] = uint32_t(sid[i]); hs[2 * i + 1] = uint32_t(sid[i] >> 32); }
    float *dp = nullptr, *dop = nullptr, *dos = nullptr;
    uint32_t *dsid = nullptr, *dctr = nullptr;
    int* dkind = nullptr;
    CK(cudaMalloc(&dp, sizeof(float) * 3 * n));
    CK(cudaMalloc(&dsid, sizeof(uint32_t) * 2 * n));
    CK(cudaMalloc(&dop, sizeof(float) * 9 * n));
    CK(cudaMalloc(&dos, sizeof(float) * 3 * n));
    CK(cudaMalloc(&dkind, sizeof(int) * 3 * n));
    CK(cudaMalloc(&dctr, sizeof(uint32_t) * n));
    CK(h2d(c, dp, hp.data(), sizeof(float) * 3 * n));
    CK(h2d(c, dsid, hs.data(), sizeof(uint32_t) * 2 * n));
    CK(cudaMemsetAsync(dop, 0, sizeof(float) * 9 * n, c->stream));
    CK(cudaMemsetAsync(dos, 0, sizeof(float) * 3 * n, c->stream));
    StepArgs A = make_args(c, 0.0, 1, 0, 0);
    size_t smem = c->blob.size() + 16;
    CK(cudaFuncSetAttribute(k_test_sampler, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int blocks = int((n + 127) / 128);
    k_test_sampler<<<blocks, 128, smem, c->stream>>>(A, species, proc_index, n, dp, dsid, dop, dos, dkind, dctr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    std::vector<float> hop(9 * n), hos(3 * n);
    CK(d2h(c, hop.data(), dop, sizeof(float) * 9 * n));
    CK(d2h(c, hos.data(), dos, sizeof(float) * 3 * n));
    CK(d2h(c, out_kind, dkind, sizeof(int) * 3 * n));
    CK(d2h(c, out_ctr, dctr, sizeof(uint32_t) * n));
    for (int64_t i = 0; i < 9 * n; ++i) out_p[i] = p_to_si(hop[i]);
    for (int64_t i = 0; i < 3 * n; ++i) out_s[i] = hos[i];
    cudaFree(dp); cudaFree(dsid); cudaFree(dop); cudaFree(dos); cudaFree(dkind); cudaFree(dctr);
    return PCL_OK;
}

}  // extern "C"
