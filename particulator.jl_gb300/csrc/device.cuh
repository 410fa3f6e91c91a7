// Types shared by the host context code and the device step kernels.
//
// HBM layout of a population (one per species, double-buffered for
// compaction): three arrays of 16-byte records, slot i of each holding
//   xw[i]   = {x, y, z (m), w}
//   ps[i]   = {px, py, pz (m_e c), s}
//   meta[i] = {sid_lo, sid_hi, ctr, t_off bits}
// 48 B per particle, one 128-bit load per record (float4-vectorised, fully
// coalesced when consecutive lanes hold consecutive slots).  A slot whose ctr
// is DEAD_CTR is a removed particle (remove_particle!, population.jl:120-122);
// the step updates particles in place and appends secondaries, and the
// compaction kernels (repack!, population.jl:229-259) squeeze dead slots out.
//
// The per-species collision tables, continuum-loss fits and process
// parameters are packed on the host into one "table blob" that every block
// copies into shared memory with one cp.async.bulk at kernel start.
#pragma once
#include <stdint.h>

#define PCL_DEAD_CTR 0xFFFFFFFFu
#define PCL_MAX_STEPS_PER_LAUNCH 64

namespace pcl {

// Device view of one process (normalised units).
struct DevProc {
    int32_t kind;
    int32_t sb;       // Seltzer-Berger table index, -1 otherwise
    int32_t nbind;    // photoelectric: number of binding energies
    int32_t learn;    // learned sampler: 0 none, PCL_LEARN_SB, PCL_LEARN_MOLLER
    float   p[8];     // kind-specific, see ctx.cu:pack_proc
    uint32_t learn_ok[2];  // 64 bins of a = (log10(T/eV) - 6) / 2 over [-1, 1): network used where set
    uint32_t pad[2];
};

struct SpeciesHdr {
    int32_t nproc;
    int32_t order;
    int32_t k;            // binary intervals of the collision table
    int32_t tally_only;
    float   xscale;       // 1 / xmax (normalised energy)
    float   cut;          // energy cut (m_e c^2)
    int32_t rate_off;     // float offset of rate[i][j][order] in the blob
    int32_t rb_off;       // float offset of ratebound[i][order]
    int32_t cl_off;       // float offset of the continuum-loss fit [i][order], -1 = none
    int32_t cl_k;
    int32_t cl_order;
    float   cl_xscale;
    float   charge;       // -1, 0, +1
    int32_t hist_bins;    // tally-only: histogram bins (0 = none)
    float   hist_lmin;    // log(Emin) (device energy units)
    float   hist_linv;    // bins / (log Emax - log Emin)
    int32_t rbB_off;      // swarm mode: float offset of B in ratebound = A + Fdt B (device rate per N s), -1 = none
    int32_t table_kind;   // 0: Chebyshev on binary intervals, 1: linear energy grid
    int32_t lin_n;        // linear grid: points
    float   lin_e0;       // linear grid: first energy (m_e c^2)
    float   lin_inv_step; // linear grid: 1 / step
    int32_t wall_coord;   // WallCallback (callback.jl:146-184): axis 0-2, -1 = none
    float   wall_v;       // wall position (m)
    int32_t wall_drop;    // drop the particle once recorded
    int32_t frozen;       // not pushed (RestrictedPusher / NullPusher): the clock only
    DevProc proc[16];
};

struct SBHdr {
    int32_t ne;        // primary energies
    int32_t ncum;      // cumulative-probability points (pcum = LinRange(0, 1, ncum))
    int32_t le_off;    // float offset of log(T / m_e c^2) [ne] in the blob
    float   inv_dp;    // ncum - 1
    float   ymargin;   // largest step of the pcum = 0 column between grid energies
};

struct BlobHdr {
    SpeciesHdr sp[3];
    SBHdr sb[4];
    float E[3];        // e E / (m_e c) per ns   (force per unit charge)
    float B[3];        // e B / m_e per ns       (times beta x B)
    int32_t nsb;
    int32_t bytes;     // total blob size (multiple of 16)
    int32_t nswarm;    // swarm mode: swarms batched in this context (0: classic single population)
    int32_t swarm_off; // float offset of [nswarm][4] = {E field (device units), Fdt (N s)}
    // position-dependent E (field.jl:10-52), lengths in m, fields in the units of E:
    // 0 homogeneous (E), 1 double layer {z1, z2, v[3]}, 2 step {z, v1[3], v2[3]},
    // 3 confined double layer {1/(2 sx^2), 1/(2 sy^2), 1/(2 sz^2), ez0, 1/sx^2, 1/sy^2, 1/sz^2}
    int32_t field_kind;
    int32_t pad_f;
    float   fp[8];
    // position-dependent B (ElectromagneticField with a field functor as b,
    // field.jl:54-70): the same kinds and layout, fields in the units of B
    int32_t bfield_kind;
    int32_t pad_b[3];
    float   bp[8];
};

// Device-side counters of one context (global memory, zeroed per launch
// where noted by the host).
struct Control {
    unsigned long long n[3];          // slots in use (live + dead); appends add here
    unsigned long long n_start[3];    // slots present at launch start (work space)
    unsigned long long head;          // work-fetch cursor over the concatenated work space
    unsigned long long spill_n;       // children written to the spill queue by this launch
    unsigned long long coll[3][16];   // real collisions per table position
    unsigned long long nulls[3];
    unsigned long long spawned[3];
    unsigned long long tally_count[3];
    double             tally_w[3];
    double             tally_wE[3];   // device energy units
    unsigned long long err[8];
    unsigned long long live_end[PCL_MAX_STEPS_PER_LAUNCH][3];  // live at the end of step k
    unsigned long long live_start[PCL_MAX_STEPS_PER_LAUNCH];   // particle-steps of step k
    unsigned long long dead[3];       // slots marked dead by this launch
    int                timeout;
    unsigned int       launch_seq;    // launch groups so far (k_begin), tags wall records
};

// Arguments of the step kernel (passed by value).
struct StepArgs {
    float4* xw[3];
    float4* ps[3];
    uint4*  meta[3];
    long long cap[3];
    // where population launches read their input slots: the population arrays
    // above, or (host-direct mode of pcl_advance_host) the caller's page-locked
    // host arrays, read over the CPU-GPU link
    const float4* in_xw[3];
    const float4* in_ps[3];
    const uint4*  in_meta[3];
    // host-direct mode: every slot write (update, dead mark, append) is also
    // made to these host arrays, for slots below hx_cap (nullptr: none)
    float4* hx_xw[3];
    float4* hx_ps[3];
    uint4*  hx_meta[3];
    long long hx_cap[3];
    // spill queues: the kernel reads `sp_in` (spill mode) and writes `sp_out`
    float4* sp_in_xw; float4* sp_in_ps; uint4* sp_in_meta;
    float4* sp_out_xw; float4* sp_out_ps; uint4* sp_out_meta;
    long long sp_cap;
    const unsigned long long* sp_in_n;   // spill-mode input count (device)
    unsigned long long* sp_out_n;        // spill output count (device)
    Control* ctl;
    const float4* blob;                  // table blob (global), staged to shared
    const float* sb_data[4];             // Seltzer-Berger tables [ne][ncum] (energy-major)
    double* hist_w[3];                   // tally-only histogram weights (device)
    unsigned long long* hist_n[3];       // tally-only histogram counts (device)
    uint32_t key0, key1;                 // Philox key
    double dt;                           // step length (ns)
    int nsteps;                          // steps in this launch
    int spill_mode;                      // 0: populations, 1: spill queue, 2: suspended collisions (resume)
    int blob_bytes;
    // learned sampler: collisions handed to the network are suspended into
    // lq_out (xw, ps, m1 = {sid_lo, sid_hi, ctr, ctr0}, m2 = {th, tlo, u,
    // species | k << 2 | j << 8 | nsub << 16}); a resume pass reads lq_in and
    // the network outputs lq_in_y.  lq_out_n == nullptr: no learned mode.
    float4* lq_out_xw; float4* lq_out_ps; uint4* lq_out_m1; float4* lq_out_m2;
    unsigned long long* lq_out_n;
    const float4* lq_in_xw; const float4* lq_in_ps; const uint4* lq_in_m1; const float4* lq_in_m2;
    const float* lq_in_y;
    const unsigned long long* lq_in_n;
    long long lq_cap;
    // wall crossings: {x, y, z, w}, {px, py, pz, t (ns since the launch start)},
    // {sid_lo, sid_hi, species, launch index}
    float4* wall_xw; float4* wall_pt; uint4* wall_meta;
    unsigned long long* wall_n;
    long long wall_cap;
    int general;    // a position-dependent field or a wall is set: the general step kernel runs
    int event;      // the event step kernel runs (parked collisions in full-warp batches)
    int stash;      // event kernel: stash entries per warp in use (1 to PCL_STASH_MAX)
    int learn;      // learned samplers attached: the kernel with suspend/resume runs
    // population launches over part of the work: concatenated indices
    // [g_lo, g_hi) of the species ranges (g_hi == 0: all of them)
    long long g_lo, g_hi;
    unsigned long long* head;   // work counter of this launch (the control block's, or a chunk's own)
};

// Network index of each (species, table position) with a learned sampler (-1: none).
struct LearnPick {
    int8_t net[48];
};

// Arguments of the compaction kernels (repack!, population.jl:229-259).
struct CompactArgs {
    const float4* sxw[3]; const float4* sps[3]; const uint4* smeta[3];
    float4* dxw[3]; float4* dps[3]; uint4* dmeta[3];
    const unsigned long long* n;   // slots per species (ctl->n)
    unsigned int* tile_cnt[3];
    unsigned long long* tile_off[3];
    unsigned long long* n_out;     // live counts per species (copied to ctl->n after the scatter)
    int ntiles_max;
};

}  // namespace pcl
