/*
 * particulator_gb300.h — C ABI of the GB300 null-collision Monte Carlo step.
 *
 * This is the drop-in boundary for the hot path of Particulator.jl: a Julia
 * host keeps building its populations, collision tables and pusher with the
 * package API and calls these entry points through `ccall` instead of running
 * `advance!` / `run!` on the CPU.  Every entry point takes plain pointers and
 * sizes, returns PCL_OK (0) or a negative PCL_ERR_* status, never throws and
 * never traps.  The library copies host buffers it is given; it owns all
 * device memory.  A context is externally single-threaded; all parallelism is
 * on the GPU.  There is no CPU fallback: without a CUDA device every call that
 * needs one returns PCL_ERR_CUDA.
 *
 * Units at this boundary are the reference's SI units in FP64 (m, kg m/s, J,
 * s, 1/s, m^2) unless a name says otherwise; the library converts to its FP32
 * device units on upload (momentum in m_e c, energy in m_e c^2, time in ns).
 *
 * Reference interfaces each entry point replaces are cited as file:line in the
 * Particulator.jl source tree.
 */
#ifndef PARTICULATOR_GB300_H
#define PARTICULATOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PCL_OK               0
#define PCL_ERR_INVALID     -1  /* bad argument or size                              */
#define PCL_ERR_CUDA        -2  /* CUDA runtime error or no device                   */
#define PCL_ERR_CAPACITY    -3  /* a population outgrew its capacity (population.jl:107) */
#define PCL_ERR_UNSUPPORTED -4  /* process kind or option with no device implementation */
#define PCL_ERR_STATE       -5  /* call order (e.g. advance before a species is set)  */
#define PCL_ERR_TIMEOUT     -6  /* a bounded device wait gave up                      */
#define PCL_ERR_NUMERIC     -7  /* numeric guard tripped (see pcl_tallies.errors)     */

/* ---- species (MultiPopulation(:electron, :photon, :positron), mixed_population.jl:4-12) */
#define PCL_ELECTRON  0
#define PCL_PHOTON    1
#define PCL_POSITRON  2
#define PCL_NSPECIES  3

/* species flags */
#define PCL_SPECIES_TRACKED     0  /* a normal Population (population.jl:7-21)            */
#define PCL_SPECIES_TALLY_ONLY  1  /* secondaries are counted and binned, never stored    */

/* ---- collision process kinds (closed set; arbitrary Julia `collide` methods
 * are rejected with PCL_ERR_UNSUPPORTED) --------------------------------- */
#define PCL_PROC_MOLLER          1  /* moller.jl:8-87                 */
#define PCL_PROC_RBEB            2  /* rbeb.jl:5-196                  */
#define PCL_PROC_SELTZER_BERGER  3  /* seltzer.jl:9-231               */
#define PCL_PROC_REL_COULOMB     4  /* relativistic_coulomb.jl:5-75   */
#define PCL_PROC_COMPTON         5  /* compton.jl:1-3, 59-144         */
#define PCL_PROC_KN_COMPTON      6  /* compton.jl:5-7, 34-47          */
#define PCL_PROC_PHOTOELECTRIC   7  /* photo_electric.jl:7-99         */
#define PCL_PROC_BETHE_HEITLER   8  /* bethe_heitler.jl:1-193         */
#define PCL_PROC_BHABHA          9  /* bhaba.jl:4-91                  */
#define PCL_PROC_ANNIHILATION   10  /* anihilation.jl:1-67            */
/* Low-energy swarm processes (slow-electron.jl:70-139), applied to the
 * relativistic electron state with a linear-grid table (the reference's
 * SlowElectronState path is not wired into advance!): */
#define PCL_PROC_ELASTIC        11  /* Elastic(mass_ratio): isotropic in the centre of mass (slow-electron.jl:133-139) */
#define PCL_PROC_EXCITATION     12  /* Excitation(threshold): loses the threshold, isotropic (slow-electron.jl:108-114) */
#define PCL_PROC_NULL_COLLISION 13  /* NullCollision as an explicit table entry (collisions.jl:3,58; lxcat.jl:115-119) */
#define PCL_PROC_IONIZATION     14  /* Ionization(threshold): two electrons share E - threshold, isotropic (slow-electron.jl:117-127) */
#define PCL_PROC_ATTACHMENT     15  /* Attachment(threshold): the electron is removed (slow-electron.jl:129-131) */

#define PCL_MAX_PROC      16   /* processes per species table              */
#define PCL_MAX_ORDER      4   /* Chebyshev terms per interval             */
#define PCL_MAX_INTERVALS 63   /* binary intervals (k); k+1 fits are kept  */
#define PCL_MAX_SB         4   /* distinct Seltzer-Berger tables (one per Z) */
#define PCL_NERR           8   /* error counters in pcl_tallies            */

/* error counter slots (pcl_tallies.errors[]) */
#define PCL_E_RATEBOUND   0  /* xi < 0 after all processes (collisions.jl:186 @assert)      */
#define PCL_E_TABLE_RANGE 1  /* energy outside a table's fitted range (extrapolated)         */
#define PCL_E_REJECT_CAP  2  /* a rejection loop hit its iteration cap                       */
#define PCL_E_SUBSTEP_CAP 3  /* a particle hit the sub-step cap inside one step              */
#define PCL_E_SPILL       4  /* warp child-stack overflow (children handled by a spill pass) */
#define PCL_E_CAPACITY    5  /* particles dropped because a population was full             */
#define PCL_E_KINEMATICS  6  /* sampler precondition failed (seltzer.jl:73, rbeb.jl:63, ...) */
#define PCL_E_NEG_RATE    7  /* rate bound <= 0 above the cut (treated as 0)                 */

/* ---- process descriptor ---------------------------------------------------
 * One entry of the reference's `processes` list `(coef, proc)`
 * (collision_table.jl:115-133).  `param` meaning per kind, SI units:
 *   MOLLER, BHABHA : param[0] = tcut (J)                       (moller.jl:8-11, bhaba.jl:4-7)
 *   RBEB           : param[0] = B (J), param[1] = U (J), param[2] = N  (rbeb.jl:5-14)
 *   REL_COULOMB    : Z (may be fractional via param[0] when Z == 0)     (relativistic_coulomb.jl:5-8)
 *   ANNIHILATION   : Z (may be fractional via param[0] when Z == 0)     (anihilation.jl:1-4)
 *   PHOTOELECTRIC  : param[0..nparam) = shell binding energies (J) in the order of
 *                    binding_energies(Z) (atomic_shells.jl:481-486), at most 8;
 *                    aux0/aux1 = SANDIA left energies (J) and coefficients [naux][4]
 *                    (SI: m^2 J^i per atom) used only for the cross section
 *   SELTZER_BERGER : aux0 = log primary energy (log J) [naux], aux1 = total
 *                    cross section (m^2) [naux], aux2 = inverse-CDF table
 *                    log(k/T) [naux2 = ncum][naux] column-major (pcum fastest),
 *                    exactly the fields of SeltzerBerger (seltzer.jl:9-21)
 *   COMPTON, KN_COMPTON, BETHE_HEITLER : Z only
 *   ELASTIC        : param[0] = electron / target mass ratio
 *   EXCITATION     : param[0] = threshold (J)
 *   NULL_COLLISION : none
 */
typedef struct pcl_process {
    int32_t kind;
    int32_t Z;
    double  coef;        /* scatterer density (1/m^3) multiplying speed * totalcs */
    double  param[8];
    int32_t nparam;
    int32_t naux;
    const double* aux0;
    const double* aux1;
    const double* aux2;
    int32_t naux2;
    int32_t reserved;
} pcl_process;

/* ---- context configuration --------------------------------------------- */
#define PCL_STASH_MAX 72   /* event kernel: collision-stash entries per warp */

typedef struct pcl_config {
    uint64_t seed;             /* Philox4x32-10 key for every particle stream        */
    int32_t  device;           /* CUDA device ordinal                                 */
    int32_t  block_size;       /* threads per block of the step kernel (0 = 256)      */
    int32_t  grid_blocks;      /* persistent grid size (0 = blocks_per_sm x SM count) */
    int32_t  steps_per_launch; /* time steps fused into one launch (0/1 = one)        */
    int32_t  compaction_period;/* compact dead slots every this many steps (0 = 8)    */
    int32_t  use_graph;        /* capture the step sequence of pcl_run in a CUDA graph */
    int32_t  blocks_per_sm;    /* classic kernel: resident blocks per SM, 2, 3 or 4 (0 = 4) */
    int32_t  classic_step;     /* 0 (default): colliding particles are parked and collided in
                                  full-warp batches (event kernel, 3 blocks per SM); 1: each
                                  lane collides in place (blocks_per_sm applies)            */
    int32_t  stash_entries;    /* event kernel: entries per warp of its collision stash in use
                                  (0 = all PCL_STASH_MAX; fewer, so that collisions find it
                                  full more often: the results do not depend on it)         */
    int32_t  reserved;
} pcl_config;

/* ---- per-context tallies (FP64 / int64 on the device) -------------------- */
typedef struct pcl_tallies {
    double  t;                                   /* simulated time (s)                     */
    int64_t steps;                               /* time steps completed                   */
    int64_t n[PCL_NSPECIES];                     /* slots in use (live + dead)              */
    int64_t live[PCL_NSPECIES];                  /* live particles after the last step      */
    int64_t particle_steps;                      /* sum over steps of live particles at step start */
    int64_t collisions[PCL_NSPECIES][PCL_MAX_PROC]; /* real collisions, table order (callback.jl:118-141) */
    int64_t nulls[PCL_NSPECIES];                 /* null collisions                          */
    int64_t spawned[PCL_NSPECIES];               /* secondaries stored (above the cut)      */
    int64_t tally_count[PCL_NSPECIES];           /* tally-only species: secondaries counted */
    double  tally_w[PCL_NSPECIES];               /* ... their summed weight                  */
    double  tally_wE[PCL_NSPECIES];              /* ... and weight x kinetic energy (J)       */
    int64_t errors[PCL_NERR];                    /* PCL_E_* counters                          */
} pcl_tallies;

/* ---- run options (run!, run.jl:1-29, with the device-side callbacks) ---- */
typedef struct pcl_run_opts {
    int32_t target_species;  /* PopulationTargetCallback{S} (callback.jl:253-267); -1 = none */
    int32_t target_ismax;    /* 1: stop when live >= target_n; 0: stop when live <= target_n */
    int64_t target_n;
    int64_t max_steps;       /* 0 = no limit besides tfinal */
} pcl_run_opts;

/* ---- packed device layout (FP32 device units), used for zero-conversion
 * host<->device transfers: three arrays of 16-byte records per species.
 *   xw[i]   = {x, y, z (m), w}
 *   ps[i]   = {px, py, pz (m_e c), s}
 *   meta[i] = {sid_lo, sid_hi, ctr (0xFFFFFFFF = dead slot), bits of t_off (ns, float)}
 * t_off is the particle's time relative to the context's simulated time. */
typedef struct pcl_packed {
    float*    xw;
    float*    ps;
    uint32_t* meta;
} pcl_packed;

/* ======================================================================= */
/* Host-side table builders (FP64).  They restate the reference's init path so
 * that a caller without Julia can produce the tables the step consumes.     */

/* Seltzer-Berger sampling table from a G4Physics2DVector (RawG4Physics2DVector,
 * util.jl:165-190): x = k/T fractions [nx], y = ln(T/MeV) [ny], value[ny][nx]
 * row-major (row = primary energy).  Replaces SeltzerBerger(d, Z; ncum, pcum,
 * gamma_min, gamma_max, energy_scale) (seltzer.jl:23-64) with pcum = LinRange(0,1,ncum).
 * Outputs: log_energy[ny], totalcs[ny], data[ncum*ny] (column-major, pcum fastest). */
int pcl_sb_build(int Z, int nx, int ny, const double* x, const double* y, const double* value,
                 int ncum, double gamma_min, double gamma_max, double energy_scale,
                 double* log_energy, double* totalcs, double* data);

/* Total cross section (m^2 per target) of one process at n kinetic energies (J):
 * totalcs(proc, E) of the process files above. */
int pcl_totalcs(const pcl_process* proc, int64_t n, const double* energy, double* out);

/* collision_table_from_processes(processes, particle, Fdt; safety, nintervals,
 * order, max_energy) (collision_table.jl:115-149) with compratebound (152-167).
 * rate is written in the reference's column-major a[k, j, i] layout:
 *   rate[k + order*(j + nproc*i)], k < order, j < nproc (table order), i <= nintervals;
 * ratebound[k + order*i]; perm[j] = index into procs of table position j. */
int pcl_build_collision_table(int species, int nproc, const pcl_process* procs, double Fdt,
                              double safety, int nintervals, int order, double max_energy,
                              double* rate, double* ratebound, int32_t* perm);

/* compratebound (collision_table.jl:152-167) is linear in Fdt, so the rate bound
 * of a table for any field is A + Fdt * B: A = the summed process fits,
 * B = the fit of gamma^3 v |d(sum nu)/dE| safety.  Inputs as written by
 * pcl_build_collision_table; A and B are [order][nintervals+1] column-major. */
int pcl_ratebound_split(int species, int order, int nproc, int nintervals, double xmax, const double* rate,
                        double safety, double* A, double* B);

/* ChebContinuumLoss(ContinuumLoss(nel, I, Tcut), Tmax, n) (continuum.jl:36-43,
 * 63-139).  Writes k (number of binary intervals), xmax = 2^k Tcut, and the
 * electron / positron coefficient matrices ec, pc [n][k+1] column-major
 * (term fastest).  cap = capacity of ec/pc in doubles. */
int pcl_build_continuum_loss(double nel, double I, double Tcut, double Tmax, int n,
                             int* k, double* xmax, double* ec, double* pc, int cap);

/* ======================================================================= */
/* Context and device state                                                 */

int  pcl_create(const pcl_config* cfg, void** ctx);
void pcl_destroy(void* ctx);
const char* pcl_last_error(void* ctx);
const char* pcl_version(void);
int  pcl_device_count(void);

/* Population(max_particles, inparticles, collisions, energy_cut) (population.jl:34-44),
 * the capacity / cut half: allocates the double-buffered device SoA. */
int pcl_set_species(void* ctx, int species, double energy_cut, int64_t capacity, int flags);

/* The table half of Population: a ChebyshevCollisionTable (collision_table.jl:63-106)
 * in the layout written by pcl_build_collision_table; procs are in table order.
 * nproc = 0 gives a species with no processes (rate bound 0). */
int pcl_set_collision_table(void* ctx, int species, int order, int nproc, int nintervals,
                            double xmax, const double* rate, const double* ratebound,
                            const pcl_process* procs);

/* The linear-grid CollisionTable (collision_table.jl:15-57): rates on the
 * energy grid LinRange(e0, e1, n) (J), rate[j + nproc*k] = rate of table
 * process j at grid point k (the reference's rate[j, k], column-major), and a
 * rate bound that is either one number (nrb = 1: ratebound(x::Number), line 232)
 * or one value per grid point (nrb = n, interpolated, lines 234-242).
 * Energies are located with indweight(LinRange) (util.jl:23-32). */
int pcl_set_linear_table(void* ctx, int species, int nproc, int n, double e0, double e1, const double* rate,
                         const double* ratebound, int nrb, const pcl_process* procs);

/* RK2Pusher(CombinedForcing(ElectromagneticField(HomogeneousField(E), HomogeneousField(B)),
 *           ChebContinuumLoss(...)))  (pusher.jl:37-63, field.jl:4-8,54-70, continuum.jl:25-57).
 * cl_order = 0 disables continuum losses. */
int pcl_set_forcing(void* ctx, const double E[3], const double B[3], int cl_order, int cl_k,
                    double cl_xmax, const double* cl_ec, const double* cl_pc);
/* Position-dependent electric field replacing the homogeneous E of
 * pcl_set_forcing (field.jl:10-52), SI: kind 0 homogeneous (no params),
 * 1 DoubleLayerField {z1, z2, vx, vy, vz}, 2 StepField {z, v1x, v1y, v1z, v2x,
 * v2y, v2z}, 3 ConfinedDoubleLayerField {sx, sy, sz, ez0}.  Evaluated at each
 * RK2 stage's position (pusher.jl:41-63).  Batched swarms keep their own
 * homogeneous fields. */
/* RestrictedPusher{T}(p) / NullPusher (pusher.jl:67-76) and
 * RestrictedForcing{T}(f) (pusher.jl:28-34), as species bit masks (bit s =
 * 1 << species): `pushed`, the species that move at all (the others only
 * advance their clocks, and still collide); `field`, those the EM field acts
 * on; `loss`, those the continuum loss acts on.  7 = every species (the
 * default). */
int pcl_set_push_mask(void* ctx, int pushed, int field, int loss);
/* A position-dependent B (ElectromagneticField(e, b) with b a field functor,
 * field.jl:54-70): the kinds and parameters of pcl_set_field, fields in T;
 * kind 0 = the homogeneous B of pcl_set_forcing.  Runs on the general step
 * kernel. */
int pcl_set_bfield(void* ctx, int kind, const double* params, int nparams);
int pcl_set_field(void* ctx, int kind, const double* params, int nparams);
/* WallCallback{P}(coord, v, drop) (callback.jl:146-184): while advancing,
 * a particle of `species` crossing the plane x[coord] = v (coord 0-2; -1
 * removes the wall) in the +axis direction is recorded as lincomb(new, old, w)
 * of its sub-step (electron.jl:127-132), which draws s like any state
 * constructor, and is dropped if drop != 0.  Records go to a device buffer of
 * `capacity`; pcl_get_wall copies them out (SI: x, p, w, t) and clears it
 * (species == NULL: *n = pending records). */
/* roulette! (population.jl:291-311): keep each live particle of `species`
 * with probability pkeep (one draw from its stream), dividing its weight by
 * pkeep, else remove it.  split! (population.jl:318-335): divide each live
 * particle's weight by 1 + p and add Poisson(p) copies (one draw; copies get
 * stream ids derived from the parent's).  As RouletteCallback / SplitCallback
 * (callback.jl:210-247) do, follow with pcl_compact. */
int pcl_roulette(void* ctx, int species, double pkeep);
/* Batched swarms: roulette! with keep probability pkeep[s] for swarm s (the
 * top 8 bits of the stream id); pkeep >= 1 leaves a swarm untouched.  Used to
 * hold each swarm at a population cap. */
int pcl_roulette_swarms(void* ctx, int species, int nswarm, const double* pkeep);
int pcl_split(void* ctx, int species, double p);
/* roulette!(f, popl) and split!(f, popl) (population.jl:291-305, 316-331)
 * with f a function of the particle's kinetic energy, given as a table of n
 * nodes (1 to 4096): energies in J, >= 0 and strictly increasing, and the
 * keep probabilities (any finite value: <= 0 removes, >= 1 keeps and divides
 * the weight by it, as rand() < p does) or the mean numbers of copies (in
 * [0, 64]).  f(E) is linear in E between nodes and constant beyond the ends,
 * evaluated on the device in FP64 from the particle's FP32 momentum.  A
 * caller with f as code (a Julia closure) tabulates it first.  Draws and
 * copies as for pcl_roulette / pcl_split. */
int pcl_roulette_fn(void* ctx, int species, int n, const double* energy, const double* pkeep);
int pcl_split_fn(void* ctx, int species, int n, const double* energy, const double* mean);
int pcl_set_wall(void* ctx, int species, int coord, double v, int drop, int64_t capacity);
int pcl_get_wall(void* ctx, int64_t* n, int32_t* species, uint64_t* sid, double* x, double* p, double* w,
                 double* t);

/* Batched form: nswarm (1..256) independent swarms share one context and every
 * launch; particle i belongs to swarm (sid >> 56) and its secondaries inherit
 * that (their other 56 stream-id bits are drawn as usual).  Swarm s feels the
 * homogeneous field E[3s..3s+2] (V/m; B stays global) and its lepton rate bound
 * is A + Fdt[s] B (pcl_ratebound_split with the safety factor given), the
 * table compratebound builds for that field.  A swarm run alone (nswarm = 1)
 * and the same swarm inside a batch execute the same arithmetic.  nswarm = 0
 * returns to the classic single population.  No reference counterpart: the
 * reference runs one MultiPopulation per swarm. */
int pcl_set_swarms(void* ctx, int nswarm, const double* E, const double* Fdt, double safety);

/* Per-swarm FP64 moments of one species: out[6*s + q] = {live, sum w,
 * sum w E (J), sum w z, sum w z^2, sum w (x^2 + y^2)} (m). */
int pcl_swarm_moments(void* ctx, int species, int nswarm, double* out);
/* Energy spectrum of the live particles of one species, as the reference's
 * scripts compute it with StatsBase.fit(Histogram, E, edges, weights(w))
 * (scripts/beam.jl:137-147, scripts/swarm.jl:149-158): counts[i] and
 * weights[i] (sum of w) over edges[i] <= E < edges[i+1], kinetic energies in
 * J, edges strictly increasing (2 <= nedges <= PCL_MAX_HIST_EDGES); energies
 * outside [edges[0], edges[nedges-1]) are not counted.  swarm >= 0 (batched
 * contexts) keeps that swarm only; -1 takes every particle. */
#define PCL_MAX_HIST_EDGES 4097
int pcl_energy_histogram(void* ctx, int species, int swarm, int nedges, const double* edges, int64_t* counts,
                         double* weights);
/* Live particles of each swarm of one species (out[s], s < nswarm; with
 * nswarm = 1 the whole population). */
int pcl_swarm_counts(void* ctx, int species, int nswarm, int64_t* out);
/* RouletteCallback(m) (callback.jl:210-227) on the device, per swarm: after
 * every launch group of pcl_run, each swarm of `species` (the whole
 * population when no swarms are set) with n > cap live particles gets
 * roulette!(cap / n).  Counting and roulette run on the context stream with
 * no host read-back; the removed particles are compacted with the next
 * periodic compaction.  The reference checks after every step: with
 * steps_per_launch = 1 so does this.  cap = 0 turns the cap off. */
int pcl_set_swarm_cap(void* ctx, int species, int64_t cap);

/* Replace the species' population with n particles (SI, FP64): x[3n], p[3n]
 * (interleaved xyz), w[n], t[n] (absolute, s).  s[n] = normalised time to the
 * next collision or NULL to draw s = -log U from each particle's stream, as the
 * state constructors do (electron.jl:30-33).  sid[n] = stream ids or NULL for
 * sid = sid_base + i.  Mirrors filling Population + init! (mixed_population.jl:20-35). */
int pcl_upload(void* ctx, int species, int64_t n, const double* x, const double* p,
               const double* w, const double* t, const double* s, const uint64_t* sid,
               uint64_t sid_base);

/* Copy the live particles of a species out (SI, FP64).  *n in: capacity of the
 * arrays, out: live particles written.  ctr = draws consumed per particle. */
int pcl_download(void* ctx, int species, int64_t* n, double* x, double* p, double* w,
                 double* t, double* s, uint64_t* sid, uint32_t* ctr);

/* Zero-conversion transfers of the packed layout (dead slots included on
 * download; *n in: capacity, out: slots).  Host buffers should be pinned. */
int pcl_upload_packed(void* ctx, int species, int64_t n, const pcl_packed* host);
int pcl_download_packed(void* ctx, int species, int64_t* n, pcl_packed* host);

/* advance!(mpopl, pusher, tfinal) followed by foreach(droplow!, mpopl)
 * (mixed_population.jl:38-47, population.jl:273-284, run.jl:7-8): advance every
 * live particle and every secondary born in the step to tfinal, drop particles
 * below their cut.  tfinal must be > the context time. */
int pcl_advance(void* ctx, double tfinal);

/* advance! of populations that live in host memory (packed layout, one
 * pcl_packed per species): the result equals pcl_upload_packed(in[s]) for
 * every species, pcl_advance(tfinal), pcl_download_packed(out[s]) - slots
 * updated in place with removed particles marked dead (ctr 0xFFFFFFFF), the
 * step's secondaries appended after n_in[s] - but runs as a pipeline: the
 * work is cut into `nchunks` (1-64) ranges, each uploaded on one copy stream,
 * stepped by a population launch over its range, and downloaded on another
 * copy stream while later ranges are still uploading or stepping.
 * compact != 0 repacks the population on the device (repack!,
 * population.jl:229-259) before it is downloaded (no download overlap that
 * step).  in and out may be the same buffers; n_out[s] <= out_cap[s] or
 * PCL_ERR_CAPACITY, returned after the step (the context holds the stepped
 * population; pcl_download_packed reads it into larger arrays).  No copy is
 * in flight when the call returns.  Host buffers should be pinned. */
int pcl_advance_host(void* ctx, double tfinal, const int64_t* n_in, const pcl_packed* in, int64_t* n_out,
                     pcl_packed* out, const int64_t* out_cap, int nchunks, int compact);
/* How pcl_advance_host moves the population over the CPU-GPU link (no
 * counterpart in the reference, whose populations never leave host memory):
 * PCL_HOST_IO_COPY: the chunked copy-engine pipeline above.
 * PCL_HOST_IO_DIRECT: one launch of the step kernel reads every input slot
 *   from the caller's page-locked arrays and writes every result (updated
 *   slots, dead marks, appended secondaries) to the output arrays over the
 *   link, with no copies (the context's device copy is written as well);
 *   nchunks is ignored.  The arrays must be page-locked (pcl_host_alloc,
 *   pcl_host_register, cudaHostAlloc) and usable by the device, else
 *   PCL_ERR_INVALID.  A compacting step (compact != 0) downloads the
 *   compacted population with copies as in the other mode.
 * PCL_HOST_IO_AUTO (default): the faster of the two on GB300, COPY (a step of
 *   16.8 M particles: 6.8 ms against 11.9 ms for DIRECT; SM loads and copy
 *   engines reach the same link rates, and DIRECT exposes the link's latency
 *   to every particle load of the step kernel). */
#define PCL_HOST_IO_AUTO   0
#define PCL_HOST_IO_COPY   1
#define PCL_HOST_IO_DIRECT 2
int pcl_set_host_io(void* ctx, int mode);
/* Page-lock (and release) caller-owned host memory so that the copies of
 * pcl_advance_host / pcl_upload_packed / pcl_download_packed from it run
 * asynchronously at full link speed (cudaHostRegister / cudaHostUnregister on
 * the current device; bytes > 0). */
int pcl_host_register(void* ptr, size_t bytes);
int pcl_host_unregister(void* ptr);
/* Page-locked host memory allocated by CUDA (cudaHostAlloc), for hosts that
 * can wrap a foreign buffer (Julia unsafe_wrap, numpy); *ptr = NULL on failure. */
int pcl_host_alloc(void** ptr, size_t bytes);
int pcl_host_free(void* ptr);

/* run!(mpopl, pusher, tfinal, dt, callback) (run.jl:1-29) with the device-side
 * PopulationTargetCallback / CollisionCounter.  Steps of dt until tfinal, the
 * target or max_steps; fills *out.  The target is tested after every step, as
 * run! does: with steps_per_launch > 1 the launches shrink near the target
 * (to one step until a per-step change has been seen, then to the steps the
 * fastest change seen so far needs, with a margin), so the run stops on the
 * same step as with one step per launch. */
int pcl_run(void* ctx, double tfinal, double dt, const pcl_run_opts* opts, pcl_tallies* out);

/* Counters, population statistics and maintenance. */
int pcl_get_tallies(void* ctx, pcl_tallies* out);
int pcl_reset_tallies(void* ctx);
/* FP64 weighted moments of the live particles of a species:
 * out = {sum w, sum w*E (J), sum w*x, y, z (m), sum w*x^2, y^2, z^2, max E (J), live count}
 * (weight, meanenergy, spread, posvar, maxenergy, nactives: population.jl:89-223). */
int pcl_moments(void* ctx, int species, double out[10]);
/* repack! (population.jl:229-259): compact dead slots (order-preserving). */
int pcl_compact(void* ctx);
/* Energy histogram of a tally-only species' secondaries: nbins log bins over
 * [emin, emax] J, set once; read returns counts (int64) and summed weights. */
int pcl_set_tally_histogram(void* ctx, int species, int nbins, double emin, double emax);
int pcl_get_tally_histogram(void* ctx, int species, int nbins, int64_t* counts, double* weights);

/* Synchronise the context stream and report the first sticky error. */
int pcl_sync(void* ctx);

/* ---- measurement (no reference counterpart: instrumentation) -------------
 * pcl_timer_start / pcl_timer_stop record CUDA events on the context's own
 * stream and return the elapsed device time in ms.  pcl_kernel_stats returns,
 * since the last reset, the summed event time (ms) of the step kernel's
 * main-pass launches, how many there were, the number of kernels the library
 * launched in total, and the step kernel's algorithmic HBM bytes
 * (48 B per slot read + 48 B per particle written + 4 B per slot marked dead). */
int pcl_timer_start(void* ctx);
int pcl_timer_stop(void* ctx, double* ms);
int pcl_kernel_stats(void* ctx, double* step_kernel_ms, int64_t* step_launches, int64_t* launches,
                     double* step_bytes, int reset);

/* ---- test hook: run one process sampler on the device --------------------
 * For each of n primaries (species of the table, energies via p[3n] in SI,
 * stream ids sid[n], counter 0), performs do_one_collision! forced onto table
 * position `proc_index` (collisions.jl:168-176, without the selection draw) and
 * writes the outcome: out_p[3*(3n)] momenta (primary, child 1, child 2; SI),
 * out_s[3n], out_kind[3n] (species of each slot, -1 = none / removed),
 * out_ctr[n] = draws consumed. */
int pcl_test_sampler(void* ctx, int species, int proc_index, int64_t n, const double* p,
                     const uint64_t* sid, double* out_p, double* out_s, int32_t* out_kind,
                     uint32_t* out_ctr);

/* Test hook of failure detection: a kernel waits, with the bounded wait every
 * device wait of the library uses and a limit of max_iters polls (1 .. 2^20),
 * on an mbarrier that nothing ever completes.  Returns PCL_ERR_TIMEOUT with
 * the context left usable (the flag is cleared). */
int pcl_test_timeout(void* ctx, int max_iters);

/* ---- compaction without device allocation --------------------------------
 * No counterpart in the reference: an extra entry point for callers that
 * cannot call cudaMalloc (a host whose memory pool owns the device, code on a
 * stream being captured, a latency-critical loop that must not allocate or
 * synchronise).  Same result as pcl_compact for one species, on device
 * buffers the caller owns: the n slots of xw/ps/meta (packed layout, dead
 * slots included) are compacted in order into out_xw/out_ps/out_meta and the
 * live count is written to the device int64 *n_out.  Scratch lives in a
 * static device array of PCL_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library keeps until exit; n above PCL_NOALLOC_MAX_SLOTS returns
 * PCL_ERR_CAPACITY.  All calls share that array, so calls that overlap on the
 * GPU race.  The input and output buffers must not overlap (an in-place
 * call would race between tiles): overlapping ranges return PCL_ERR_INVALID.
 * The first call on each device looks up the array's address and caches it
 * for the life of the process; make it before any stream capture, and do not
 * call this after cudaDeviceReset.  `stream` is a cudaStream_t (NULL =
 * default stream).  Context-free errors: pcl_last_error(NULL). */
#define PCL_NOALLOC_MAX_SLOTS (1 << 25)
#define PCL_NOALLOC_SCRATCH_BYTES 196864
int pcl_compact_noalloc(int64_t n, const float* xw, const float* ps, const uint32_t* meta,
                        float* out_xw, float* out_ps, uint32_t* out_meta, int64_t* n_out, void* stream);

/* ---- launch autotuner -------------------------------------------------------
 * No counterpart in the reference (its loop has no launch shape).  Advances
 * the simulation by up to steps_budget real steps of dt (the physics does not
 * depend on the launch parameters) while a coordinate search times candidate
 * launch shapes with CUDA events: step kernel {event, classic with 2, 3, 4
 * blocks per SM}, steps per launch {1, 2, 4, 8, 16, 32, 64}, compaction
 * period {2, 4, 8, 16, 32}, graph replay {0, 1}, in that order, then the
 * other step kernels once more at the chosen shape (the best kernel depends
 * on the steps per launch); each trial max(64, steps_budget / 21 rounded down
 * to a multiple of 64) steps, a whole number of launches; the search stops
 * when the budget is spent (a full search takes 21 x 64 = 1344 steps).  The
 * context keeps the fastest shape (particle-steps per second). */
typedef struct pcl_tune_result {
    int32_t blocks_per_sm, steps_per_launch, compaction_period, use_graph;   /* blocks_per_sm 0: event kernel */
    double  rate;              /* particle-steps per second of the kept shape */
    int32_t trials;
    int32_t steps;             /* steps advanced by the search */
    int32_t reserved[2];
} pcl_tune_result;
int pcl_autotune(void* ctx, double dt, int32_t steps_budget, pcl_tune_result* out);
/* Set the launch shape directly (e.g. one tuned on another context of the
 * same workload): blocks per SM (0: event kernel; 2-4: classic kernel with
 * that many blocks per SM), steps per launch (1-64), compaction period
 * (>= 1), graph replay (0/1). */
int pcl_set_launch(void* ctx, int32_t blocks_per_sm, int32_t steps_per_launch, int32_t compaction_period,
                   int32_t use_graph);

/* ---- learned inverse-CDF sampler network ---------------------------------
 * No single counterpart in the reference: a learned replacement for the
 * secondary-energy samplers of SeltzerBerger.collide (seltzer.jl:97-122) and
 * Moller.collide (moller.jl:64-87).  One network maps (a, b) to one output,
 * a = (log10(T / eV) - 6) / 2 over T in [1e4, 1e8] eV, b = 2u - 1 with u the
 * sampler's uniform; layers 2 -> 128 -> 128 -> 128 -> 1 with GELU, the two
 * 128 x 128 layers in BF16 on the tensor cores with FP32 accumulation.
 * Parameters are PCL_MLP_NPARAM floats: W1[128][2], b1[128], W2[128][128],
 * b2[128], W3[128][128], b3[128], w4[128], b4. */
#define PCL_MLP_NPARAM 33537
int pcl_mlp_create(int device, uint64_t seed, void** out);
void pcl_mlp_destroy(void* mlp);
const char* pcl_mlp_last_error(void* mlp);
int pcl_mlp_set_params(void* mlp, const float* params, int64_t n);
int pcl_mlp_get_params(void* mlp, float* params, int64_t n);
/* y[i] = net(x[2i], x[2i+1]) for host arrays */
int pcl_mlp_forward(void* mlp, int64_t n, const float* x, float* y);
/* gradient of mean((net(x) - t)^2) over the n rows, and the loss */
int pcl_mlp_gradient(void* mlp, int64_t n, const float* x, const float* t, float* grad, double* loss);
/* Adam (beta 0.9 / 0.999, cosine decay to 5 % of lr) over `steps` minibatches
 * of `batch` rows (a multiple of 128) drawn from the n-row dataset; *loss =
 * mean loss of the last 100 steps */
int pcl_mlp_train(void* mlp, int64_t n, const float* x, const float* t, int64_t steps, int32_t batch, double lr,
                  uint64_t seed, double* loss);

/* ---- learned sampler in the step ------------------------------------------
 * A context can hand the secondary-energy draw of a Seltzer-Berger or Moller
 * process to a network: the collision is suspended, the network evaluates all
 * suspended collisions of the launch in one batch on the tensor cores, and a
 * resume pass finishes them (angles, secondary, rest of the step).  The table
 * sampler is kept outside the trained range T in [1e4, 1e8] eV and where the
 * network is not monotone in u (checked on a grid when it is attached).
 * Outputs, both in [0, 1] and increasing in u: PCL_LEARN_SB h with
 * ln(k / T) = (1 - h) ln(kmin / T), kmin / T the table's pcum = 0 value at T;
 * PCL_LEARN_MOLLER v with eps = e0 / (1 - v (1 - 2 e0)), e0 = tcut / T. */
#define PCL_LEARN_SB     1
#define PCL_LEARN_MOLLER 2
/* Attach (mlp != NULL) or detach the network of table position proc_index. */
int pcl_set_learned(void* ctx, int species, int proc_index, int kind, void* mlp);
/* Training set from the table sampler of proc_index: per_T samples at each of
 * nT energies a_g = -1 + 2 g / (nT - 1), histogrammed on the device and turned
 * into Q quantile targets per energy: x_out[2 (g Q + i) + {0,1}] = (a_g,
 * 2 u_i - 1), u_i = (i + 1/2) / Q, t_out[g Q + i] = the output variable.
 * Energies outside the kind's domain give no rows; *nrows = rows written. */
int pcl_learn_data(void* ctx, int species, int proc_index, int kind, int nT, int64_t per_T, int Q, uint64_t seed,
                   float* x_out, float* t_out, int64_t* nrows);
/* Measurement hook (no counterpart in the reference): the cost of one
 * secondary-energy draw, table sampler against network.  n primaries
 * (1 .. 2^26) at E_i = 10^(4 + 4 (i + 1/2) / n) eV; the table path draws
 * k / T (PCL_LEARN_SB) or eps (PCL_LEARN_MOLLER) with the table sampler of
 * proc_index (seltzer.jl:97-122, moller.jl:64-87; one kernel); the network path
 * draws one uniform per primary, evaluates mlp on the tensor cores and maps its
 * output to the same quantity (three kernels).  Each path runs reps (1 .. 100)
 * times on the context's stream, timed with CUDA events; *ms_table / *ms_net
 * = the fastest repetition.  out_table / out_net (n floats) receive the draws
 * and draws_table (n) the uniforms the table sampler used per primary (the
 * network path uses one); each may be NULL. */
int pcl_time_energy_draw(void* ctx, int species, int proc_index, int kind, void* mlp, int64_t n, int reps,
                         double* ms_table, double* ms_net, float* out_table, float* out_net, uint32_t* draws_table);
/* Collisions answered by a network and rounds run since the context was made. */
int pcl_learn_stats(void* ctx, int64_t* suspended, int64_t* rounds);

#ifdef __cplusplus
}
#endif
#endif /* PARTICULATOR_GB300_H */
