// oracle.cpp — CPU restatement (C++17, Float64, SI units) of Particulator.jl's
// null-collision Monte Carlo step, used ONLY as test infrastructure: the GPU
// library is checked against it, and bench.py times it as the CPU baseline.
// Nothing in the shipped library includes, links or calls this file.
//
// PARITY UNPINNED: the reference is Julia, Julia is not available here, and
// the reference ships no golden vectors (test/runtests.jl is an empty
// testset), so this restatement is checked against the reference only by
// reading.  Each function cites the reference lines it restates.
//
// What it restates (paths inside the Particulator.jl tree):
//   advance!/advance1!/advance_init! .... src/mixed_population.jl:38-112
//   droplow!/repack! .................... src/population.jl:229-284
//   add_particle!/remove_particle! ...... src/population.jl:103-122
//   setr!/apply!/do_one_collision! ...... src/collisions.jl:63-199
//   precheb/chebval/rate/ratebound ...... src/cheby.jl:57-143, src/collision_table.jl:82-106
//   RK2Pusher/CombinedForcing ........... src/pusher.jl:14-63
//   RestrictedForcing/RestrictedPusher/
//   NullPusher (species masks) .......... src/pusher.jl:28-34, 67-76
//   ElectromagneticField (E and B as any
//   field of field.jl) .................. src/field.jl:4-70
//   roulette!/split! (constant, f(E)) ... src/population.jl:291-335
//   ChebContinuumLoss.force ............. src/continuum.jl:45-57
//   kinenergy/velocity/gamma ............ src/electron.jl:47-56, positron.jl:34-43, photon.jl:46-52
//   turn, nextcoll, modified Tsai ....... src/util.jl:17, 40-57, 143-159
//   samplers ............................ moller.jl:13-87, rbeb.jl:54-80,156-196,
//                                         seltzer.jl:67-122, relativistic_coulomb.jl:10-51,
//                                         compton.jl:9-28,119-144, photo_electric.jl:38-99,
//                                         bethe_heitler.jl:5-25,85-193, bhaba.jl:9-91,
//                                         anihilation.jl:6-67
//
// Random numbers: the reference draws from Julia's task-local Xoshiro; here
// every particle owns a Philox4x32-10 stream (key = seed, counter = (draw/4,
// sid_lo, sid_hi, 0)) and draws are consumed in exactly the order of the
// Julia code, including the draw for `s` in every state constructor.  The
// same streams drive the GPU, so both sides see identical uniforms.
//
// Documented deviations, shared with the GPU path:
//  * turn(): s = hypot(mu_x, mu_y) instead of sqrt(1 - mu_z^2) (identical for a
//    unit vector; the reference divides 0 by 0 at mu_z = +-1); at s = 0 the
//    azimuth reference is the x axis.  1 - cos^2 is clamped at 0.
//  * precheb beyond the last interval (x >= xmax, where the reference reads past
//    its array) extrapolates the last interval; a rate bound <= 0 counts as 0.
//  * rejection loops stop after 10000 iterations (counted), sub-steps after 2^20.
//  * rand(Bool) in Bethe-Heitler is U < 0.5.
//  * secondaries get their own stream, id drawn from the parent stream in
//    counter domain 1 at the parent's counter at the start of the collision.
//
// Tie tracking: every comparison whose outcome could flip between Float64 and
// the GPU's FP32 (u < g, nu > xi, trem > s/r, E vs cut, grid searches) records
// its relative margin; a particle with a margin below `tie_tol` is marked, and
// so are its descendants.  Bit-exact checks skip marked lineages.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <mutex>
#include <thread>
#include <algorithm>
#include <limits>

namespace orc {

// ---- constants (src/constants.jl) ----
constexpr double c = 299792458.0;
constexpr double e = 1.6021766208e-19;
constexpr double eV = 1.6021766208e-19;
constexpr double m_e = 9.10938356e-31;
constexpr double hbar = 1.0545718001391127e-34;
constexpr double alpha = 0.0072973525664;
constexpr double pi = 3.141592653589793;
constexpr double mc2 = m_e * (c * c);
constexpr double mc = m_e * c;
constexpr double epsilon_0 = 8.854187817620389e-12;
constexpr double r_e = e * e / (m_e * (c * c)) / (4.0 * pi * epsilon_0);
constexpr double a_0 = hbar / (m_e * c * alpha);
constexpr double EPS_T = 2.220446049250313e-16;  // eps(Float64) (mixed_population.jl:66)

enum { ELECTRON = 0, PHOTON = 1, POSITRON = 2 };
enum {
    P_MOLLER = 1, P_RBEB, P_SB, P_COULOMB, P_COMPTON, P_KN, P_PE, P_BH, P_BHABHA, P_ANN, P_ELASTIC, P_EXCITATION,
    P_NULL, P_IONIZATION, P_ATTACHMENT
};
enum { E_RATEBOUND = 0, E_TABLE_RANGE, E_REJECT_CAP, E_SUBSTEP_CAP, E_SPILL, E_CAPACITY, E_KINEMATICS, E_NEG_RATE };
constexpr int REJECT_CAP = 10000;
constexpr int SUBSTEP_CAP = 1 << 20;

// ---- Philox4x32-10 (Salmon et al. 2011) ----
static inline void philox(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t m0 = uint64_t(0xD2511F53u) * c0;
        uint64_t m1 = uint64_t(0xCD9E8D57u) * c2;
        uint32_t hi0 = uint32_t(m0 >> 32), lo0 = uint32_t(m0);
        uint32_t hi1 = uint32_t(m1 >> 32), lo1 = uint32_t(m1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

struct Proc {
    int kind = 0;
    int Z = 0;
    double p[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int np = 0;
    // Seltzer-Berger table (seltzer.jl:9-21): log_energy (log J), data[ncum][ne] col-major
    std::vector<double> le, data;
    int ncum = 0;
};

struct Table {
    int order = 1, nproc = 0, k = 1;
    double xmax = 1.0;
    std::vector<double> rate, rb;  // a[k,j,i] column-major, rb[k,i]; linear: rate[j,k], rb[k]
    std::vector<Proc> procs;
    // CollisionTable on LinRange(e0, e1, n) (collision_table.jl:15-57)
    bool linear = false;
    double e0 = 0, e1 = 0;
    int n = 0;
};

// LinRange(a, b, len)[i] for 0-based i (Julia's lerp form)
static inline double linrange(double a, double b, int len, int i) {
    double d = double(len - 1);
    return (a * (d - i) + b * i) / d;
}

// indweight(::LinRange, x) (util.jl:23-32): 0-based left index and weight;
// outside the grid the end interval is extrapolated (counted).
static inline int indweight(const Table& T, double x, double& w, bool& oor) {
    double step = (T.e1 - T.e0) / (T.n - 1);
    int i = int(std::floor((x - T.e0) / step));
    if (i < 0) { i = 0; oor = true; }
    if (i > T.n - 2) { i = T.n - 2; oor = true; }
    w = (linrange(T.e0, T.e1, T.n, i + 1) - x) / step;
    return i;
}

struct Part {
    double x[3], p[3], w, t, s, r;
    bool active;
    uint64_t sid;
    uint32_t ctr;
    uint8_t tie;
};

struct Species {
    bool set = false;
    double cut = std::numeric_limits<double>::infinity();
    bool tally_only = false;
    int wall_coord = -1;        // WallCallback (callback.jl:146-184): axis, position, drop
    double wall_v = 0.0;
    bool wall_drop = true;
    Table tab;
    std::vector<Part> parts;
};

struct Counters {
    int64_t coll[3][16] = {};
    int64_t nulls[3] = {};
    int64_t spawned[3] = {};
    int64_t tally_count[3] = {};
    double tally_w[3] = {};
    double tally_wE[3] = {};
    int64_t err[8] = {};
    int64_t ties = 0;
    void add(const Counters& o) {
        for (int s = 0; s < 3; ++s) {
            for (int j = 0; j < 16; ++j) coll[s][j] += o.coll[s][j];
            nulls[s] += o.nulls[s]; spawned[s] += o.spawned[s]; tally_count[s] += o.tally_count[s];
            tally_w[s] += o.tally_w[s]; tally_wE[s] += o.tally_wE[s];
        }
        for (int q = 0; q < 8; ++q) err[q] += o.err[q];
        ties += o.ties;
    }
};

struct World {
    uint32_t k0 = 0, k1 = 0;
    double tie_tol = 2e-5;
    Species sp[3];
    double E[3] = {0, 0, 0}, B[3] = {0, 0, 0};
    // position-dependent E (field.jl:10-52): 0 homogeneous, 1 double layer
    // {z1, z2, v[3]}, 2 step {z, v1[3], v2[3]}, 3 confined double layer {sx, sy, sz, ez0}
    int field_kind = 0;
    double fp[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // species bits (1 << species): pushed at all (RestrictedPusher /
    // NullPusher, pusher.jl:67-76), feeling the EM field, feeling the
    // continuum loss (RestrictedForcing, pusher.jl:28-34)
    int push_mask = 7, field_mask = 7, loss_mask = 7;
    // position-dependent B (field.jl:54-70 with a field functor as b): the
    // kinds and layout of the E field's, in T
    int bfield_kind = 0;
    double bp[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // wall crossings: {species, sid, x[3], p[3], w, t}
    struct WallRec { int species; uint64_t sid; double x[3], p[3], w, t; };
    mutable std::vector<WallRec> wall;   // appended by walkers (which see a const World)
    mutable std::mutex wall_mu;
    // swarm mode: swarm = top 8 bits of the stream id; per-swarm field and rate bound
    int nswarm = 0;
    std::vector<double> swarm_E;          // [nswarm][3]
    std::vector<double> swarm_rb[3];      // [nswarm][order*(k+1)] per species (empty: table's own)
    int cl_order = 0, cl_k = 0;
    double cl_xmax = 0;
    std::vector<double> ec, pc;
    Counters cnt;
};

// A particle being advanced: its state plus the cached Philox block.
struct Walker {
    Part* P;
    const World* W;
    Counters* C;
    uint32_t blk[4];
    uint32_t blk_id;
    bool blk_valid = false;
    // secondaries produced by the current collision
    struct Child { int species; double p[3]; double s; int idx; };
    Child kids[2];
    int nkids = 0;

    uint32_t bits() {
        uint32_t b = P->ctr >> 2;
        if (!blk_valid || b != blk_id) {
            uint32_t a = b, q = uint32_t(P->sid), r = uint32_t(P->sid >> 32), d = 0;
            philox(a, q, r, d, W->k0, W->k1);
            blk[0] = a; blk[1] = q; blk[2] = r; blk[3] = d;
            blk_id = b;
            blk_valid = true;
        }
        uint32_t v = blk[P->ctr & 3u];
        P->ctr += 1;
        return v;
    }
    static double to_u(uint32_t v) { return double(((v >> 9) << 1) | 1u) * 5.9604644775390625e-8; }
    double rand() { return to_u(bits()); }
    double nextcoll() { return -std::log(rand()); }  // util.jl:17

    // margin bookkeeping
    void near(double a, double b, double scale) {
        double m = std::fabs(a - b);
        double s = std::max(std::fabs(scale), 1e-300);
        if (m <= W->tie_tol * s) { if (!P->tie) C->ties++; P->tie = 1; }
    }
    bool lt(double a, double b) {  // a < b with tie check
        near(a, b, std::max(std::fabs(a), std::fabs(b)));
        return a < b;
    }
    void err(int q) { C->err[q]++; }
};

// ---- kinematics ----
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// kinenergy (electron.jl:53, positron.jl:40, photon.jl:50)
static inline double kinenergy(int species, const double* p) {
    if (species == PHOTON) return std::sqrt(dot3(p, p)) * c;
    return std::sqrt(mc2 * mc2 + c * c * dot3(p, p)) - mc2;
}

// ---- Chebyshev on binary intervals ----
// precheb (cheby.jl:127-143); x >= xmax extrapolates the last interval.
// *edge = relative distance of x to the nearest interval boundary (the
// piecewise fits are discontinuous there at the level of the fit error).
static inline int precheb(double x, int k, double xmax, int n, double* t, bool& oor, double* edge = nullptr) {
    double x1 = x / xmax;
    int l = 0;
    double s = std::frexp(x1, &l);
    int i = (x1 == 0.0) ? 0 : l + k;
    double xi;
    if (i > 0) {
        xi = 4 * s - 3;
        if (edge) *edge = std::min((s - 0.5) / 0.5, (1.0 - s));
        if (i > k) { oor = true; i = k; xi = 4 * x1 - 3; }
    } else {
        xi = std::ldexp(1.0, k + 1) * x1 - 1;
        if (edge) *edge = (1.0 - xi) / 2;
        i = 0;
    }
    t[0] = 1.0;
    if (n > 1) t[1] = xi;
    for (int j = 2; j < n; ++j) t[j] = 2 * xi * t[j - 1] - t[j - 2];
    return i;
}

// ratebound (collision_table.jl:94-106) and setr! (collisions.jl:63-74)
static double setr(Walker& Wk, int species) {
    const Species& S = Wk.W->sp[species];
    double eng = kinenergy(species, Wk.P->p);
    Wk.near(eng, S.cut, S.cut);
    if (eng < S.cut) return 0.0;
    const Table& T = S.tab;
    if (T.linear) {
        double w;
        bool oor = false;
        int i = indweight(T, eng, w, oor);
        if (oor) Wk.err(E_TABLE_RANGE);
        double r = w * T.rb[i] + (1 - w) * T.rb[i + 1];
        if (!(r > 0)) {
            if (T.nproc > 0) Wk.err(E_NEG_RATE);
            return 0.0;
        }
        return r;
    }
    double t[4];
    bool oor = false;
    double edge = 1.0;
    int i = precheb(eng, T.k, T.xmax, T.order, t, oor, &edge);
    if (oor) Wk.err(E_TABLE_RANGE);
    if (T.nproc > 0) Wk.near(edge, 0.0, 1.0);
    double r = 0.0;
    const double* rb = T.rb.data();
    const World& Wd = *Wk.W;
    if (Wd.nswarm > 0 && !Wd.swarm_rb[species].empty()) {
        int sw = std::min(int(Wk.P->sid >> 56), Wd.nswarm - 1);
        rb = Wd.swarm_rb[species].data() + size_t(sw) * T.order * (T.k + 1);
    }
    for (int q = 0; q < T.order; ++q) r += rb[q + T.order * i] * t[q];
    if (!(r > 0)) {
        if (T.nproc > 0) Wk.err(E_NEG_RATE);
        return 0.0;
    }
    return r;
}

// ---- forces and the RK2 push ----
// velocity (electron.jl:56, photon.jl:46)
static inline void velocity(int species, const double* p, double* v) {
    if (species == PHOTON) {
        double f = c / std::sqrt(dot3(p, p));
        for (int a = 0; a < 3; ++a) v[a] = p[a] * f;
        return;
    }
    double g = std::sqrt(1 + c * c * dot3(p, p) / (mc2 * mc2));
    double f = 1 / (m_e * g);
    for (int a = 0; a < 3; ++a) v[a] = p[a] * f;
}

// force(CombinedForcing(ElectromagneticField, ChebContinuumLoss), s)
// (pusher.jl:14-23, field.jl:54-70, continuum.jl:45-57)
// A field of field.jl:4-52 at position r: kind 0 the homogeneous value h.
// The double-layer and step fields jump at their planes: a stage position
// within the tie tolerance of one is a tie.
static void field_at(Walker& Wk, int kind, const double* fp, const double* h, const double* r, double* Eo) {
    switch (kind) {
        case 1: {  // DoubleLayerField: v between z1 and z2, else 0
            const double sc = std::max(std::fabs(fp[1] - fp[0]), 1e-9);
            Wk.near(r[2], fp[0], sc);
            Wk.near(r[2], fp[1], sc);
            bool in = fp[0] < r[2] && r[2] < fp[1];
            for (int a = 0; a < 3; ++a) Eo[a] = in ? fp[2 + a] : 0.0;
            break;
        }
        case 2: {  // StepField: v1 below z, v2 above
            Wk.near(r[2], fp[0], std::max(std::fabs(fp[0]), 1e-3));
            bool below = r[2] < fp[0];
            for (int a = 0; a < 3; ++a) Eo[a] = below ? fp[1 + a] : fp[4 + a];
            break;
        }
        case 3: {  // ConfinedDoubleLayerField
            double sx = fp[0], sy = fp[1], sz = fp[2], ez0 = fp[3];
            double g = ez0 * std::exp(-(r[0] * r[0] / (2 * sx * sx) + r[1] * r[1] / (2 * sy * sy) +
                                        r[2] * r[2] / (2 * sz * sz)));
            Eo[0] = -(g * r[0] * r[2]) / (sx * sx);
            Eo[1] = -(g * r[1] * r[2]) / (sy * sy);
            Eo[2] = g - (g * r[2] * r[2]) / (sz * sz);
            break;
        }
        default:
            for (int a = 0; a < 3; ++a) Eo[a] = h[a];
    }
}

static void efield(Walker& Wk, const World& W, const double* r, double* Eo) {
    field_at(Wk, W.field_kind, W.fp, W.E, r, Eo);
}

static void force(Walker& Wk, int species, const double* p, double* f, const double* r) {
    f[0] = f[1] = f[2] = 0.0;
    if (species == PHOTON) return;
    const World& W = *Wk.W;
    double v[3];
    velocity(species, p, v);
    double q = ((W.field_mask >> species) & 1) ? (species == ELECTRON ? -1.0 : 1.0) * e : 0.0;
    double Eloc[3];
    efield(Wk, W, r, Eloc);
    const double* Ef = Eloc;
    if (W.nswarm > 0) Ef = W.swarm_E.data() + 3 * size_t(std::min(int(Wk.P->sid >> 56), W.nswarm - 1));
    double Bl[3];
    field_at(Wk, W.bfield_kind, W.bp, W.B, r, Bl);
    f[0] = q * (Ef[0] + (v[1] * Bl[2] - v[2] * Bl[1]));
    f[1] = q * (Ef[1] + (v[2] * Bl[0] - v[0] * Bl[2]));
    f[2] = q * (Ef[2] + (v[0] * Bl[1] - v[1] * Bl[0]));
    if (W.cl_order > 0 && ((W.loss_mask >> species) & 1)) {
        double x = kinenergy(species, p);
        const std::vector<double>& a = (species == ELECTRON) ? W.ec : W.pc;
        double t[4];
        bool oor = false;
        int i = precheb(x, W.cl_k, W.cl_xmax, W.cl_order, t, oor);
        if (oor) Wk.err(E_TABLE_RANGE);
        double fl = 0.0;
        for (int j = 0; j < W.cl_order; ++j) fl += a[j + W.cl_order * i] * t[j];
        double pn = std::sqrt(dot3(p, p));
        if (pn > 0) {
            double k = -fl / pn;
            for (int a2 = 0; a2 < 3; ++a2) f[a2] += p[a2] * k;
        }
    }
}

// advance_particle(RK2Pusher, y, dt) (pusher.jl:41-63)
static void advance_particle(Walker& Wk, int species, double dt) {
    Part& y = *Wk.P;
    if (!((Wk.W->push_mask >> species) & 1)) {  // not pushed: the clock only (pusher.jl:73, 76)
        y.t = y.t + dt;
        return;
    }
    double v1[3], f1[3], v2[3], f2[3], p2[3];
    double x2[3];
    velocity(species, y.p, v1);
    force(Wk, species, y.p, f1, y.x);
    for (int a = 0; a < 3; ++a) {
        p2[a] = y.p[a] + 2 * dt * f1[a] / 3;
        x2[a] = y.x[a] + 2 * dt * v1[a] / 3;
    }
    velocity(species, p2, v2);
    force(Wk, species, p2, f2, x2);
    for (int a = 0; a < 3; ++a) {
        y.x[a] = y.x[a] + dt * (v1[a] / 4 + 3 * v2[a] / 4);
        y.p[a] = y.p[a] + dt * (f1[a] / 4 + 3 * f2[a] / 4);
    }
    y.t = y.t + dt;
}

// turn(u, cos theta, phi, n) (util.jl:40-57)
static void turn(const double* u, double cth, double phi, double n, double* out) {
    double un = std::sqrt(dot3(u, u));
    double mu[3] = {u[0] / un, u[1] / un, u[2] / un};
    double sphi = std::sin(phi), cphi = std::cos(phi);
    double sth = std::sqrt(std::max(0.0, 1 - cth * cth));
    double s = std::hypot(mu[0], mu[1]);
    double ca = 1.0, sa = 0.0;
    if (s > 0) { ca = mu[0] / s; sa = mu[1] / s; }
    out[0] = n * (sth * (ca * mu[2] * cphi - sa * sphi) + mu[0] * cth);
    out[1] = n * (sth * (sa * mu[2] * cphi + ca * sphi) + mu[1] * cth);
    out[2] = n * (-s * sth * cphi + mu[2] * cth);
}

// sample_modified_tsai_cos_theta(T) (util.jl:143-159)
static double tsai(Walker& Wk, double T) {
    double umax = 2 * (1 + T / (m_e * c * c));
    double a1 = 1.6, a2 = a1 / 3, border = 0.25;
    double u = 0;
    for (int it = 0;; ++it) {
        double r1 = Wk.rand();
        double r2 = Wk.rand();
        double uu = -std::log(r1 * r2);
        double r3 = Wk.rand();
        Wk.near(border, r3, border);
        u = border > r3 ? uu * a1 : uu * a2;
        Wk.near(u, umax, umax);
        if (u <= umax) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); u = umax; break; }
    }
    return 1 - 2 * u * u / (umax * umax);
}

static inline double momentum_norm_from_kin(double kin) {  // electron.jl:51
    return std::sqrt((kin + mc2) * (kin + mc2) - mc2 * mc2) / c;
}

// constructors of secondaries (add to the current collision's outcome)
static void child(Walker& Wk, int species, const double* p, double s, int idx) {
    Walker::Child& k = Wk.kids[Wk.nkids++];
    k.species = species;
    k.p[0] = p[0]; k.p[1] = p[1]; k.p[2] = p[2];
    k.s = s;
    k.idx = idx;
}

// ---- samplers ----
// relativistic_coulomb.jl:10-51
static void s_coulomb(Walker& Wk, const Proc& P, int species) {
    Part& L = *Wk.P;
    double phi = 2 * pi * Wk.rand();
    double v[3];
    velocity(species, L.p, v);
    double beta = std::sqrt(dot3(v, v)) / c;
    double Z = (P.Z == 0) ? P.p[0] : double(P.Z);
    double a = 1.3413 * std::pow(Z, -1.0 / 3.0) * a_0;
    double al = hbar * hbar / (4 * dot3(L.p, L.p) * a * a);
    double x = 0;
    for (int it = 0;; ++it) {
        double u = Wk.rand();
        x = al * u / (al + 1 - u);
        double z = Wk.rand();
        if (Wk.lt(z, 1 - beta * beta * x)) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
    }
    double cth = 1 - 2 * x;
    double pn[3];
    turn(L.p, cth, phi, std::sqrt(dot3(L.p, L.p)), pn);
    std::memcpy(L.p, pn, sizeof(pn));
    L.s = Wk.nextcoll();
}

// Lehtinen angles (moller.jl:26-28)
static inline void lehtinen(double E0, double E1, double E2, double& c1, double& c2) {
    c1 = std::sqrt(E1 * (E0 + 2 * mc2) / (E0 * (E1 + 2 * mc2)));
    c2 = std::sqrt(E2 * (E0 + 2 * mc2) / (E0 * (E2 + 2 * mc2)));
}

// moller.jl:13-37, 64-87
static void s_moller(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    double tcut = P.p[0];
    double e0 = tcut / eng;
    double g = 1 + eng / mc2;
    double eps = 0.5;
    for (int it = 0;; ++it) {
        double r = Wk.rand();
        eps = e0 / (1 - r + 2 * e0 * r);
        double gg = 4 / (9 * g * g - 10 * g + 5) *
                    ((g - 1) * (g - 1) * eps * eps - (2 * g * g + 2 * g - 1) * (eps / (1 - eps)) +
                     g * g / ((1 - eps) * (1 - eps)));
        if (Wk.lt(Wk.rand(), gg)) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
    }
    double E2 = eps * eng, E0 = eng, E1 = E0 - E2;
    double p1 = std::sqrt(E1 * E1 + 2 * mc2 * E1) / c;
    double p2 = std::sqrt(E2 * E2 + 2 * mc2 * E2) / c;
    double c1, c2;
    lehtinen(E0, E1, E2, c1, c2);
    double phi = 2 * pi * Wk.rand();
    double a[3], b[3];
    turn(L.p, c1, phi, p1, a);
    turn(L.p, c2, -phi, p2, b);
    std::memcpy(L.p, a, sizeof(a));
    L.s = Wk.nextcoll();
    double s2 = Wk.nextcoll();
    child(Wk, ELECTRON, b, s2, 0);
}

// rbeb.jl:54-80, 156-196
static void s_rbeb(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    double B = P.p[0];
    Wk.near(eng, B, B);
    if (!(eng > B)) { Wk.err(E_KINEMATICS); L.s = Wk.nextcoll(); return; }
    double t1 = eng / mc2, b1 = B / mc2;
    double bt2 = 1 - 1 / ((1 + t1) * (1 + t1));
    double t = eng / B;
    double A = -(1 + 2 * t1) / (t + 1) / ((1 + t1) * (1 + t1));
    double Bc = 1;
    double C = std::log(bt2 / (1 - bt2)) - bt2 - std::log(2 * b1);
    double M = b1 * b1 / ((1 + t1) * (1 + t1));
    double w = 0;
    for (int it = 0;; ++it) {
        double u = Wk.rand();
        w = u / ((t + 1) / (t - 1) - u);
        double pb = (2 * Bc + 2 * C + (t + 1) * (t + 1) * Bc * M / 4) / ((1 + w) * (1 + w));
        auto g = [&](int q) { return 1 / std::pow(w + 1, q) + 1 / std::pow(t - w, q); };
        double p0 = A * g(1) + Bc * (g(2) + M) + C * g(3);
        if (Wk.lt(Wk.rand() * pb, p0)) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
    }
    double E0 = eng, E2 = B * w, E1 = E0 - E2 - B;
    if (!(E2 < E1)) Wk.err(E_KINEMATICS);
    double p1 = std::sqrt(E1 * E1 + 2 * mc2 * E1) / c;
    double p2 = std::sqrt(E2 * E2 + 2 * mc2 * E2) / c;
    double c1, c2;
    lehtinen(E0, E1, E2, c1, c2);
    double phi = 2 * pi * Wk.rand();
    double a[3], b[3];
    turn(L.p, c1, phi, p1, a);
    turn(L.p, c2, -phi, p2, b);
    std::memcpy(L.p, a, sizeof(a));
    L.s = Wk.nextcoll();
    double s2 = Wk.nextcoll();
    child(Wk, ELECTRON, b, s2, 0);
}

// seltzer.jl:67-122 (interpolation weights exactly as written at 278-284)
static void s_sb(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    const int ncum = P.ncum, ne = int(P.le.size());
    double x = Wk.rand();
    double y = std::log(eng);
    // i2 = searchsortedfirst(pcum, x): pcum[i] = i / (ncum - 1) (LinRange(0, 1, ncum))
    int i1 = int(std::floor(x * (ncum - 1)));
    if (i1 > ncum - 2) i1 = ncum - 2;
    int i2 = i1 + 1;
    double xa = double(i1) / (ncum - 1), xb = double(i2) / (ncum - 1);
    // j2 = searchsortedfirst(log_energy, y)
    int j2 = int(std::lower_bound(P.le.begin(), P.le.end(), y) - P.le.begin());
    for (int q = std::max(0, j2 - 1); q <= std::min(ne - 1, j2); ++q) Wk.near(y, P.le[q], 1.0);
    int j1 = j2 - 1;
    if (j1 < 0) { j1 = 0; Wk.err(E_TABLE_RANGE); }
    if (j1 > ne - 2) { j1 = ne - 2; Wk.err(E_TABLE_RANGE); }
    j2 = j1 + 1;
    double y1 = P.le[j1], y2 = P.le[j2];
    auto u = [&](int i, int j) { return P.data[size_t(i) + size_t(ncum) * j]; };
    double A = (xb - xa) * (y2 - y1);
    double S = (u(i1, j1) * (xb - x) * (y2 - y) + u(i1, j2) * (x - xa) * (y2 - y) +
                u(i2, j1) * (xb - x) * (y - y1) + u(i2, j2) * (x - xa) * (y - y1));
    double k = eng * std::exp(S / A);
    if (!(k < eng)) Wk.err(E_KINEMATICS);
    double photon_p_norm = k / c;
    double cth = tsai(Wk, eng);
    double phi = 2 * pi * Wk.rand();
    double pph[3];
    turn(L.p, cth, phi, photon_p_norm, pph);
    for (int a = 0; a < 3; ++a) L.p[a] = L.p[a] - pph[a];
    L.s = Wk.nextcoll();
    double s2 = Wk.nextcoll();
    child(Wk, PHOTON, pph, s2, 0);
}

// compton.jl:9-28, 119-144
static void s_compton(Walker& Wk, double eng) {
    Part& L = *Wk.P;
    double e0 = mc2 / (mc2 + 2 * eng);
    double a1 = -std::log(e0);
    double a2 = (1 - e0 * e0) / 2;
    double t = 0, eps = 1;
    for (int it = 0;; ++it) {
        if (Wk.lt(Wk.rand(), a1 / (a1 + a2))) eps = std::exp(-Wk.rand() * a1);
        else eps = std::sqrt(e0 * e0 + (1 - e0 * e0) * Wk.rand());
        t = mc2 * (1 - eps) / (eps * eng);
        double g = (1 - eps / (1 + eps * eps) * t * (2 - t));
        if (Wk.lt(Wk.rand(), g)) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
    }
    double cth = 1 - t, E1 = eps * eng;
    double phi = 2 * pi * Wk.rand();
    double pg[3];
    turn(L.p, cth, phi, E1 / c, pg);
    double pe[3] = {L.p[0] - pg[0], L.p[1] - pg[1], L.p[2] - pg[2]};
    std::memcpy(L.p, pg, sizeof(pg));
    L.s = Wk.nextcoll();
    double s2 = Wk.nextcoll();
    child(Wk, ELECTRON, pe, s2, 0);
}

// photo_electric.jl:38-52, 60-99
static void s_pe(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    double b = P.p[0];
    for (int m = 0; m < P.np; ++m) {
        b = P.p[m];
        Wk.near(eng, b, b);
        if (eng > b) break;
    }
    if (!(eng > b)) Wk.err(E_KINEMATICS);
    double Ee = eng - b;
    double g = 1 + Ee / mc2;
    double beta = std::sqrt(1 - 1 / (g * g));
    double A = 1 / beta - 1;
    auto gf = [&](double nu) { return (2 - nu) * (1 / (A + nu) + beta * g * (g - 1) * (g - 2) / 2); };
    double nu = 0;
    for (int it = 0;; ++it) {
        double xi = Wk.rand();
        nu = 2 * A / ((A + 2) * (A + 2) - 4 * xi) * (2 * xi + (A + 2) * std::sqrt(xi));
        double xi1 = Wk.rand();
        if (Wk.lt(xi1 * gf(0), gf(nu))) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
    }
    double cth = 1 - nu;
    double phi = 2 * pi * Wk.rand();
    double pe[3];
    turn(L.p, cth, phi, momentum_norm_from_kin(Ee), pe);
    double s2 = Wk.nextcoll();
    L.active = false;
    child(Wk, ELECTRON, pe, s2, 0);
}

// bethe_heitler.jl:153-193
static double screen1(double d) { return d > 1.4 ? 42.038 - 8.29 * std::log(d + 0.958) : 42.184 - d * (7.444 - 1.623 * d); }
static double screen2(double d) { return d > 1.4 ? 42.038 - 8.29 * std::log(d + 0.958) : 41.326 - d * (5.848 - 0.902 * d); }
static double fc_quirk(double) {  // _fc uses alpha where alpha Z is meant (bethe_heitler.jl:153-161)
    double aZ = alpha, aZ2 = aZ * aZ, aZ4 = aZ2 * aZ2, aZ6 = aZ4 * aZ2;
    double f1 = 1 / (1 + aZ2) + 0.20206 - 0.0369 * aZ2 + 0.0083 * aZ4 - 0.0020 * aZ6;
    return f1 * aZ2;
}

// bethe_heitler.jl:5-25, 85-146
static void s_bh(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    const double Z = P.Z;
    double e0 = mc2 / eng;
    if (!(e0 < 0.5)) Wk.err(E_KINEMATICS);
    double eps;
    Wk.near(eng, 2e6 * eV, 2e6 * eV);
    if (eng < 2e6 * eV) {
        eps = e0 + (0.5 - e0) * Wk.rand();
    } else {
        double d0 = 136 * e0 / std::pow(Z, 1.0 / 3.0);
        double FZ = 8 * std::log(Z) / 3;
        Wk.near(eng, 50e6 * eV, 50e6 * eV);
        if (eng > 50e6 * eV) FZ += 8 * fc_quirk(Z);
        double dmin = 4 * d0;
        double dmax = std::exp((42.24 - FZ) / 8.368) - 0.952;
        double ep = (1 - std::sqrt(1 - dmin / dmax)) / 2;
        double emin = std::max(e0, ep);
        double er = 0.5 - emin;
        double F10 = screen1(dmin) - FZ, F20 = screen2(dmin) - FZ;
        double NF1 = std::max(F10 * er * er, 0.0);
        double NF2 = std::max(1.5 * F20, 0.0);
        double NC = NF1 / (NF1 + NF2);
        for (int it = 0;; ++it) {
            bool acc;
            if (Wk.lt(Wk.rand(), NC)) {  // NC > rand()
                eps = 0.5 - er * std::pow(Wk.rand(), 1.0 / 3.0);
                double d = d0 / (eps * (1 - eps));
                acc = Wk.lt(Wk.rand(), (screen1(d) - FZ) / F10);
            } else {
                eps = emin + er * Wk.rand();
                double d = d0 / (eps * (1 - eps));
                acc = Wk.lt(Wk.rand(), (screen2(d) - FZ) / F20);
            }
            if (acc) break;
            if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
        }
    }
    double etot, ptot;
    if (Wk.lt(Wk.rand(), 0.5)) { etot = (1 - eps) * eng; ptot = eps * eng; }
    else { ptot = (1 - eps) * eng; etot = eps * eng; }
    double ekin = std::max(0.0, etot - mc2), pkin = std::max(0.0, ptot - mc2);
    // collide binds the returned (ekin, pkin) as (pkin, ekin)
    double pkin_c = ekin, ekin_c = pkin;
    double phi = 2 * pi * Wk.rand();
    double cth = tsai(Wk, ekin_c);
    double pe[3], pp[3];
    turn(L.p, cth, phi, momentum_norm_from_kin(ekin_c), pe);
    cth = tsai(Wk, pkin_c);
    turn(L.p, cth, phi, momentum_norm_from_kin(pkin_c), pp);
    double se = Wk.nextcoll();
    double spz = Wk.nextcoll();
    L.active = false;
    child(Wk, ELECTRON, pe, se, 0);
    child(Wk, POSITRON, pp, spz, 1);
}

// bhaba.jl:9-33, 55-91
static void s_bhabha(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    double tcut = P.p[0];
    double e0 = tcut / eng;
    double g = 1 + eng / mc2;
    double y = 1 / (g + 1);
    double B0 = g * g / (g * g - 1);
    double B1 = 2 - y * y, B2 = (1 - 2 * y) * (3 + y * y);
    double B3 = (1 - 2 * y) * (1 - 2 * y) + std::pow(1 - 2 * y, 3), B4 = std::pow(1 - 2 * y, 3);
    double eps = e0;
    for (int it = 0;; ++it) {
        double r = Wk.rand();
        eps = e0 / (1 - r + e0 * r);
        double g1 = B0 + B1 * eps + B2 * eps * eps + B3 * eps * eps * eps + B4 * eps * eps * eps * eps;
        double g2 = B0 + B1 * e0 + B2 * e0 * e0 + B3 * e0 * e0 * e0 + B4 * e0 * e0 * e0 * e0;
        if (Wk.lt(Wk.rand(), g1 / g2)) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
    }
    double E0 = eng, E2 = eps * eng, E1 = E0 - E2;
    double p1 = std::sqrt(E1 * E1 + 2 * mc2 * E1) / c;
    double p2 = std::sqrt(E2 * E2 + 2 * mc2 * E2) / c;
    double c1, c2;
    lehtinen(E0, E1, E2, c1, c2);
    double phi = 2 * pi * Wk.rand();
    double a[3], b[3];
    turn(L.p, c1, phi, p1, a);
    turn(L.p, c2, -phi, p2, b);
    std::memcpy(L.p, a, sizeof(a));
    L.s = Wk.nextcoll();
    double s2 = Wk.nextcoll();
    child(Wk, ELECTRON, b, s2, 0);
}

// anihilation.jl:6-23, 39-67
static void s_ann(Walker& Wk, double eng) {
    Part& L = *Wk.P;
    double g = 1 + eng / mc2;
    double emax = (1 + std::sqrt((g - 1) / (g + 1))) / 2;
    double emin = (1 - std::sqrt((g - 1) / (g + 1))) / 2;
    double eps = 0.5;
    for (int it = 0;; ++it) {
        eps = emin * std::pow(emax / emin, Wk.rand());
        double gg = 1 - eps + (2 * g * eps - 1) / (eps * (g + 1) * (g + 1));
        if (Wk.lt(Wk.rand(), gg)) break;
        if (it + 1 >= REJECT_CAP) { Wk.err(E_REJECT_CAP); break; }
    }
    double cth = (eps * (g + 1) - 1) / (eps * std::sqrt(g * g - 1));
    // Near the kinematic limits eps -> eps_min/max, sin(theta) ~ sqrt(q - 2|eps - 1/2|)
    // has an infinite derivative: the FP32 rounding of E alone moves the photon
    // directions there, so that window (1e-3 of q) is an ill-conditioned tie.
    {
        double q = std::sqrt((g - 1) / (g + 1));
        Wk.near(2 * std::fabs(eps - 0.5), q, 50.0 * q);
    }
    double phi = 2 * pi * Wk.rand();
    double Etot = eng + 2 * mc2;
    double pa[3];
    turn(L.p, cth, phi, eps * Etot / c, pa);
    double pb[3] = {L.p[0] - pa[0], L.p[1] - pa[1], L.p[2] - pa[2]};
    double sa = Wk.nextcoll();
    double sb = Wk.nextcoll();
    L.active = false;
    child(Wk, PHOTON, pa, sa, 0);
    child(Wk, PHOTON, pb, sb, 1);
}

// randsphere() (util.jl:4-12)
static void randsphere(Walker& Wk, double* d) {
    double phi = 2 * pi * Wk.rand();
    double sp = std::sin(phi), cp = std::cos(phi);
    double u = 2 * Wk.rand() - 1;
    double v = std::sqrt(1 - u * u);
    d[0] = v * cp; d[1] = v * sp; d[2] = u;
}

// collide(::Elastic, ...) (slow-electron.jl:133-139) on the momentum
static void s_elastic(Walker& Wk, const Proc& P) {
    Part& L = *Wk.P;
    double mr = P.p[0];
    double cm[3], d[3];
    for (int a = 0; a < 3; ++a) cm[a] = (mr / (1 + mr)) * L.p[a];
    double dv[3] = {L.p[0] - cm[0], L.p[1] - cm[1], L.p[2] - cm[2]};
    double dn = std::sqrt(dot3(dv, dv));
    randsphere(Wk, d);
    for (int a = 0; a < 3; ++a) L.p[a] = d[a] * dn + cm[a];
    L.s = Wk.nextcoll();
}

// collide(::Excitation, ...) (slow-electron.jl:108-114)
static void s_excitation(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    double E1 = std::max(0.0, eng - P.p[0]);
    double pn = momentum_norm_from_kin(E1);
    double d[3];
    randsphere(Wk, d);
    for (int a = 0; a < 3; ++a) L.p[a] = d[a] * pn;
    L.s = Wk.nextcoll();
}

// collide(::Ionization, ...) (slow-electron.jl:117-127)
static void s_ionization(Walker& Wk, const Proc& P, double eng) {
    Part& L = *Wk.P;
    double E1 = 0.5 * std::max(0.0, eng - P.p[0]);
    double pn = momentum_norm_from_kin(E1);
    double u[3], v[3];
    randsphere(Wk, u);
    randsphere(Wk, v);
    for (int a = 0; a < 3; ++a) L.p[a] = u[a] * pn;
    L.s = Wk.nextcoll();
    double cs = Wk.nextcoll();
    double q[3] = {v[0] * pn, v[1] * pn, v[2] * pn};
    child(Wk, ELECTRON, q, cs, 0);
}

static void sample(Walker& Wk, const Proc& P, int species, double eng) {
    switch (P.kind) {
        case P_COULOMB: s_coulomb(Wk, P, species); break;
        case P_MOLLER: s_moller(Wk, P, eng); break;
        case P_RBEB: s_rbeb(Wk, P, eng); break;
        case P_SB: s_sb(Wk, P, eng); break;
        case P_COMPTON:
        case P_KN: s_compton(Wk, eng); break;
        case P_PE: s_pe(Wk, P, eng); break;
        case P_BH: s_bh(Wk, P, eng); break;
        case P_BHABHA: s_bhabha(Wk, P, eng); break;
        case P_ANN: s_ann(Wk, eng); break;
        case P_ELASTIC: s_elastic(Wk, P); break;
        case P_EXCITATION: s_excitation(Wk, P, eng); break;
        case P_IONIZATION: s_ionization(Wk, P, eng); break;
        case P_ATTACHMENT: Wk.P->active = false; break;  // RemoveParticleOutcome
        case P_NULL: Wk.P->s = Wk.nextcoll(); break;  // NullOutcome (collisions.jl:83-88)
        default: Wk.err(E_KINEMATICS); break;
    }
}

// Secondaries produced during a sweep, per thread.
struct SpawnBuf {
    std::vector<Part> q[3];
};

// apply! for the secondaries (collisions.jl:96-133 -> add_particle!, population.jl:103-113)
static void flush_kids(Walker& Wk, uint32_t ctr0, SpawnBuf& out) {
    const World& W = *Wk.W;
    for (int q = 0; q < Wk.nkids; ++q) {
        const Walker::Child& k = Wk.kids[q];
        const Species& S = W.sp[k.species];
        double E = kinenergy(k.species, k.p);
        Wk.near(E, S.cut, S.cut);
        if (E <= S.cut) continue;
        if (S.tally_only) {
            Wk.C->tally_count[k.species] += 1;
            Wk.C->tally_w[k.species] += Wk.P->w;
            Wk.C->tally_wE[k.species] += Wk.P->w * E;
            continue;
        }
        uint32_t a = ctr0, b = uint32_t(Wk.P->sid), c2 = uint32_t(Wk.P->sid >> 32), d = 1u;
        philox(a, b, c2, d, W.k0, W.k1);
        Part n;
        std::memcpy(n.x, Wk.P->x, sizeof(n.x));
        std::memcpy(n.p, k.p, sizeof(n.p));
        n.w = Wk.P->w;
        n.t = Wk.P->t;
        n.s = k.s;
        n.active = true;
        n.sid = k.idx ? (uint64_t(c2) | (uint64_t(d) << 32)) : (uint64_t(a) | (uint64_t(b) << 32));
        if (W.nswarm > 0) n.sid = (n.sid & 0x00FFFFFFFFFFFFFFull) | (Wk.P->sid & 0xFF00000000000000ull);
        n.ctr = 0;
        n.tie = Wk.P->tie;
        Walker Wc{&n, Wk.W, Wk.C};
        n.r = setr(Wc, k.species);
        Wk.C->spawned[k.species] += 1;
        out.q[k.species].push_back(n);
    }
    Wk.nkids = 0;
}

// do_one_collision! (collisions.jl:142-199)
static void do_one_collision(Walker& Wk, int species, SpawnBuf& out) {
    const Species& S = Wk.W->sp[species];
    Part& L = *Wk.P;
    if (L.r == 0) return;
    double eng = kinenergy(species, L.p);
    Wk.near(eng, S.cut, S.cut);
    if (!(eng >= S.cut)) return;
    const Table& T = S.tab;
    uint32_t ctr0 = L.ctr;
    int j = 0;
    if (T.linear) {  // rate(::CollisionTable, j, pre) (collision_table.jl:53-57)
        double w;
        bool oor = false;
        int i = indweight(T, eng, w, oor);
        if (oor) Wk.err(E_TABLE_RANGE);
        double xi = Wk.rand() * L.r;
        for (; j < T.nproc; ++j) {
            double nu = w * T.rate[j + size_t(T.nproc) * i] + (1 - w) * T.rate[j + size_t(T.nproc) * (i + 1)];
            Wk.near(nu, xi, L.r);
            if (nu > xi) break;
            xi -= nu;
        }
    } else {
        double t[4];
        bool oor = false;
        double edge = 1.0;
        int i = precheb(eng, T.k, T.xmax, T.order, t, oor, &edge);
        if (oor) Wk.err(E_TABLE_RANGE);
        Wk.near(edge, 0.0, 1.0);
        double xi = Wk.rand() * L.r;
        for (; j < T.nproc; ++j) {
            double nu = 0;
            for (int q = 0; q < T.order; ++q) nu += T.rate[q + T.order * (j + T.nproc * i)] * t[q];
            Wk.near(nu, xi, L.r);
            if (nu > xi) break;
            xi -= nu;
        }
    }
    if (j == T.nproc) {  // NullOutcome: setr!, s = nextcoll() (collisions.jl:83-88)
        Wk.C->nulls[species] += 1;
        L.r = setr(Wk, species);
        L.s = Wk.nextcoll();
        return;
    }
    Wk.C->coll[species][j] += 1;
    sample(Wk, T.procs[j], species, eng);
    if (L.active) L.r = setr(Wk, species);
    flush_kids(Wk, ctr0, out);
}

// The per-particle loop of advance1! (mixed_population.jl:60-84)
static void advance_one(Walker& Wk, int species, double tfinal, SpawnBuf& out) {
    Part& L = *Wk.P;
    if (!L.active) return;
    double trem = tfinal - L.t;
    int nsub = 0;
    for (;;) {
        Wk.near(trem, EPS_T, EPS_T);
        if (!(trem > EPS_T && L.active)) break;
        if (++nsub > SUBSTEP_CAP) { Wk.err(E_SUBSTEP_CAP); break; }
        double tnext = L.s / L.r;
        double dt;
        bool collides;
        if (std::isfinite(tnext)) Wk.near(trem, tnext, std::max(trem, tnext));
        if (trem > tnext) { dt = tnext; collides = true; }
        else { dt = trem; collides = false; L.s -= dt * L.r; }
        const Species& Sp = Wk.W->sp[species];
        double xo[3], po[3], to = L.t;
        if (Sp.wall_coord >= 0) { std::memcpy(xo, L.x, sizeof(xo)); std::memcpy(po, L.p, sizeof(po)); }
        advance_particle(Wk, species, dt);
        if (Sp.wall_coord >= 0) {
            // onadvance(WallCallback) (callback.jl:167-184): a crossing in the +axis
            // direction records lincomb(new, old, w) (electron.jl:127-132; its
            // constructor draws s) and drops the particle if asked to
            const int q = Sp.wall_coord;
            const double v = Sp.wall_v;
            Wk.near(L.x[q], v, std::fabs(L.x[q] - xo[q]) + std::fabs(v));
            Wk.near(xo[q], v, std::fabs(L.x[q] - xo[q]) + std::fabs(v));
            if (xo[q] < v && v < L.x[q]) {
                const double w = (v - xo[q]) / (L.x[q] - xo[q]);
                World::WallRec r;
                r.species = species;
                r.sid = L.sid;
                for (int a = 0; a < 3; ++a) {
                    r.x[a] = L.x[a] * w + xo[a] * (1 - w);
                    r.p[a] = L.p[a] * w + po[a] * (1 - w);
                }
                r.w = L.w;
                r.t = L.t * w + to * (1 - w);
                (void)Wk.rand();
                {
                    std::lock_guard<std::mutex> g(Wk.W->wall_mu);
                    Wk.W->wall.push_back(r);
                }
                if (Sp.wall_drop) L.active = false;
            }
        }
        if (collides && L.active) do_one_collision(Wk, species, out);
        trem -= dt;
    }
}

// advance!(mpopl, pusher, tfinal) + foreach(droplow!, mpopl)
// (mixed_population.jl:38-112, run.jl:7-8, population.jl:273-284)
static void advance(World& W, double tfinal, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    // advance_init!: setr! for every active particle
    for (int s = 0; s < 3; ++s) {
        for (auto& P : W.sp[s].parts) {
            if (!P.active) continue;
            Walker Wk{&P, &W, &W.cnt};
            P.r = setr(Wk, s);
        }
    }
    size_t iup[3] = {0, 0, 0};
    for (;;) {
        size_t total = 0;
        for (int s = 0; s < 3; ++s) {
            std::vector<Part>& parts = W.sp[s].parts;
            size_t ilast = parts.size();
            size_t n = ilast - iup[s];
            total += n;
            if (n > 0) {
                int nt = int(std::min<size_t>(nthreads, (n + 63) / 64));
                if (nt < 1) nt = 1;
                std::vector<SpawnBuf> bufs(nt);
                std::vector<Counters> cnts(nt);
                auto work = [&](int tid) {
                    size_t a = iup[s] + n * tid / nt, b = iup[s] + n * (tid + 1) / nt;
                    for (size_t i = a; i < b; ++i) {
                        Walker Wk{&parts[i], &W, &cnts[tid]};
                        advance_one(Wk, s, tfinal, bufs[tid]);
                    }
                };
                if (nt == 1) {
                    work(0);
                } else {
                    std::vector<std::thread> th;
                    for (int tid = 0; tid < nt; ++tid) th.emplace_back(work, tid);
                    for (auto& t : th) t.join();
                }
                for (int tid = 0; tid < nt; ++tid) {
                    W.cnt.add(cnts[tid]);
                    for (int q = 0; q < 3; ++q)
                        W.sp[q].parts.insert(W.sp[q].parts.end(), bufs[tid].q[q].begin(), bufs[tid].q[q].end());
                }
            }
            iup[s] = ilast;
        }
        if (total == 0) break;
    }
    // droplow!: deactivate active particles below the cut, then repack
    for (int s = 0; s < 3; ++s) {
        std::vector<Part>& parts = W.sp[s].parts;
        std::vector<Part> keep;
        keep.reserve(parts.size());
        for (auto& P : parts) {
            if (!P.active) continue;
            Walker Wk{&P, &W, &W.cnt};
            double E = kinenergy(s, P.p);
            Wk.near(E, W.sp[s].cut, W.sp[s].cut);
            if (E < W.sp[s].cut) continue;
            keep.push_back(P);
        }
        parts.swap(keep);
    }
}

}  // namespace orc

using namespace orc;

// ================================================================ C API ===
extern "C" {

void* orc_create(uint64_t seed, double tie_tol) {
    World* W = new World();
    W->k0 = uint32_t(seed);
    W->k1 = uint32_t(seed >> 32);
    W->tie_tol = tie_tol;
    return W;
}

void orc_destroy(void* w) { delete static_cast<World*>(w); }

int orc_set_species(void* w, int species, double cut, int tally_only) {
    World* W = static_cast<World*>(w);
    if (species < 0 || species > 2) return -1;
    W->sp[species].set = true;
    W->sp[species].cut = cut;
    W->sp[species].tally_only = tally_only != 0;
    W->sp[species].parts.clear();
    return 0;
}

// kinds/Z/nparam [nproc], params [nproc][8] (SI, meaning as in the library's pcl_process)
int orc_set_table(void* w, int species, int order, int nproc, int nint, double xmax, const double* rate,
                  const double* rb, const int32_t* kinds, const int32_t* Z, const double* params,
                  const int32_t* nparam) {
    World* W = static_cast<World*>(w);
    if (species < 0 || species > 2 || order < 1 || order > 4 || nproc < 0 || nproc > 16) return -1;
    Table& T = W->sp[species].tab;
    T.order = order; T.nproc = nproc; T.k = nint; T.xmax = xmax;
    T.rate.assign(rate, rate + size_t(order) * nproc * (nint + 1));
    T.rb.assign(rb, rb + size_t(order) * (nint + 1));
    T.procs.assign(nproc, Proc());
    for (int j = 0; j < nproc; ++j) {
        T.procs[j].kind = kinds[j];
        T.procs[j].Z = Z[j];
        T.procs[j].np = nparam[j];
        for (int q = 0; q < 8; ++q) T.procs[j].p[q] = params[8 * j + q];
    }
    return 0;
}

int orc_set_linear_table(void* w, int species, int nproc, int n, double e0, double e1, const double* rate,
                         const double* rb, const int32_t* kinds, const double* params) {
    World* W = static_cast<World*>(w);
    if (species < 0 || species > 2 || nproc < 0 || nproc > 16 || n < 2) return -1;
    Table& T = W->sp[species].tab;
    T = Table();
    T.linear = true;
    T.nproc = nproc; T.n = n; T.e0 = e0; T.e1 = e1;
    T.rate.assign(rate, rate + size_t(nproc) * n);
    T.rb.assign(rb, rb + n);
    T.procs.assign(nproc, Proc());
    for (int j = 0; j < nproc; ++j) {
        T.procs[j].kind = kinds[j];
        for (int q = 0; q < 8; ++q) T.procs[j].p[q] = params[8 * j + q];
    }
    return 0;
}

// swarm mode: E[nswarm][3] (V/m); rb_e / rb_p = per-swarm rate-bound tables of
// the electron / positron Chebyshev tables (NULL: keep the table's own)
int orc_set_swarms(void* w, int nswarm, const double* E, const double* rb_e, const double* rb_p) {
    World* W = static_cast<World*>(w);
    W->nswarm = nswarm;
    W->swarm_E.assign(E, E + 3 * size_t(nswarm));
    const double* src[3] = {rb_e, nullptr, rb_p};
    for (int s = 0; s < 3; ++s) {
        W->swarm_rb[s].clear();
        if (!src[s]) continue;
        const Table& T = W->sp[s].tab;
        size_t len = size_t(T.order) * (T.k + 1) * nswarm;
        W->swarm_rb[s].assign(src[s], src[s] + len);
    }
    return 0;
}

int orc_set_sb(void* w, int species, int j, int ne, int ncum, const double* log_energy, const double* data) {
    World* W = static_cast<World*>(w);
    Table& T = W->sp[species].tab;
    if (j < 0 || j >= T.nproc) return -1;
    T.procs[j].le.assign(log_energy, log_energy + ne);
    T.procs[j].data.assign(data, data + size_t(ne) * ncum);
    T.procs[j].ncum = ncum;
    return 0;
}

// roulette! / split! (population.jl:291-335) on the particles of a species,
// draws as the device takes them: one from the particle's stream each; split
// copies take stream ids from Philox block (ctr, sid, 2 + j/2) of the parent.
static uint32_t stream_word(const World& W, uint32_t ctr, uint64_t sid) {
    uint32_t a = ctr >> 2, b = uint32_t(sid), c2 = uint32_t(sid >> 32), d = 0;
    philox(a, b, c2, d, W.k0, W.k1);
    const uint32_t q[4] = {a, b, c2, d};
    return q[ctr & 3u];
}

int orc_roulette(void* w, int species, double pkeep) {
    World* W = static_cast<World*>(w);
    for (Part& P : W->sp[species].parts) {
        if (!P.active) continue;
        const uint32_t v = stream_word(*W, P.ctr, P.sid);
        const double u = double(((v >> 9) << 1) | 1u) * 5.9604644775390625e-8;
        P.ctr += 1;
        if (u < pkeep) P.w /= pkeep;
        else P.active = false;
    }
    auto& v = W->sp[species].parts;
    v.erase(std::remove_if(v.begin(), v.end(), [](const Part& q) { return !q.active; }), v.end());
    return 0;
}

// Poisson(p) by inversion for split!, the pmf summed in Float64 from exp(-p)
// as the device does it (p rounded to FP32 first; at most 1024 copies)
static int poisson_inv(float pf, float u) {
    int k = 0;
    const double pd = double(pf);
    double P = std::exp(-pd), F = P;
    while (double(u) > F && k < 1024) { ++k; P = P * (pd / double(k)); F = F + P; }
    return k;
}

int orc_poisson_inv(double p, double u) { return poisson_inv(float(p), float(u)); }

int orc_split(void* w, int species, double p) {
    World* W = static_cast<World*>(w);
    auto& v = W->sp[species].parts;
    const size_t n0 = v.size();
    const float pf = float(p);
    for (size_t i = 0; i < n0; ++i) {
        if (!v[i].active) continue;
        v[i].w /= (1.0 + p);
        const uint32_t word = stream_word(*W, v[i].ctr, v[i].sid);
        const uint32_t ctr0 = v[i].ctr;
        v[i].ctr += 1;
        const float u = float(double(((word >> 9) << 1) | 1u) * 5.9604644775390625e-8);
        const int k = poisson_inv(pf, u);
        for (int j = 0; j < k; ++j) {
            uint32_t a = ctr0, b = uint32_t(v[i].sid), c2 = uint32_t(v[i].sid >> 32), d = 2u + uint32_t(j >> 1);
            philox(a, b, c2, d, W->k0, W->k1);
            Part q = v[i];
            q.sid = (j & 1) ? (uint64_t(c2) | (uint64_t(d) << 32)) : (uint64_t(a) | (uint64_t(b) << 32));
            if (W->nswarm > 0)   // the copy stays in its parent's swarm (top 8 bits of the stream id)
                q.sid = (q.sid & 0x00FFFFFFFFFFFFFFull) | (v[i].sid & 0xFF00000000000000ull);
            q.ctr = 0;
            v.push_back(q);
        }
    }
    return 0;
}

// f(E) of a table (energies in J, ascending), linear in E between nodes and
// constant beyond the ends, as the device evaluates it: v_i + (E - E_i) s_i
// with the interval's slope s_i (population.jl:291-305 and 316-331 take f as
// a function; the library takes it tabulated).
static double table_fn(const double* tE, const double* tV, int n, double e) {
    if (!(e > tE[0])) return tV[0];
    if (!(e < tE[n - 1])) return tV[n - 1];
    const int lo = int(std::upper_bound(tE, tE + n, e) - tE) - 1;
    const double s = (tV[lo + 1] - tV[lo]) / (tE[lo + 1] - tE[lo]);
    return std::fma(e - tE[lo], s, tV[lo]);
}

// roulette!(f, popl) (population.jl:291-305) with f(kinenergy) from a table;
// the keep probability rounded to FP32 as the device holds it
int orc_roulette_fn(void* w, int species, int n, const double* tE, const double* tV) {
    World* W = static_cast<World*>(w);
    for (Part& P : W->sp[species].parts) {
        if (!P.active) continue;
        const double q = double(float(table_fn(tE, tV, n, kinenergy(species, P.p))));
        const uint32_t v = stream_word(*W, P.ctr, P.sid);
        const double u = double(((v >> 9) << 1) | 1u) * 5.9604644775390625e-8;
        P.ctr += 1;
        if (u < q) P.w /= q;
        else P.active = false;
    }
    auto& v = W->sp[species].parts;
    v.erase(std::remove_if(v.begin(), v.end(), [](const Part& q) { return !q.active; }), v.end());
    return 0;
}

// split!(f, popl) (population.jl:316-331) with the mean number of copies
// f(kinenergy) from a table, rounded to FP32 as the device holds it
int orc_split_fn(void* w, int species, int n, const double* tE, const double* tV) {
    World* W = static_cast<World*>(w);
    auto& v = W->sp[species].parts;
    const size_t n0 = v.size();
    for (size_t i = 0; i < n0; ++i) {
        if (!v[i].active) continue;
        const float pf = float(table_fn(tE, tV, n, kinenergy(species, v[i].p)));
        v[i].w /= (1.0 + double(pf));
        const uint32_t word = stream_word(*W, v[i].ctr, v[i].sid);
        const uint32_t ctr0 = v[i].ctr;
        v[i].ctr += 1;
        const float u = float(double(((word >> 9) << 1) | 1u) * 5.9604644775390625e-8);
        const int k = poisson_inv(pf, u);
        for (int j = 0; j < k; ++j) {
            uint32_t a = ctr0, b = uint32_t(v[i].sid), c2 = uint32_t(v[i].sid >> 32), d = 2u + uint32_t(j >> 1);
            philox(a, b, c2, d, W->k0, W->k1);
            Part q = v[i];
            q.sid = (j & 1) ? (uint64_t(c2) | (uint64_t(d) << 32)) : (uint64_t(a) | (uint64_t(b) << 32));
            if (W->nswarm > 0)
                q.sid = (q.sid & 0x00FFFFFFFFFFFFFFull) | (v[i].sid & 0xFF00000000000000ull);
            q.ctr = 0;
            v.push_back(q);
        }
    }
    return 0;
}

int orc_set_wall(void* w, int species, int coord, double v, int drop) {
    World* W = static_cast<World*>(w);
    W->sp[species].wall_coord = coord;
    W->sp[species].wall_v = v;
    W->sp[species].wall_drop = drop != 0;
    return 0;
}

// wall records so far: species, sid, x[3n], p[3n], w, t; returns the count
// (arrays may be NULL to query it)
int64_t orc_get_wall(void* w, int32_t* species, uint64_t* sid, double* x, double* p, double* wt, double* t) {
    World* W = static_cast<World*>(w);
    const size_t n = W->wall.size();
    if (species) {
        for (size_t i = 0; i < n; ++i) {
            const World::WallRec& r = W->wall[i];
            species[i] = r.species; sid[i] = r.sid; wt[i] = r.w; t[i] = r.t;
            for (int a = 0; a < 3; ++a) { x[3 * i + a] = r.x[a]; p[3 * i + a] = r.p[a]; }
        }
    }
    return int64_t(n);
}

// position-dependent E (SI): kind 1 {z1, z2, vx, vy, vz}, 2 {z, v1[3], v2[3]}, 3 {sx, sy, sz, ez0}
int orc_set_field(void* w, int kind, const double* params, int n) {
    World* W = static_cast<World*>(w);
    W->field_kind = kind;
    for (int i = 0; i < 8; ++i) W->fp[i] = (i < n) ? params[i] : 0.0;
    return 0;
}

int orc_set_bfield(void* w, int kind, const double* params, int n) {
    World* W = static_cast<World*>(w);
    W->bfield_kind = kind;
    for (int i = 0; i < 8; ++i) W->bp[i] = (i < n) ? params[i] : 0.0;
    return 0;
}

int orc_set_push_mask(void* w, int push, int field, int loss) {
    World* W = static_cast<World*>(w);
    W->push_mask = push; W->field_mask = field; W->loss_mask = loss;
    return 0;
}

int orc_set_forcing(void* w, const double* E, const double* B, int cl_order, int cl_k, double cl_xmax,
                    const double* ec, const double* pc) {
    World* W = static_cast<World*>(w);
    for (int a = 0; a < 3; ++a) { W->E[a] = E[a]; W->B[a] = B[a]; }
    W->cl_order = cl_order;
    if (cl_order > 0) {
        W->cl_k = cl_k;
        W->cl_xmax = cl_xmax;
        W->ec.assign(ec, ec + size_t(cl_order) * (cl_k + 1));
        W->pc.assign(pc, pc + size_t(cl_order) * (cl_k + 1));
    }
    return 0;
}

int orc_upload(void* w, int species, int64_t n, const double* x, const double* p, const double* wt,
               const double* t, const double* s, const uint64_t* sid, const uint32_t* ctr) {
    World* W = static_cast<World*>(w);
    std::vector<Part>& parts = W->sp[species].parts;
    parts.clear();
    parts.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        Part& P = parts[i];
        for (int a = 0; a < 3; ++a) { P.x[a] = x[3 * i + a]; P.p[a] = p[3 * i + a]; }
        P.w = wt[i]; P.t = t[i]; P.s = s[i]; P.r = 0; P.active = true;
        P.sid = sid[i]; P.ctr = ctr[i]; P.tie = 0;
    }
    return 0;
}

int orc_advance(void* w, double tfinal, int nthreads) {
    advance(*static_cast<World*>(w), tfinal, nthreads);
    return 0;
}

int64_t orc_count(void* w, int species) { return int64_t(static_cast<World*>(w)->sp[species].parts.size()); }

int orc_download(void* w, int species, double* x, double* p, double* wt, double* t, double* s, uint64_t* sid,
                 uint32_t* ctr, uint8_t* tie) {
    World* W = static_cast<World*>(w);
    const std::vector<Part>& parts = W->sp[species].parts;
    for (size_t i = 0; i < parts.size(); ++i) {
        const Part& P = parts[i];
        for (int a = 0; a < 3; ++a) { x[3 * i + a] = P.x[a]; p[3 * i + a] = P.p[a]; }
        wt[i] = P.w; t[i] = P.t; s[i] = P.s; sid[i] = P.sid; ctr[i] = P.ctr; tie[i] = P.tie;
    }
    return 0;
}

// coll[48], nulls[3], spawned[3], tally_count[3], err[8] (int64); tally_w[3], tally_wE[3] (J)
int orc_counters(void* w, int64_t* coll, int64_t* nulls, int64_t* spawned, int64_t* tally_count,
                 double* tally_w, double* tally_wE, int64_t* err, int64_t* ties) {
    const Counters& C = static_cast<World*>(w)->cnt;
    for (int s = 0; s < 3; ++s) {
        for (int j = 0; j < 16; ++j) coll[16 * s + j] = C.coll[s][j];
        nulls[s] = C.nulls[s]; spawned[s] = C.spawned[s]; tally_count[s] = C.tally_count[s];
        tally_w[s] = C.tally_w[s]; tally_wE[s] = C.tally_wE[s];
    }
    for (int q = 0; q < 8; ++q) err[q] = C.err[q];
    *ties = C.ties;
    return 0;
}

void orc_reset_counters(void* w) { static_cast<World*>(w)->cnt = Counters(); }

// Mirror of the library's sampler test hook: force table position j for n
// primaries with momentum p (SI), stream sid, counter 0; records the
// outcome without applying cuts.
int orc_sample(void* w, int species, int j, int64_t n, const double* p, const uint64_t* sid, double* out_p,
               double* out_s, int32_t* out_kind, uint32_t* out_ctr, uint8_t* out_tie) {
    World* W = static_cast<World*>(w);
    const Table& T = W->sp[species].tab;
    if (j < 0 || j >= T.nproc) return -1;
    Counters C;
    for (int64_t i = 0; i < n; ++i) {
        Part P;
        std::memset(&P, 0, sizeof(P));
        for (int a = 0; a < 3; ++a) P.p[a] = p[3 * i + a];
        P.w = 1; P.active = true; P.sid = sid[i]; P.ctr = 0;
        Walker Wk{&P, W, &C};
        double eng = kinenergy(species, P.p);
        sample(Wk, T.procs[j], species, eng);
        for (int q = 0; q < 3; ++q) out_kind[3 * i + q] = -1;
        for (int q = 0; q < 9; ++q) out_p[9 * i + q] = 0;
        if (P.active) {
            for (int a = 0; a < 3; ++a) out_p[9 * i + a] = P.p[a];
            out_s[3 * i] = P.s;
            out_kind[3 * i] = species;
        }
        for (int q = 0; q < Wk.nkids; ++q) {
            for (int a = 0; a < 3; ++a) out_p[9 * i + 3 * (q + 1) + a] = Wk.kids[q].p[a];
            out_s[3 * i + q + 1] = Wk.kids[q].s;
            out_kind[3 * i + q + 1] = Wk.kids[q].species;
        }
        out_ctr[i] = P.ctr;
        out_tie[i] = P.tie;
    }
    return 0;
}

// Philox4x32-10 known-answer hook
void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    uint32_t a = ctr[0], b = ctr[1], c2 = ctr[2], d = ctr[3];
    philox(a, b, c2, d, key[0], key[1]);
    out[0] = a; out[1] = b; out[2] = c2; out[3] = d;
}

}  // extern "C"
