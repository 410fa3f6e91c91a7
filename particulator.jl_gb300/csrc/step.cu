// GB300 (sm_103a) kernels of the null-collision Monte Carlo step.
//
// One thread owns one particle at a time and runs the reference's per-particle
// sub-step loop (advance1!, mixed_population.jl:56-93): null-collision clock
// s / r, Ralston RK2 push (pusher.jl:41-63) with the homogeneous field and the
// Chebyshev continuum loss (field.jl:54-70, continuum.jl:45-57), and, at the
// end of a sub-step that reaches the clock, do_one_collision!
// (collisions.jl:142-199): Chebyshev rates on binary intervals (cheby.jl:127-143,
// collision_table.jl:82-106), linear scan of xi = U r, then one of the
// process samplers.  Lanes are refilled after every sub-step, so a warp never
// idles on lanes whose particle finished early: an idle lane first pops a
// secondary from its warp's child stack in shared memory (secondaries are
// advanced from their birth time to the end of the step, as the reference's
// repeated advance1! passes do, mixed_population.jl:43-46), then takes the
// next input slot from a warp-private chunk of the work space.
//
// Every random number comes from the particle's own Philox4x32-10 stream
// (Salmon et al., SC'11): key = context seed, counter = (draw / 4, sid_lo,
// sid_hi, 0).  A secondary's stream id is drawn from the parent's stream in a
// separate counter domain, so results do not depend on thread scheduling.
// Each uniform is u = (2 floor(x / 2^9) + 1) 2^-24, exactly representable in
// FP32 and FP64, in (0, 1).
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "device.cuh"
#include "../../include/particulator_gb300.h"

// Samplers of rare events (photon, positron, bremsstrahlung, swarm) are inlined
// (measured faster than out-of-line calls, whose ABI spills in the 64-register
// build); PCL_OUTLINE_RARE keeps them out of line instead.
#ifdef PCL_OUTLINE_RARE
#define PCL_RARE __noinline__
#else
#define PCL_RARE __forceinline__
#endif

namespace pcl {

constexpr int   kWarpStack   = 32;          // child-stack entries per warp
constexpr int   kCollStash   = PCL_STASH_MAX;  // event kernel: per-warp entries, parked collisions from the
                                            // bottom and held particles from the top
constexpr int   kBatchMin    = 24;          // event kernel: free lanes that collide without the hold
constexpr int   kRejectCap   = 10000;       // rejection-loop iteration cap
constexpr int   kSubstepCap  = 1 << 20;     // sub-steps per particle per step
constexpr float kEpsT        = 2.220446049250313e-7f;  // eps(Float64) s in ns (mixed_population.jl:66)
constexpr float kCns         = 0.299792458f;           // c in m/ns

// block-tally word offsets (uint32 in shared memory)
constexpr int T_COLL = 0;              // [3][16]
constexpr int T_NULL = 48;             // [3]
constexpr int T_SPAWN = 51;            // [3]
constexpr int T_DEAD = 54;             // [3]
constexpr int T_ERR = 57;              // [8]
constexpr int T_LEND = 65;             // [64][3]
constexpr int T_LSTART = T_LEND + 3 * PCL_MAX_STEPS_PER_LAUNCH;  // [64]
constexpr int T_FLY = T_LSTART + PCL_MAX_STEPS_PER_LAUNCH;       // [64] photon flights over whole steps (differences)
constexpr int T_WORDS = T_FLY + PCL_MAX_STEPS_PER_LAUNCH;         // 385

// ------------------------------------------------------------ Philox ----
__device__ __forceinline__ void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                              uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

// ----------------------------------------------------------- lane state --
struct Lane {
    float x, y, z, w;
    float px, py, pz, s;
    float r;
    float th, tlo;             // time left in the current step (ns), as an unevaluated
                               // sum th + tlo (double-float: ~48-bit precision on FP32 pipes)
    uint32_t sid_lo, sid_hi, ctr;
    uint32_t c0, c1, c2, c3;   // Philox words not yet consumed (front = c0)
    int slot;                  // input slot, or -1 for a secondary (appended on finish)
    int species;
    int sw;                    // swarm of a batched context (top 8 bits of the stream id)
    int k;                     // time step within this launch
    int nsub;
    bool alive, rvalid;
};


// Double-float arithmetic for the per-particle step clock (Knuth's TwoSum and
// Dekker's Fast2Sum; only additions, so no contraction can break them).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
// (th, tlo) += (ah, al)
__device__ __forceinline__ void dd_add(float& th, float& tlo, float ah, float al) {
    float s, e;
    two_sum(th, ah, s, e);
    e = __fadd_rn(e, __fadd_rn(tlo, al));
    fast_two_sum(s, e, th, tlo);
}
__device__ __forceinline__ float dd_val(float th, float tlo) { return __fadd_rn(th, tlo); }

struct KCtx {
    const BlobHdr* H;
    const float* blob;
    float4* stk;       // this warp's child stack: entry e = stk[3e .. 3e+2]
    int* top;          // this warp's stack top
    uint32_t* tal;     // block tallies
    const StepArgs* A;
    // test-hook capture of secondaries (pcl_test_sampler): when non-null,
    // secondaries go to cap[0..1] instead of the stack
    float* cap;
    int* ncap;
    bool hasB = true;    // a magnetic field is set (v x B is skipped when B = 0)
    bool eregs = false;  // the homogeneous E field is held in E0..E2 (multi-step instance)
    float E0 = 0.0f, E1 = 0.0f, E2 = 0.0f;
};

__device__ __forceinline__ uint32_t next_bits(Lane& L, uint32_t k0, uint32_t k1) {
    uint32_t sh = L.ctr & 3u;
    if (!L.rvalid || sh == 0u) {
        uint32_t a = L.ctr >> 2, b = L.sid_lo, c = L.sid_hi, d = 0u;
        philox4x32_10(a, b, c, d, k0, k1);
        if (sh == 0u) { L.c0 = a; L.c1 = b; L.c2 = c; L.c3 = d; }
        else if (sh == 1u) { L.c0 = b; L.c1 = c; L.c2 = d; }
        else if (sh == 2u) { L.c0 = c; L.c1 = d; }
        else { L.c0 = d; }
        L.rvalid = true;
    }
    uint32_t v = L.c0;
    L.c0 = L.c1; L.c1 = L.c2; L.c2 = L.c3;
    L.ctr += 1u;
    return v;
}

// (2 (v >> 9) + 1) 2^-24, in (0, 1), without an integer-to-float conversion:
// 1 + (v >> 9) 2^-23 is built in the mantissa, subtracting 1 is exact, and so is
// adding 2^-24 (the result has at most 24 significant bits).
__device__ __forceinline__ float bits_to_u(uint32_t v) {
    return __fadd_rn(__fsub_rn(__uint_as_float(0x3f800000u | (v >> 9)), 1.0f), 5.9604644775390625e-8f);
}

__device__ __forceinline__ float U(Lane& L, const KCtx& K) {
    return bits_to_u(next_bits(L, K.A->key0, K.A->key1));
}

// nextcoll() = -log(rand()) (util.jl:17)
__device__ __forceinline__ float nextcoll(Lane& L, const KCtx& K) { return -logf(U(L, K)); }

__device__ __forceinline__ void err(const KCtx& K, int e) { atomicAdd(&K.tal[T_ERR + e], 1u); }

// ------------------------------------------------------------ kinematics --
// kinenergy (electron.jl:53, positron.jl:40, photon.jl:50) with the
// cancellation-free form p^2 / (gamma + 1) for leptons (device units).
__device__ __forceinline__ float kin_energy(int species, float px, float py, float pz) {
    float p2 = px * px + py * py + pz * pz;
    if (species == PCL_PHOTON) return sqrtf(p2);
    // p^2/(gamma + 1) = p^2 (1/gamma) / (1 + 1/gamma)
    float ig = rsqrtf(1.0f + p2);
    return __fdividef(p2 * ig, 1.0f + ig);
}

// The same with IEEE square root and division: used once per collision for the
// energy handed to setr! and the samplers, where FP32 rounding feeds decisions.
__device__ __forceinline__ float kin_energy_exact(int species, float px, float py, float pz) {
    float p2 = px * px + py * py + pz * pz;
    if (species == PCL_PHOTON) return sqrtf(p2);
    return p2 / (sqrtf(1.0f + p2) + 1.0f);
}

// precheb (cheby.jl:127-143).  Energies beyond the table (x >= xmax, where the
// reference indexes past its array) extrapolate the last interval.
__device__ __forceinline__ int precheb(float x, int k, float xscale, float t[4], bool& oor) {
    float x1 = x * xscale;
    uint32_t bits = __float_as_uint(x1);
    int e = int((bits >> 23) & 0xffu);
    int i;
    float xi;
    float two_k1 = __uint_as_float(uint32_t(127 + k + 1) << 23);
    if (!(x1 > 0.0f) || e == 0) {
        i = 0;
        xi = two_k1 * x1 - 1.0f;
    } else {
        i = (e - 126) + k;
        if (i > 0) {
            float s = __uint_as_float((bits & 0x807fffffu) | 0x3f000000u);
            xi = 4.0f * s - 3.0f;
            if (i > k) {
                oor = true;
                i = k;
                xi = 4.0f * x1 - 3.0f;
            }
        } else {
            i = 0;
            xi = two_k1 * x1 - 1.0f;
        }
    }
    t[0] = 1.0f;
    t[1] = xi;
    t[2] = 2.0f * xi * t[1] - t[0];
    t[3] = 2.0f * xi * t[2] - t[1];
    return i;
}

__device__ __forceinline__ float cheb_dot(const float* a, const float t[4], int order) {
    float s = a[0] * t[0];
    if (order > 1) s += a[1] * t[1];
    if (order > 2) s += a[2] * t[2];
    if (order > 3) s += a[3] * t[3];
    return s;
}

// setr! (collisions.jl:63-74): r = ratebound(E) above the cut, else 0.
// indweight(LinRange, x) (util.jl:23-32): left grid point i and weight w of
// point i (1 - w of point i + 1).  Outside the grid the end interval is
// extrapolated (the reference asserts 0 <= w <= 1 there).
__device__ __forceinline__ int lin_index(const SpeciesHdr& S, const KCtx& K, float E, float& w) {
    float u = (E - S.lin_e0) * S.lin_inv_step;
    int i = int(floorf(u));
    if (i < 0) { i = 0; err(K, PCL_E_TABLE_RANGE); }
    else if (i > S.lin_n - 2) { i = S.lin_n - 2; err(K, PCL_E_TABLE_RANGE); }
    w = float(i + 1) - u;
    return i;
}

__device__ __forceinline__ float setr(const SpeciesHdr& S, const KCtx& K, float E, int sw) {
    if (E < S.cut) return 0.0f;
    float rb;
    if (S.table_kind == 1) {  // ratebound(::CollisionTable) (collision_table.jl:32-43)
        float w;
        int i = lin_index(S, K, E, w);
        const float* b = K.blob + S.rb_off + i;
        rb = w * b[0] + (1.0f - w) * b[1];
    } else {
        float t[4];
        bool oor = false;
        int i = precheb(E, S.k, S.xscale, t, oor);
        if (oor) err(K, PCL_E_TABLE_RANGE);
        rb = cheb_dot(K.blob + S.rb_off + i * S.order, t, S.order);
        if (S.rbB_off >= 0) {  // batched swarms: compratebound is linear in Fdt
            const float fdt = K.blob[K.H->swarm_off + 4 * sw + 3];   // Fdt (N s)
            rb += fdt * cheb_dot(K.blob + S.rbB_off + i * S.order, t, S.order);
        }
    }
    if (!(rb > 0.0f)) {
        if (S.nproc > 0) err(K, PCL_E_NEG_RATE);
        return 0.0f;
    }
    return rb;
}

// ChebContinuumLoss.force magnitude (continuum.jl:45-57), device force units.
__device__ __forceinline__ float cl_mag(const SpeciesHdr& S, const KCtx& K, float E) {
    if (S.cl_off < 0) return 0.0f;
    float t[4];
    bool oor = false;
    int i = precheb(E, S.cl_k, S.cl_xscale, t, oor);
    if (oor) err(K, PCL_E_TABLE_RANGE);
    return cheb_dot(K.blob + S.cl_off + i * S.cl_order, t, S.cl_order);
}

// A field of field.jl:4-52 at position (x, y, z): kind 0 the homogeneous
// value h, 1 double layer, 2 step, 3 confined double layer (parameters f).
__device__ __forceinline__ void field_at(int kind, const float* f, const float* h, float x, float y, float z,
                                         float& ex, float& ey, float& ez) {
    switch (kind) {
        case 1: {  // DoubleLayerField
            const bool in = f[0] < z && z < f[1];
            ex = in ? f[2] : 0.0f; ey = in ? f[3] : 0.0f; ez = in ? f[4] : 0.0f;
            break;
        }
        case 2: {  // StepField
            const bool below = z < f[0];
            ex = below ? f[1] : f[4]; ey = below ? f[2] : f[5]; ez = below ? f[3] : f[6];
            break;
        }
        case 3: {  // ConfinedDoubleLayerField: f = {1/(2 sx^2), 1/(2 sy^2), 1/(2 sz^2), ez0, 1/sx^2, 1/sy^2, 1/sz^2}
            const float g = f[3] * expf(-(x * x * f[0] + y * y * f[1] + z * z * f[2]));
            ex = -(g * x * z) * f[4];
            ey = -(g * y * z) * f[5];
            ez = g - (g * z * z) * f[6];
            break;
        }
        default:
            ex = h[0]; ey = h[1]; ez = h[2];
    }
}

// E at position (x, y, z); a batched swarm's own field wins.
__device__ __forceinline__ void efield(const KCtx& K, int sw, float x, float y, float z, float& ex, float& ey,
                                       float& ez) {
    const BlobHdr* H = K.H;
    if (H->nswarm > 0) {
        const float* E = K.blob + H->swarm_off + 4 * sw;
        ex = E[0]; ey = E[1]; ez = E[2];
        return;
    }
    field_at(H->field_kind, H->fp, H->E, x, y, z, ex, ey, ez);
}

// force(CombinedForcing(ElectromagneticField, ChebContinuumLoss), lepton)
// (pusher.jl:14-23, field.jl:54-70, continuum.jl:45-57) at position (x, y, z);
// GENERAL = false: homogeneous E (or the swarm's), position unused.
// Returns beta too.
template <bool GENERAL>
__device__ __forceinline__ void lepton_force(const SpeciesHdr& S, const KCtx& K, int sw, float x, float y, float z,
                                             float px, float py, float pz, float& bx, float& by, float& bz,
                                             float& fx, float& fy, float& fz) {
    // Every product and sum below is rounded explicitly (no contraction left
    // to the compiler), so that each instance of the step kernel, and each
    // place it is inlined, gives the same bits.
    float p2 = __fmaf_rn(pz, pz, __fmaf_rn(py, py, __fmul_rn(px, px)));
    float ig = rsqrtf(1.0f + p2);   // 1 / gamma
    bx = __fmul_rn(px, ig); by = __fmul_rn(py, ig); bz = __fmul_rn(pz, ig);
    const float q = S.charge;
    float ex, ey, ez;
    if (GENERAL) {
        efield(K, sw, x, y, z, ex, ey, ez);
    } else {
        if (K.eregs) {
            ex = K.E0; ey = K.E1; ez = K.E2;
        } else {
            const float* E = (K.H->nswarm > 0) ? K.blob + K.H->swarm_off + 4 * sw : K.H->E;
            ex = E[0]; ey = E[1]; ez = E[2];
        }
    }
    if (K.hasB) {
        float B[3];
        if (GENERAL) field_at(K.H->bfield_kind, K.H->bp, K.H->B, x, y, z, B[0], B[1], B[2]);
        else { B[0] = K.H->B[0]; B[1] = K.H->B[1]; B[2] = K.H->B[2]; }
        fx = __fmul_rn(q, __fadd_rn(ex, __fmaf_rn(by, B[2], -__fmul_rn(bz, B[1]))));
        fy = __fmul_rn(q, __fadd_rn(ey, __fmaf_rn(bz, B[0], -__fmul_rn(bx, B[2]))));
        fz = __fmul_rn(q, __fadd_rn(ez, __fmaf_rn(bx, B[1], -__fmul_rn(by, B[0]))));
    } else {  // the same values: adding the zero v x B term changes no finite component
        fx = __fmul_rn(q, ex); fy = __fmul_rn(q, ey); fz = __fmul_rn(q, ez);
    }
    float f = cl_mag(S, K, __fdividef(__fmul_rn(p2, ig), 1.0f + ig));
    if (f != 0.0f && p2 > 0.0f) {
        float c = __fmul_rn(f, rsqrtf(p2));
        fx = __fmaf_rn(-c, px, fx); fy = __fmaf_rn(-c, py, fy); fz = __fmaf_rn(-c, pz, fz);
    }
}

// advance_particle(RK2Pusher, y, dt) (pusher.jl:41-63); photons move in a
// straight line (photon.jl:46-52; both forcings vanish on photons).  Rounded
// explicitly like lepton_force: a photon's flight over whole steps in the
// multi-step instances and its steps in the loop give the same bits.
template <bool GENERAL>
__device__ __forceinline__ void push(Lane& L, const SpeciesHdr& S, const KCtx& K, float h) {
    if (L.species == PCL_PHOTON) {
        const float p2 = __fmaf_rn(L.pz, L.pz, __fmaf_rn(L.py, L.py, __fmul_rn(L.px, L.px)));
        const float v = __fmul_rn(__fmul_rn(h, kCns), rsqrtf(p2));
        L.x = __fmaf_rn(v, L.px, L.x); L.y = __fmaf_rn(v, L.py, L.y); L.z = __fmaf_rn(v, L.pz, L.z);
        return;
    }
    float b1x, b1y, b1z, f1x, f1y, f1z;
    lepton_force<GENERAL>(S, K, L.sw, L.x, L.y, L.z, L.px, L.py, L.pz, b1x, b1y, b1z, f1x, f1y, f1z);
    const float h23 = __fmul_rn(h, 2.0f / 3.0f);
    const float qx = __fmaf_rn(h23, f1x, L.px), qy = __fmaf_rn(h23, f1y, L.py), qz = __fmaf_rn(h23, f1z, L.pz);
    // second stage at x + 2 dt v1 / 3 (only a position-dependent field reads it)
    const float c23 = GENERAL ? __fmul_rn(h23, kCns) : 0.0f;
    float b2x, b2y, b2z, f2x, f2y, f2z;
    lepton_force<GENERAL>(S, K, L.sw, __fmaf_rn(c23, b1x, L.x), __fmaf_rn(c23, b1y, L.y), __fmaf_rn(c23, b1z, L.z),
                          qx, qy, qz, b2x, b2y, b2z, f2x, f2y, f2z);
    const float hc = __fmul_rn(h, kCns);
    L.x = __fmaf_rn(hc, __fmaf_rn(0.75f, b2x, __fmul_rn(0.25f, b1x)), L.x);
    L.y = __fmaf_rn(hc, __fmaf_rn(0.75f, b2y, __fmul_rn(0.25f, b1y)), L.y);
    L.z = __fmaf_rn(hc, __fmaf_rn(0.75f, b2z, __fmul_rn(0.25f, b1z)), L.z);
    L.px = __fmaf_rn(h, __fmaf_rn(0.75f, f2x, __fmul_rn(0.25f, f1x)), L.px);
    L.py = __fmaf_rn(h, __fmaf_rn(0.75f, f2y, __fmul_rn(0.25f, f1y)), L.py);
    L.pz = __fmaf_rn(h, __fmaf_rn(0.75f, f2z, __fmul_rn(0.25f, f1z)), L.pz);
}

// The general kernel's push (one call site of push<true>, whose field
// evaluations are the larger part of its code), with the WallCallback's
// onadvance (callback.jl:167-184) when the species has a wall: a crossing of
// the wall in the +axis direction records lincomb(new, old, w) (electron.jl:
// 127-132), whose constructor draws s (one draw), and drops the particle if
// the wall is set to.  The sub-step starts (k + 1) dt - th in ns since the
// launch start (dt_hi: dt in ns).
__device__ __forceinline__ void push_general(Lane& L, const SpeciesHdr& S, const KCtx& K, float h, float dt_hi) {
    if (S.frozen) return;   // RestrictedPusher / NullPusher (pusher.jl:73, 76): the clock only
    const float ox = L.x, oy = L.y, oz = L.z, opx = L.px, opy = L.py, opz = L.pz;
    const float t_in = __fmaf_rn(float(L.k + 1), dt_hi, -dd_val(L.th, L.tlo));
    push<true>(L, S, K, h);
    const int q = S.wall_coord;
    if (q < 0) return;
    const float o = (q == 0) ? ox : (q == 1 ? oy : oz);
    const float n = (q == 0) ? L.x : (q == 1 ? L.y : L.z);
    const float v = S.wall_v;
    if (!(o < v && v < n)) return;
    const float w = (v - o) / (n - o), u = 1.0f - w;
    const StepArgs& A = *K.A;
    const unsigned long long r = atomicAdd(A.wall_n, 1ull);
    if ((long long)r < A.wall_cap) {
        A.wall_xw[r] = make_float4(__fmaf_rn(L.x, w, __fmul_rn(ox, u)), __fmaf_rn(L.y, w, __fmul_rn(oy, u)),
                                   __fmaf_rn(L.z, w, __fmul_rn(oz, u)), L.w);
        A.wall_pt[r] = make_float4(__fmaf_rn(L.px, w, __fmul_rn(opx, u)), __fmaf_rn(L.py, w, __fmul_rn(opy, u)),
                                   __fmaf_rn(L.pz, w, __fmul_rn(opz, u)), __fmaf_rn(w, h, t_in));
        A.wall_meta[r] = make_uint4(L.sid_lo, L.sid_hi, uint32_t(L.species), A.ctl->launch_seq);
    } else {
        err(K, PCL_E_CAPACITY);
    }
    (void)U(L, K);
    if (S.wall_drop) L.alive = false;
}

// turn(u, cos theta, phi, n) (util.jl:40-57).  s = hypot(mu_x, mu_y) replaces
// sqrt(1 - mu_z^2) (identical for a unit vector, but free of the singularity
// at mu_z = +-1); at s = 0 the azimuth reference is the x axis.  sin theta is
// passed in, computed by each sampler without cancellation.
__device__ __forceinline__ void turn(float ux, float uy, float uz, float cth, float sth, float cph,
                                     float sph, float n, float& ox, float& oy, float& oz) {
    float iu = rsqrtf(ux * ux + uy * uy + uz * uz);
    float mx = ux * iu, my = uy * iu, mz = uz * iu;
    float s2 = mx * mx + my * my;
    float s = 0.0f, ca = 1.0f, sa = 0.0f;
    if (s2 > 0.0f) { float is = rsqrtf(s2); s = s2 * is; ca = mx * is; sa = my * is; }
    float ax = sth * (ca * mz * cph - sa * sph) + mx * cth;
    float ay = sth * (sa * mz * cph + ca * sph) + my * cth;
    float az = -s * sth * cph + mz * cth;
    ox = n * ax; oy = n * ay; oz = n * az;
}

// sample_modified_tsai_cos_theta(T) (util.jl:143-159); returns x = u^2/umax^2,
// cos theta = 1 - 2x.
__device__ __forceinline__ float tsai_x(Lane& L, const KCtx& K, float T) {
    const float umax = 2.0f * (1.0f + T);
    float u = 0.0f;
    int it = 0;
    for (;;) {
        float r1 = U(L, K);
        float r2 = U(L, K);
        float uu = -logf(r1 * r2);
        float r3 = U(L, K);
        u = (0.25f > r3) ? uu * 1.6f : uu * (1.6f / 3.0f);
        if (u <= umax) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); u = umax; break; }
    }
    float q = u / umax;
    return q * q;
}

__device__ __forceinline__ void sincos_2pi(float u, float& s, float& c) { sincospif(2.0f * u, &s, &c); }

// Lehtinen angles for a binary collision (moller.jl:26-28): energies E0
// (primary before), Ei (outgoing), d = E0 - Ei.  sin^2 = 2 d / (E0 (Ei + 2)).
__device__ __forceinline__ void lehtinen(float E0, float Ei, float d, float& c, float& s) {
    float den = E0 * (Ei + 2.0f);
    c = sqrtf(Ei * (E0 + 2.0f) / den);
    s = sqrtf(2.0f * d / den);
}

// add_particle! (population.jl:103-113) of a secondary born in a collision.
// The secondary's stream id comes from the parent's stream in domain 1 at the
// parent's counter at the start of the collision; child index 0 / 1 takes
// words (0,1) / (2,3).
__device__ void emit(Lane& L, const KCtx& K, int sp, float cpx, float cpy, float cpz, float cs,
                     int cidx, uint32_t ctr0) {
    const SpeciesHdr& S = K.H->sp[sp];
    float E = kin_energy(sp, cpx, cpy, cpz);
    if (K.cap) {  // test hook: record every outcome, cut applied by the caller
        int n = *K.ncap;
        float* o = K.cap + 4 * n;
        o[0] = cpx; o[1] = cpy; o[2] = cpz; o[3] = cs;
        *K.ncap = n + 1;
        return;
    }
    if (!(E > S.cut)) return;
    if (S.tally_only) {
        atomicAdd(&K.A->ctl->tally_count[sp], 1ull);
        atomicAdd(&K.A->ctl->tally_w[sp], double(L.w));
        atomicAdd(&K.A->ctl->tally_wE[sp], double(L.w) * double(E));
        if (S.hist_bins > 0 && K.A->hist_n[sp]) {
            int b = int(floorf((logf(E) - S.hist_lmin) * S.hist_linv));
            if (b >= 0 && b < S.hist_bins) {
                atomicAdd(&K.A->hist_n[sp][b], 1ull);
                atomicAdd(&K.A->hist_w[sp][b], double(L.w));
            }
        }
        return;
    }
    uint32_t a = ctr0, b = L.sid_lo, c = L.sid_hi, d = 1u;
    philox4x32_10(a, b, c, d, K.A->key0, K.A->key1);
    uint32_t slo = cidx ? c : a, shi = cidx ? d : b;
    if (K.H->nswarm > 0) shi = (shi & 0x00FFFFFFu) | (L.sid_hi & 0xFF000000u);  // inherit the swarm
    atomicAdd(&K.tal[T_SPAWN + sp], 1u);
    float4 e0 = make_float4(L.x, L.y, L.z, L.w);
    float4 e1 = make_float4(cpx, cpy, cpz, cs);
    uint4 e2 = make_uint4(slo, shi, uint32_t(sp) | (uint32_t(L.k) << 2), __float_as_uint(dd_val(L.th, L.tlo)));
    int pos = atomicAdd(K.top, 1);
    if (pos < kWarpStack) {
        K.stk[3 * pos + 0] = e0;
        K.stk[3 * pos + 1] = e1;
        K.stk[3 * pos + 2] = make_float4(__uint_as_float(e2.x), __uint_as_float(e2.y),
                                         __uint_as_float(e2.z), __uint_as_float(e2.w));
    } else {
        err(K, PCL_E_SPILL);
        unsigned long long q = atomicAdd(K.A->sp_out_n, 1ull);
        if ((long long)q < K.A->sp_cap) {
            K.A->sp_out_xw[q] = e0;
            K.A->sp_out_ps[q] = e1;
            K.A->sp_out_meta[q] = e2;
        } else {
            err(K, PCL_E_CAPACITY);
        }
    }
}

// ----------------------------------------------------------- samplers ----
// relativistic_coulomb.jl:10-51
__device__ void s_coulomb(Lane& L, const KCtx& K, const DevProc& P) {
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float p2 = L.px * L.px + L.py * L.py + L.pz * L.pz;
    float pn = sqrtf(p2);
    float b2 = p2 / (1.0f + p2);
    float al = P.p[0] / p2;
    float x = 0.0f;
    int it = 0;
    for (;;) {
        float u = U(L, K);
        x = al * u / (al + (1.0f - u));
        float z = U(L, K);
        if (z < 1.0f - b2 * x) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
    }
    float cth = 1.0f - 2.0f * x, sth = 2.0f * sqrtf(x * (1.0f - x));
    turn(L.px, L.py, L.pz, cth, sth, cph, sph, pn, L.px, L.py, L.pz);
    L.s = nextcoll(L, K);
}

// moller.jl:19-37: energies, Lehtinen angles, shared azimuth, secondary
__device__ __forceinline__ void moller_tail(Lane& L, const KCtx& K, float E, float eps, uint32_t ctr0) {
    float E2 = eps * E, E1 = E - E2;
    float p1 = sqrtf(E1 * (E1 + 2.0f)), p2 = sqrtf(E2 * (E2 + 2.0f));
    float c1, s1, cc2, s2;
    lehtinen(E, E1, E2, c1, s1);
    lehtinen(E, E2, E1, cc2, s2);
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float ax, ay, az, bx, by, bz;
    turn(L.px, L.py, L.pz, c1, s1, cph, sph, p1, ax, ay, az);
    turn(L.px, L.py, L.pz, cc2, s2, cph, -sph, p2, bx, by, bz);
    L.px = ax; L.py = ay; L.pz = az;
    L.s = nextcoll(L, K);
    float cs = nextcoll(L, K);
    emit(L, K, PCL_ELECTRON, bx, by, bz, cs, 0, ctr0);
}

// sample_secondary_energy(Moller) (moller.jl:64-87): eps by rejection
__device__ __forceinline__ float moller_eps(Lane& L, const KCtx& K, const DevProc& P, float E) {
    const float e0 = P.p[0] / E;
    const float g = 1.0f + E;
    const float nrm = 4.0f / (9.0f * g * g - 10.0f * g + 5.0f);
    const float c2 = 2.0f * g * g + 2.0f * g - 1.0f;
    const float g2 = g * g, em2 = E * E;
    float eps = 0.5f;
    int it = 0;
    for (;;) {
        float r = U(L, K);
        eps = e0 / (1.0f - r + 2.0f * e0 * r);
        float om = 1.0f - eps;
        float gg = nrm * (em2 * eps * eps - c2 * (eps / om) + g2 / (om * om));
        if (U(L, K) < gg) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
    }
    return eps;
}

// moller.jl:13-37, 64-87
__device__ void s_moller(Lane& L, const KCtx& K, const DevProc& P, float E, uint32_t ctr0) {
    moller_tail(L, K, E, moller_eps(L, K, P, E), ctr0);
}

// rbeb.jl:54-80, 156-196
__device__ PCL_RARE void s_rbeb(Lane& L, const KCtx& K, const DevProc& P, float E, uint32_t ctr0) {
    const float B = P.p[0];
    if (!(E > B)) {  // below threshold: the reference asserts; count it and treat as null
        err(K, PCL_E_KINEMATICS);
        L.s = nextcoll(L, K);
        return;
    }
    const float t1 = E, b1 = B;
    const float op = 1.0f + t1;
    const float bt2 = t1 * (t1 + 2.0f) / (op * op);
    const float t = E / B;
    const float A = -(1.0f + 2.0f * t1) / (t + 1.0f) / (op * op);
    const float C = logf(t1 * (t1 + 2.0f)) - bt2 - logf(2.0f * b1);
    const float M = b1 * b1 / (op * op);
    const float tm1 = t - 1.0f, tp1 = t + 1.0f;
    const float pbn = 2.0f + 2.0f * C + tp1 * tp1 * M / 4.0f;
    float w = 0.0f;
    int it = 0;
    for (;;) {
        float u = U(L, K);
        // w = u / (ratio - u) with ratio = (t + 1) / (t - 1) (rbeb.jl:175), in
        // the form u (t - 1) / (t (1 - u) + 1 + u): for t = E / B in the
        // millions ratio - u cancels to a few FP32 ulps, and 1 - u is exact
        w = u * tm1 / (t * (1.0f - u) + (1.0f + u));
        float a1 = 1.0f / (w + 1.0f), a2 = 1.0f / (t - w);
        float pb = pbn * a1 * a1;
        float p0 = A * (a1 + a2) + ((a1 * a1 + a2 * a2) + M) + C * (a1 * a1 * a1 + a2 * a2 * a2);
        if (U(L, K) * pb < p0) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
    }
    float E2 = B * w, E1 = E - E2 - B;
    if (!(E2 < E1)) err(K, PCL_E_KINEMATICS);
    float p1 = sqrtf(E1 * (E1 + 2.0f)), p2 = sqrtf(E2 * (E2 + 2.0f));
    float c1, s1, cc2, s2;
    lehtinen(E, E1, E2 + B, c1, s1);
    lehtinen(E, E2, E1 + B, cc2, s2);
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float ax, ay, az, bx, by, bz;
    turn(L.px, L.py, L.pz, c1, s1, cph, sph, p1, ax, ay, az);
    turn(L.px, L.py, L.pz, cc2, s2, cph, -sph, p2, bx, by, bz);
    L.px = ax; L.py = ay; L.pz = az;
    L.s = nextcoll(L, K);
    float cs = nextcoll(L, K);
    emit(L, K, PCL_ELECTRON, bx, by, bz, cs, 0, ctr0);
}

// seltzer.jl:74-90: photon direction (modified Tsai, util.jl:143-159), recoil, photon
__device__ __forceinline__ void sb_tail(Lane& L, const KCtx& K, float E, float k, uint32_t ctr0) {
    if (!(k < E)) err(K, PCL_E_KINEMATICS);
    float xt = tsai_x(L, K, E);
    float cth = 1.0f - 2.0f * xt, sth = 2.0f * sqrtf(xt * (1.0f - xt));
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float gx, gy, gz;
    turn(L.px, L.py, L.pz, cth, sth, cph, sph, k, gx, gy, gz);
    L.px -= gx; L.py -= gy; L.pz -= gz;
    L.s = nextcoll(L, K);
    float cs = nextcoll(L, K);
    emit(L, K, PCL_PHOTON, gx, gy, gz, cs, 0, ctr0);
}

// sample_secondary_energy(SeltzerBerger) (seltzer.jl:97-122): the photon
// energy k by the inverse-CDF lookup, which reproduces the reference's
// interpolation weights as written (seltzer.jl:114-118, off-diagonal corners
// included).
__device__ __forceinline__ float sb_k(Lane& L, const KCtx& K, const DevProc& P, float E) {
    const SBHdr& T = K.H->sb[P.sb];
    const float* data = K.A->sb_data[P.sb];
    uint32_t bits = next_bits(L, K.A->key0, K.A->key1);
    float x = bits_to_u(bits);
    // i1 = searchsortedfirst(pcum, x) - 1 = floor(x (ncum - 1)), exact in integers
    unsigned long long prod = (((unsigned long long)(bits >> 9) << 1) | 1ull) * (unsigned long long)(T.ncum - 1);
    int i1 = int(prod >> 24);
    if (i1 > T.ncum - 2) i1 = T.ncum - 2;
    int i2 = i1 + 1;
    float xa = float(i1) / T.inv_dp, xb = float(i2) / T.inv_dp;
    float y = logf(E);
    const float* le = K.blob + T.le_off;
    // j2 = searchsortedfirst(log_energy, y)
    int lo = 0, hi = T.ne;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (le[mid] < y) lo = mid + 1; else hi = mid; }
    int j1 = lo - 1;
    if (j1 < 0) { j1 = 0; err(K, PCL_E_TABLE_RANGE); }
    if (j1 > T.ne - 2) { j1 = T.ne - 2; err(K, PCL_E_TABLE_RANGE); }
    int j2 = j1 + 1;
    float y1 = le[j1], y2 = le[j2];
    const float* d1 = data + (size_t)j1 * T.ncum;
    const float* d2 = data + (size_t)j2 * T.ncum;
    float u11 = __ldg(d1 + i1), u21 = __ldg(d1 + i2), u12 = __ldg(d2 + i1), u22 = __ldg(d2 + i2);
    float A = (xb - xa) * (y2 - y1);
    float S = u11 * (xb - x) * (y2 - y) + u12 * (x - xa) * (y2 - y) + u21 * (xb - x) * (y - y1) +
              u22 * (x - xa) * (y - y1);
    return E * expf(S / A);
}

// seltzer.jl:67-90: the photon energy, then its angle (util.jl:143-159)
__device__ PCL_RARE void s_sb(Lane& L, const KCtx& K, const DevProc& P, float E, uint32_t ctr0) {
    sb_tail(L, K, E, sb_k(L, K, P, E), ctr0);
}

// compton.jl:9-28, 119-144 (Compton and KleinNishinaCompton share the sampler)
// 1 - eps is carried explicitly (-expm1 in the first branch,
// (1 - e0^2)(1 - U)/(1 + eps) in the second): eps -> 1 for low-energy photons
// and the direct difference would lose most of its FP32 bits.
__device__ PCL_RARE void s_compton(Lane& L, const KCtx& K, float E, uint32_t ctr0) {
    const float e0 = 1.0f / (1.0f + 2.0f * E);
    const float a1 = log1pf(2.0f * E);
    const float ome0sq = (2.0f * E * e0) * (1.0f + e0);   // 1 - e0^2
    const float a2 = ome0sq * 0.5f;
    const float pa = a1 / (a1 + a2);
    float eps = 1.0f, t = 0.0f;
    int it = 0;
    for (;;) {
        float om;
        if (U(L, K) < pa) {
            float q = -U(L, K) * a1;
            eps = expf(q);
            om = -expm1f(q);
        } else {
            float u = U(L, K);
            eps = sqrtf(e0 * e0 + ome0sq * u);
            om = ome0sq * (1.0f - u) / (1.0f + eps);
        }
        t = om / (eps * E);
        float g = 1.0f - eps / (1.0f + eps * eps) * t * (2.0f - t);
        if (U(L, K) < g) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
    }
    float cth = 1.0f - t, sth = sqrtf(fmaxf(0.0f, t * (2.0f - t)));
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float gx, gy, gz;
    turn(L.px, L.py, L.pz, cth, sth, cph, sph, eps * E, gx, gy, gz);
    float ex = L.px - gx, ey = L.py - gy, ez = L.pz - gz;
    L.px = gx; L.py = gy; L.pz = gz;
    L.s = nextcoll(L, K);
    float cs = nextcoll(L, K);
    emit(L, K, PCL_ELECTRON, ex, ey, ez, cs, 0, ctr0);
}

// photo_electric.jl:38-52, 60-99
__device__ PCL_RARE void s_photoelectric(Lane& L, const KCtx& K, const DevProc& P, float E, uint32_t ctr0) {
    float b = P.p[0];
    for (int m = 0; m < P.nbind; ++m) { b = P.p[m]; if (E > b) break; }
    if (!(E > b)) err(K, PCL_E_KINEMATICS);
    float Ee = E - b;
    float g = 1.0f + Ee;
    float beta = sqrtf(Ee * (Ee + 2.0f)) / g;
    float A = 1.0f / beta - 1.0f;
    float k2 = beta * g * Ee * (Ee - 1.0f) * 0.5f;   // beta gamma (gamma-1)(gamma-2) / 2
    float g0 = 2.0f * (1.0f / A + k2);
    float nu = 0.0f;
    int it = 0;
    for (;;) {
        float xi = U(L, K);
        nu = 2.0f * A / ((A + 2.0f) * (A + 2.0f) - 4.0f * xi) * (2.0f * xi + (A + 2.0f) * sqrtf(xi));
        float xi1 = U(L, K);
        float gn = (2.0f - nu) * (1.0f / (A + nu) + k2);
        if (xi1 * g0 < gn) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
    }
    float cth = 1.0f - nu, sth = sqrtf(fmaxf(0.0f, nu * (2.0f - nu)));
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float ex, ey, ez;
    turn(L.px, L.py, L.pz, cth, sth, cph, sph, sqrtf(Ee * (Ee + 2.0f)), ex, ey, ez);
    float cs = nextcoll(L, K);
    L.alive = false;
    emit(L, K, PCL_ELECTRON, ex, ey, ez, cs, 0, ctr0);
}

// _screen_function1/2 (bethe_heitler.jl:163-193)
__device__ __forceinline__ float screen1(float d) {
    return d > 1.4f ? 42.038f - 8.29f * logf(d + 0.958f) : 42.184f - d * (7.444f - 1.623f * d);
}
__device__ __forceinline__ float screen2(float d) {
    return d > 1.4f ? 42.038f - 8.29f * logf(d + 0.958f) : 41.326f - d * (5.848f - 0.902f * d);
}

// bethe_heitler.jl:5-25, 85-146
__device__ PCL_RARE void s_bethe_heitler(Lane& L, const KCtx& K, const DevProc& P, float E, uint32_t ctr0) {
    const float e0 = 1.0f / E;
    if (!(e0 < 0.5f)) err(K, PCL_E_KINEMATICS);
    float eps;
    if (E < P.p[4]) {  // 2 MeV
        eps = e0 + (0.5f - e0) * U(L, K);
    } else {
        const float d0 = 136.0f * e0 / P.p[1];
        const float FZ = (E > P.p[5]) ? P.p[3] : P.p[2];  // 50 MeV
        const float dmin = 4.0f * d0;
        const float dmax = expf((42.24f - FZ) / 8.368f) - 0.952f;
        const float ep = (1.0f - sqrtf(1.0f - dmin / dmax)) * 0.5f;
        const float emin = fmaxf(e0, ep);
        const float er = 0.5f - emin;
        const float F10 = screen1(dmin) - FZ, F20 = screen2(dmin) - FZ;
        const float NF1 = fmaxf(F10 * er * er, 0.0f), NF2 = fmaxf(1.5f * F20, 0.0f);
        const float NC = NF1 / (NF1 + NF2);
        int it = 0;
        for (;;) {
            bool acc;
            if (NC > U(L, K)) {
                eps = 0.5f - er * cbrtf(U(L, K));
                float d = d0 / (eps * (1.0f - eps));
                acc = U(L, K) < (screen1(d) - FZ) / F10;
            } else {
                eps = emin + er * U(L, K);
                float d = d0 / (eps * (1.0f - eps));
                acc = U(L, K) < (screen2(d) - FZ) / F20;
            }
            if (acc) break;
            if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
        }
    }
    float etot, ptot;
    if (U(L, K) < 0.5f) { etot = (1.0f - eps) * E; ptot = eps * E; }   // rand(Bool)
    else { ptot = (1.0f - eps) * E; etot = eps * E; }
    // the sampler returns (ekin, pkin); collide binds them as (pkin, ekin)
    const float first = fmaxf(0.0f, etot - 1.0f), second = fmaxf(0.0f, ptot - 1.0f);
    const float ekin_c = second, pkin_c = first;
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float xe = tsai_x(L, K, ekin_c);
    float ex, ey, ez;
    turn(L.px, L.py, L.pz, 1.0f - 2.0f * xe, 2.0f * sqrtf(xe * (1.0f - xe)), cph, sph,
         sqrtf(ekin_c * (ekin_c + 2.0f)), ex, ey, ez);
    float xp = tsai_x(L, K, pkin_c);
    float qx, qy, qz;
    turn(L.px, L.py, L.pz, 1.0f - 2.0f * xp, 2.0f * sqrtf(xp * (1.0f - xp)), cph, sph,
         sqrtf(pkin_c * (pkin_c + 2.0f)), qx, qy, qz);
    float se = nextcoll(L, K);
    float sp = nextcoll(L, K);
    L.alive = false;
    emit(L, K, PCL_ELECTRON, ex, ey, ez, se, 0, ctr0);
    emit(L, K, PCL_POSITRON, qx, qy, qz, sp, 1, ctr0);
}

// bhaba.jl:9-33, 55-91
__device__ PCL_RARE void s_bhabha(Lane& L, const KCtx& K, const DevProc& P, float E, uint32_t ctr0) {
    const float e0 = P.p[0] / E;
    const float g = 1.0f + E;
    const float y = 1.0f / (g + 1.0f);
    const float B0 = g * g / (E * (E + 2.0f));
    const float uu = 1.0f - 2.0f * y;
    const float B1 = 2.0f - y * y, B2 = uu * (3.0f + y * y), B3 = uu * uu + uu * uu * uu,
                B4 = uu * uu * uu;
    const float g2 = B0 + B1 * e0 + B2 * e0 * e0 + B3 * e0 * e0 * e0 + B4 * e0 * e0 * e0 * e0;
    float eps = e0;
    int it = 0;
    for (;;) {
        float r = U(L, K);
        eps = e0 / (1.0f - r + e0 * r);
        float g1 = B0 + B1 * eps + B2 * eps * eps + B3 * eps * eps * eps + B4 * eps * eps * eps * eps;
        if (U(L, K) < g1 / g2) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
    }
    float E2 = eps * E, E1 = E - E2;
    float p1 = sqrtf(E1 * (E1 + 2.0f)), p2 = sqrtf(E2 * (E2 + 2.0f));
    float c1, s1, cc2, s2;
    lehtinen(E, E1, E2, c1, s1);
    lehtinen(E, E2, E1, cc2, s2);
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float ax, ay, az, bx, by, bz;
    turn(L.px, L.py, L.pz, c1, s1, cph, sph, p1, ax, ay, az);
    turn(L.px, L.py, L.pz, cc2, s2, cph, -sph, p2, bx, by, bz);
    L.px = ax; L.py = ay; L.pz = az;
    L.s = nextcoll(L, K);
    float cs = nextcoll(L, K);
    emit(L, K, PCL_ELECTRON, bx, by, bz, cs, 0, ctr0);
}

// anihilation.jl:6-23, 39-67
__device__ PCL_RARE void s_annihilation(Lane& L, const KCtx& K, float E, uint32_t ctr0) {
    // Exact rewrites for FP32: eps_min = (1 - q)/2 = 1/((E + 2)(1 + q)) (1 - q
    // cancels at high E), eps = eps_min exp(U ln(eps_max/eps_min)) with
    // eps - eps_min = eps_min expm1(U L) and eps_max - eps = -eps_max expm1((U - 1) L),
    // so sin^2 = 2 (E + 2)(eps_max - eps)(eps - eps_min) / (eps^2 P^2) has no cancellation.
    const float g = 1.0f + E;
    const float Ep2 = E + 2.0f;
    const float q = sqrtf(E / Ep2);
    const float emin = 1.0f / (Ep2 * (1.0f + q));
    const float emax = 0.5f * (1.0f + q);
    const float Lr = logf(emax / emin);
    float eps = 0.5f, u = 0.5f, ex = 0.0f;
    int it = 0;
    for (;;) {
        u = U(L, K);
        ex = expm1f(u * Lr);
        eps = emin + emin * ex;                       // eps_min (eps_max/eps_min)^U
        float gg = 1.0f - eps + (2.0f * g * eps - 1.0f) / (eps * (g + 1.0f) * (g + 1.0f));
        if (U(L, K) < gg) break;
        if (++it >= kRejectCap) { err(K, PCL_E_REJECT_CAP); break; }
    }
    const float lo = emin * ex;                       // eps - eps_min
    const float hi = -emax * expm1f((u - 1.0f) * Lr); // eps_max - eps
    const float iP = rsqrtf(E * Ep2);                 // 1 / sqrt(gamma^2 - 1)
    float cth = (eps * Ep2 - 1.0f) * iP / eps;
    float sth = sqrtf(fmaxf(0.0f, 2.0f * Ep2 * lo * hi)) * iP / eps;
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float ax, ay, az;
    turn(L.px, L.py, L.pz, cth, sth, cph, sph, eps * (E + 2.0f), ax, ay, az);
    float bx = L.px - ax, by = L.py - ay, bz = L.pz - az;
    float sa = nextcoll(L, K);
    float sb = nextcoll(L, K);
    L.alive = false;
    emit(L, K, PCL_PHOTON, ax, ay, az, sa, 0, ctr0);
    emit(L, K, PCL_PHOTON, bx, by, bz, sb, 1, ctr0);
}


// randsphere() (util.jl:4-12): phi = 2 pi rand(), u = 2 rand() - 1
__device__ __forceinline__ void randsphere(Lane& L, const KCtx& K, float& x, float& y, float& z) {
    float sph, cph;
    sincos_2pi(U(L, K), sph, cph);
    float u = 2.0f * U(L, K) - 1.0f;
    float v = sqrtf(fmaxf(0.0f, (1.0f - u) * (1.0f + u)));
    x = v * cph; y = v * sph; z = u;
}

// collide(::Elastic, ...) (slow-electron.jl:133-139) on the momentum:
// p_cm = m/(1+m) p, p' = randsphere() |p - p_cm| + p_cm
__device__ PCL_RARE void s_elastic(Lane& L, const KCtx& K, const DevProc& P) {
    const float f = P.p[0] / (1.0f + P.p[0]);
    float cx = f * L.px, cy = f * L.py, cz = f * L.pz;
    float dx = L.px - cx, dy = L.py - cy, dz = L.pz - cz;
    float dn = sqrtf(dx * dx + dy * dy + dz * dz);
    float ux, uy, uz;
    randsphere(L, K, ux, uy, uz);
    L.px = ux * dn + cx; L.py = uy * dn + cy; L.pz = uz * dn + cz;
    L.s = nextcoll(L, K);
}

// collide(::Excitation, ...) (slow-electron.jl:108-114): E1 = max(0, E - threshold),
// isotropic direction
__device__ PCL_RARE void s_excitation(Lane& L, const KCtx& K, const DevProc& P, float E) {
    float E1 = fmaxf(0.0f, E - P.p[0]);
    float pn = sqrtf(E1 * (E1 + 2.0f));
    float ux, uy, uz;
    randsphere(L, K, ux, uy, uz);
    L.px = ux * pn; L.py = uy * pn; L.pz = uz * pn;
    L.s = nextcoll(L, K);
}

// collide(::Ionization, ...) (slow-electron.jl:117-127): the primary and a new
// electron share E - threshold equally, each isotropic; draws: both
// directions, then the primary's s (its state constructor) and the new one's.
__device__ PCL_RARE void s_ionization(Lane& L, const KCtx& K, const DevProc& P, float E, uint32_t ctr0) {
    const float E1 = 0.5f * fmaxf(0.0f, E - P.p[0]);
    const float pn = sqrtf(E1 * (E1 + 2.0f));
    float ux, uy, uz, vx, vy, vz;
    randsphere(L, K, ux, uy, uz);
    randsphere(L, K, vx, vy, vz);
    L.px = ux * pn; L.py = uy * pn; L.pz = uz * pn;
    L.s = nextcoll(L, K);
    const float cs = nextcoll(L, K);
    emit(L, K, PCL_ELECTRON, vx * pn, vy * pn, vz * pn, cs, 0, ctr0);
}

// Dispatch one real collision with table position j; updates the primary
// (state change + setr!) or removes it, and emits secondaries (apply!,
// collisions.jl:83-133).
__device__ void sample_process(Lane& L, const KCtx& K, const SpeciesHdr& S, const DevProc& P, float E,
                               uint32_t ctr0) {
    switch (P.kind) {
        case PCL_PROC_REL_COULOMB: s_coulomb(L, K, P); break;
        case PCL_PROC_MOLLER: s_moller(L, K, P, E, ctr0); break;
        case PCL_PROC_RBEB: s_rbeb(L, K, P, E, ctr0); break;
        case PCL_PROC_SELTZER_BERGER: s_sb(L, K, P, E, ctr0); break;
        case PCL_PROC_COMPTON:
        case PCL_PROC_KN_COMPTON: s_compton(L, K, E, ctr0); break;
        case PCL_PROC_PHOTOELECTRIC: s_photoelectric(L, K, P, E, ctr0); break;
        case PCL_PROC_BETHE_HEITLER: s_bethe_heitler(L, K, P, E, ctr0); break;
        case PCL_PROC_BHABHA: s_bhabha(L, K, P, E, ctr0); break;
        case PCL_PROC_ANNIHILATION: s_annihilation(L, K, E, ctr0); break;
        case PCL_PROC_ELASTIC: s_elastic(L, K, P); break;
        case PCL_PROC_EXCITATION: s_excitation(L, K, P, E); break;
        case PCL_PROC_IONIZATION: s_ionization(L, K, P, E, ctr0); break;
        case PCL_PROC_ATTACHMENT: L.alive = false; break;   // RemoveParticleOutcome
        case PCL_PROC_NULL_COLLISION: L.s = nextcoll(L, K); break;  // NullOutcome (collisions.jl:83-88)
        default: err(K, PCL_E_KINEMATICS); break;
    }
    if (L.alive) L.r = setr(S, K, kin_energy_exact(L.species, L.px, L.py, L.pz), L.sw);
}

// ------------------------------------------------------- learned sampler -
// Network input a = (log10(T / eV) - 6) / 2; the network is used where its
// 64-bin map over a in [-1, 1) is set (trained range, monotone in u) and, for
// Moller, where the kinematic range is not degenerate (e0 = tcut / T < 0.45).
__device__ __forceinline__ float learn_a(float E) {
    return (log10f(E * 510998.95f) - 6.0f) * 0.5f;
}

__device__ __forceinline__ bool learned_here(const DevProc& P, float E) {
    float a = learn_a(E);
    if (!(a >= -1.0f && a < 1.0f)) return false;
    int bin = min(int((a + 1.0f) * 32.0f), 63);
    if (!((P.learn_ok[bin >> 5] >> (bin & 31)) & 1u)) return false;
    if (P.learn == PCL_LEARN_MOLLER && !(P.p[0] < 0.45f * E)) return false;
    return true;
}

// Suspend the collision: one uniform is drawn for the network, the particle
// goes to the suspended-collision queue and leaves this pass (its input slot,
// if any, is marked dead; the resume pass appends it).  False when the queue is
// full (the table sampler then runs instead).
__device__ bool suspend(Lane& L, const KCtx& K, int j, uint32_t ctr0) {
    const float u = U(L, K);
    const StepArgs& A = *K.A;
    unsigned long long q = atomicAdd(A.lq_out_n, 1ull);
    if ((long long)q >= A.lq_cap) return false;
    A.lq_out_xw[q] = make_float4(L.x, L.y, L.z, L.w);
    A.lq_out_ps[q] = make_float4(L.px, L.py, L.pz, L.s);
    A.lq_out_m1[q] = make_uint4(L.sid_lo, L.sid_hi, L.ctr, ctr0);
    uint32_t pk = uint32_t(L.species) | (uint32_t(L.k) << 2) | (uint32_t(j) << 8) |
                  (uint32_t(min(L.nsub, 0xFFFF)) << 16);
    A.lq_out_m2[q] = make_float4(L.th, L.tlo, u, __uint_as_float(pk));
    L.alive = false;
    return true;
}

// Lower bound of ln(k / T) of a Seltzer-Berger table at energy E: its
// pcum = 0 column, linear in ln T between grid energies, lowered by the
// column's largest step between grid energies (the table sampler's bilinear
// weights can reach the lower corner of either bracketing energy).  The
// bremsstrahlung network's output h = 1 - ln(k / T) / ymin lies in [0, 1].
__device__ __forceinline__ float sb_ymin(const KCtx& K, const DevProc& P, float E) {
    const SBHdr& T = K.H->sb[P.sb];
    const float* data = K.A->sb_data[P.sb];
    const float* le = K.blob + T.le_off;
    const float y = logf(E);
    int lo = 0, hi = T.ne;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (le[mid] < y) lo = mid + 1; else hi = mid; }
    const int j1 = min(max(lo - 1, 0), T.ne - 2), j2 = j1 + 1;
    const float w = fminf(fmaxf((y - le[j1]) / (le[j2] - le[j1]), 0.0f), 1.0f);
    return (1.0f - w) * __ldg(data + (size_t)j1 * T.ncum) + w * __ldg(data + (size_t)j2 * T.ncum) - T.ymargin;
}

// Finish a suspended collision with the network output y (the part of the
// sampler after its energy draw), then setr! as after every collision.
__device__ void learned_outcome(Lane& L, const KCtx& K, const SpeciesHdr& S, const DevProc& P, float E, float y,
                                uint32_t ctr0) {
    if (P.learn == PCL_LEARN_SB) {
        const float h = fminf(fmaxf(y, 0.0f), 1.0f);
        // k < T strictly (seltzer.jl:73)
        sb_tail(L, K, E, E * expf(fminf((1.0f - h) * sb_ymin(K, P, E), -1e-6f)), ctr0);
    } else {
        const float e0 = P.p[0] / E;
        const float v = fminf(fmaxf(y, 0.0f), 1.0f);
        moller_tail(L, K, E, e0 / (1.0f - v * (1.0f - 2.0f * e0)), ctr0);
    }
    if (L.alive) L.r = setr(S, K, kin_energy_exact(L.species, L.px, L.py, L.pz), L.sw);
}

// Event kernel: a lane's whole state as 5 x 16 B (the collision stash).  The
// Philox cache keeps at most three unconsumed words (c0..c2).
__device__ __forceinline__ void park_lane(const Lane& L, float4* e) {
    const uint32_t pk = uint32_t(L.species) | (uint32_t(L.k) << 2) | (uint32_t(L.sw) << 8) |
                        (L.rvalid ? (1u << 16) : 0u);
    e[0] = make_float4(L.x, L.y, L.z, L.w);
    e[1] = make_float4(L.px, L.py, L.pz, L.s);
    e[2] = make_float4(L.th, L.tlo, L.r, __uint_as_float(L.sid_lo));
    e[3] = make_float4(__uint_as_float(L.sid_hi), __uint_as_float(L.ctr), __uint_as_float(L.c0),
                       __uint_as_float(L.c1));
    e[4] = make_float4(__uint_as_float(L.c2), __uint_as_float(pk), __int_as_float(L.slot), __int_as_float(L.nsub));
}

__device__ __forceinline__ void unpark_lane(Lane& L, const float4* e) {
    const float4 a = e[0], b = e[1], c = e[2], d = e[3], f = e[4];
    L.x = a.x; L.y = a.y; L.z = a.z; L.w = a.w;
    L.px = b.x; L.py = b.y; L.pz = b.z; L.s = b.w;
    L.th = c.x; L.tlo = c.y; L.r = c.z; L.sid_lo = __float_as_uint(c.w);
    L.sid_hi = __float_as_uint(d.x); L.ctr = __float_as_uint(d.y); L.c0 = __float_as_uint(d.z);
    L.c1 = __float_as_uint(d.w);
    L.c2 = __float_as_uint(f.x);
    const uint32_t pk = __float_as_uint(f.y);
    L.species = int(pk & 3u); L.k = int((pk >> 2) & 63u); L.sw = int((pk >> 8) & 255u);
    L.rvalid = ((pk >> 16) & 1u) != 0u;
    L.slot = __float_as_int(f.z); L.nsub = __float_as_int(f.w);
    L.alive = true;
}

// do_one_collision! (collisions.jl:142-199).  LEARN: the learned samplers may
// take the collision (general step kernel only).
template <bool LEARN>
__device__ void collide(Lane& L, const KCtx& K, const SpeciesHdr& S) {
    if (L.r == 0.0f) return;
    float E = kin_energy_exact(L.species, L.px, L.py, L.pz);
    if (!(E >= S.cut)) return;
    const uint32_t ctr0 = L.ctr;
    int j = 0;
    if (S.table_kind == 1) {  // rate(::CollisionTable, j, pre) (collision_table.jl:53-57)
        float w;
        int i = lin_index(S, K, E, w);
        float xi = U(L, K) * L.r;
        const float* a = K.blob + S.rate_off + i * S.nproc;
        for (; j < S.nproc; ++j) {
            float nu = w * a[j] + (1.0f - w) * a[j + S.nproc];
            if (nu > xi) break;
            xi -= nu;
        }
    } else {
        float t[4];
        bool oor = false;
        int i = precheb(E, S.k, S.xscale, t, oor);
        if (oor) err(K, PCL_E_TABLE_RANGE);
        float xi = U(L, K) * L.r;
        const float* a = K.blob + S.rate_off + i * S.nproc * S.order;
        for (; j < S.nproc; ++j) {
            float nu = cheb_dot(a + j * S.order, t, S.order);
            if (nu > xi) break;
            xi -= nu;
        }
        if (j < S.nproc && S.proc[j].kind == PCL_PROC_REL_COULOMB && !(LEARN && S.proc[j].learn)) {
            // elastic: |p| and so E are unchanged, and setr! (collisions.jl:63-74)
            // evaluates the rate bound on the interval and basis already at hand
            atomicAdd(&K.tal[T_COLL + 16 * L.species + j], 1u);
            s_coulomb(L, K, S.proc[j]);
            float rb = cheb_dot(K.blob + S.rb_off + i * S.order, t, S.order);
            if (S.rbB_off >= 0) rb += K.blob[K.H->swarm_off + 4 * L.sw + 3] * cheb_dot(K.blob + S.rbB_off + i * S.order, t, S.order);
            if (!(rb > 0.0f)) {
                if (S.nproc > 0) err(K, PCL_E_NEG_RATE);
                rb = 0.0f;
            }
            L.r = rb;
            return;
        }
    }
    if (j == S.nproc) {  // NullOutcome (collisions.jl:83-88)
        atomicAdd(&K.tal[T_NULL + L.species], 1u);
        L.r = setr(S, K, E, L.sw);
        L.s = nextcoll(L, K);
        return;
    }
    atomicAdd(&K.tal[T_COLL + 16 * L.species + j], 1u);
    const DevProc& P = S.proc[j];
    if (LEARN && P.learn && K.A->lq_out_n && learned_here(P, E) && suspend(L, K, j, ctr0)) return;
    sample_process(L, K, S, P, E, ctr0);
}

// ---------------------------------------------------------- TMA staging --
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Wait for phase `parity` of the mbarrier at shared address `bar`, at most
// `max_iters` polls (each a try_wait plus a short sleep); false on timeout.
// Every mbarrier wait of the step kernels goes through here.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, int max_iters) {
    uint32_t done = 0;
    for (int it = 0; it < max_iters && !done; ++it) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (!done) __nanosleep(64);
    }
    return done != 0;
}

// Copy the table blob into shared memory with one bulk asynchronous copy
// (cp.async.bulk, completion on an mbarrier).  Bounded wait; false on timeout.
__device__ bool stage_blob(void* dst, const void* src, int bytes, unsigned long long* mbar) {
    uint32_t bar = smem_u32(mbar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(dst)),
            "l"(src), "r"(bytes), "r"(bar)
            : "memory");
    }
    return mbar_wait_bounded(bar, 0u, 1 << 22);
}

// Test hook of the bounded wait: every thread waits on an mbarrier that no
// thread and no copy ever arrives on, with a limit of `max_iters` polls, and
// the timeout is recorded in the control block as a staging timeout would be.
__global__ void k_test_wait(Control* ctl, int max_iters) {
    __shared__ unsigned long long bar;
    const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(&bar));
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(b), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(b, 0u, max_iters);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(&ctl->timeout, 1);
}

// Load particle data of an input slot.
__device__ __forceinline__ void load_slot(Lane& L, const float4* xw, const float4* ps, const uint4* meta,
                                          long long slot) {
    float4 a = xw[slot];
    float4 b = ps[slot];
    uint4 m = meta[slot];
    L.x = a.x; L.y = a.y; L.z = a.z; L.w = a.w;
    L.px = b.x; L.py = b.y; L.pz = b.z; L.s = b.w;
    L.sid_lo = m.x; L.sid_hi = m.y; L.ctr = m.z;
    L.th = -__uint_as_float(m.w);  // + dt by the caller (t_off <= 0 is time still owed)
    L.tlo = 0.0f;
}

// A slot of the population written at the end of a particle's launch, and in
// host-direct mode the same slot of the caller's host arrays.
__device__ __forceinline__ void put_slot(const StepArgs& A, int sp, long long slot, float4 a, float4 b, uint4 m) {
    A.xw[sp][slot] = a;
    A.ps[sp][slot] = b;
    A.meta[sp][slot] = m;
    if (A.hx_xw[sp] && slot < A.hx_cap[sp]) {
        A.hx_xw[sp][slot] = a;
        A.hx_ps[sp][slot] = b;
        A.hx_meta[sp][slot] = m;
    }
}

// ------------------------------------------------------------ the step ---
// EVENT: colliding particles are parked in a per-warp stash and collided in
// batches (the warp's free lanes, or, in MULTI, all 32 lanes with the lanes'
// other particles held in the stash meanwhile; see the loop), instead of each
// lane colliding as soon as its push ends; each particle's sequence of
// operations is unchanged.  MULTI: the instance for launches of several steps
// (the hold, guided chunks per species range, photon flights over whole steps).
template <int MINB, bool GENERAL, bool EVENT, bool LEARN, bool MULTI>
__global__ void __launch_bounds__(256, MINB) k_step(StepArgs A) {
    // a queue pass over an empty queue has nothing to stage, run or tally
    if (A.spill_mode == 1 && *A.sp_in_n == 0) return;
    if (LEARN && A.spill_mode == 2 && *A.lq_in_n == 0) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int nwarps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const unsigned lt = (1u << lane) - 1u;

    const BlobHdr* H = reinterpret_cast<const BlobHdr*>(smem);
    float4* stk_all = reinterpret_cast<float4*>(smem + A.blob_bytes);
    int* tops = reinterpret_cast<int*>(stk_all + size_t(nwarps) * kWarpStack * 3);
    uint32_t* tal = reinterpret_cast<uint32_t*>(tops + nwarps);
    unsigned long long* mbar =
        reinterpret_cast<unsigned long long*>(reinterpret_cast<uintptr_t>(tal + T_WORDS + 8) & ~uintptr_t(7));
    // event kernel: collision stash after the mbarrier (16-B aligned), counters after it
    // (parked collisions, then held particles, one of each per warp)
    float4* cs_all = reinterpret_cast<float4*>((reinterpret_cast<uintptr_t>(mbar + 1) + 15) & ~uintptr_t(15));
    int* cs_ns = reinterpret_cast<int*>(cs_all + size_t(nwarps) * kCollStash * 5);
    float4* cs = cs_all + size_t(warp) * kCollStash * 5;
    int* cs_n = cs_ns + warp;
    int* hd_n = cs_ns + nwarps + warp;

    for (int i = threadIdx.x; i < T_WORDS; i += blockDim.x) tal[i] = 0u;
    if (lane == 0) tops[warp] = 0;
    if (EVENT && lane == 0) { *cs_n = 0; *hd_n = 0; }
    bool ok = stage_blob(smem, A.blob, A.blob_bytes, mbar);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(&A.ctl->timeout, 1);
        return;
    }

    KCtx K;
    K.H = H;
    K.blob = reinterpret_cast<const float*>(smem);
    K.stk = stk_all + size_t(warp) * kWarpStack * 3;
    K.top = tops + warp;
    K.tal = tal;
    K.A = &A;
    K.cap = nullptr;
    K.ncap = nullptr;
    K.hasB = H->B[0] != 0.0f || H->B[1] != 0.0f || H->B[2] != 0.0f || H->bfield_kind != 0;
    // the multi-step instance without the learned samplers keeps a homogeneous
    // E field in registers (measured 5 % faster there; the one-step instance
    // ran slower with it, and the learned instance spilled)
    K.eregs = MULTI && !GENERAL && !LEARN && H->nswarm == 0;
    if (K.eregs) { K.E0 = H->E[0]; K.E1 = H->E[1]; K.E2 = H->E[2]; }

    Control* ctl = A.ctl;
    const float dt_hi = float(A.dt);
    const float dt_lo = float(A.dt - double(dt_hi));
    const int nsteps = A.nsteps;

    // work space: concatenated species ranges, or the spill queue
    long long nsp0, nsp1, total;
    if (LEARN && A.spill_mode == 2) {
        nsp0 = 0; nsp1 = 0;
        total = min((long long)(*A.lq_in_n), A.lq_cap);
    } else if (A.spill_mode) {
        nsp0 = 0; nsp1 = 0;
        total = min((long long)(*A.sp_in_n), A.sp_cap);
    } else {
        nsp0 = (long long)ctl->n_start[0];
        nsp1 = (long long)ctl->n_start[1];
        total = nsp0 + nsp1 + (long long)ctl->n_start[2];
    }
    long long g0 = 0;   // a population launch over part of the work: indices g0 + [0, total)
    if (!A.spill_mode && A.g_hi > 0) {
        g0 = min(A.g_lo, total);
        total = min(A.g_hi, total) - g0;
    }
    const long long nwarps_grid = (long long)gridDim.x * nwarps;

    long long cur = 0, end = 0;  // warp-private chunk (uniform)
    // small work (less than 32 slots per warp of the grid): only the first
    // warps of every block take input, so the particles spread over the SMs
    // instead of filling the first blocks to reach the work counter
    const long long per_block = (total + 32ll * gridDim.x - 1) / (32ll * gridDim.x);
    bool input_done = per_block < nwarps && warp >= max(per_block, 1ll);
    Lane L;
    L.slot = -1; L.alive = false; L.rvalid = false;
    bool has = false;
    bool pend = false;  // event kernel: a collision that found the stash full, collided next

    for (;;) {
        // ---------------- event kernel: collide parked particles in batches.
        // Mode 1: the free lanes, once the stash can fill all of them (in the
        // multi-step instance only when they are at least kBatchMin or the
        // input is taken), or when nothing else is left.  Mode 2 (multi-step
        // instance): all 32 lanes, once 32 collisions are parked; the lanes'
        // particles between collisions wait in the hold (the top of the
        // stash) and refill free lanes before children and input do.  Lanes
        // whose collision found the stash full collide here too, in their
        // lane, before any other push (one call site of the samplers).
        if (EVENT) {
            const unsigned empty = __ballot_sync(FULL, !has);
            const bool anyp = __any_sync(FULL, pend);
            __syncwarp();
            const int nstash = *cs_n;
            const int nh = MULTI ? *hd_n : 0;
            const int ne = __popc(empty);
            const bool drain = input_done && *K.top == 0;
            int mode = 0;
            if (!MULTI) {
                if (ne > 0 && nstash > 0 && (nstash >= ne || drain)) mode = 1;
            } else if (ne > 0 && nstash > 0 && ((nstash >= ne && (ne >= kBatchMin || input_done)) || drain)) {
                mode = 1;
            } else if (!anyp && nstash >= 32 && nstash + nh + (32 - ne) <= A.stash) {
                mode = 2;
            }
            if (mode || anyp) {
                int take = 0, rank = 0;
                if (!mode) {
                    // only the pending collisions
                } else if (MULTI && mode == 2) {
                    if (has) park_lane(L, cs + size_t(kCollStash - 1 - nh - __popc(~empty & lt)) * 5);
                    has = false;
                    take = 32;
                    rank = lane;
                } else {
                    take = min(ne, nstash);
                    rank = __popc(empty & lt);
                }
                bool doit = pend;
                if (!has && rank < take) {
                    unpark_lane(L, cs + size_t(nstash - 1 - rank) * 5);
                    has = true;
                    doit = true;
                }
                if (doit) {
                    pend = false;
                    collide<LEARN>(L, K, H->sp[L.species]);
                }
                __syncwarp();
                if (lane == 0 && mode) {
                    *cs_n = nstash - take;
                    if (MULTI && mode == 2) *hd_n = nh + (32 - ne);
                }
                __syncwarp();
            }
        }
        // ---------------- refill idle lanes: held particles, children, then input
        unsigned need = __ballot_sync(FULL, !has);
        if (need) {
            __syncwarp();
            if (EVENT && MULTI) {  // held particles first (the newest at the lowest index)
                const int nh = *hd_n;
                if (nh > 0) {
                    const int take = min(__popc(need), nh);
                    const int rank = __popc(need & lt);
                    if (!has && rank < take) {
                        unpark_lane(L, cs + size_t(kCollStash - nh + rank) * 5);
                        has = true;
                    }
                    __syncwarp();
                    if (lane == 0) *hd_n = nh - take;
                    __syncwarp();
                    need = __ballot_sync(FULL, !has);
                }
            }
            int top = *K.top;
            if (top > kWarpStack) top = kWarpStack;
            int take = min(__popc(need), top);
            int rank = __popc(need & lt);
            if (!has && rank < take) {
                int e = top - 1 - rank;
                float4 a = K.stk[3 * e + 0], b = K.stk[3 * e + 1], c = K.stk[3 * e + 2];
                L.x = a.x; L.y = a.y; L.z = a.z; L.w = a.w;
                L.px = b.x; L.py = b.y; L.pz = b.z; L.s = b.w;
                L.sid_lo = __float_as_uint(c.x); L.sid_hi = __float_as_uint(c.y);
                uint32_t sk = __float_as_uint(c.z);
                L.species = int(sk & 3u); L.k = int(sk >> 2);
                L.th = c.w; L.tlo = 0.0f;
                L.ctr = 0u; L.rvalid = false; L.slot = -1; L.alive = true; L.nsub = 0;
                L.sw = (H->nswarm > 0) ? min(int(L.sid_hi >> 24), H->nswarm - 1) : 0;
                L.r = setr(H->sp[L.species], K, kin_energy(L.species, L.px, L.py, L.pz), L.sw);
                has = true;
            }
            __syncwarp();
            if (lane == 0) *K.top = top - take;
            __syncwarp();
            need = __ballot_sync(FULL, !has);
            while (need && !input_done) {
                if (cur >= end) {
                    long long base = 0, len = 0;
                    if (lane == 0) {
                        // guided chunks over what is left of the work or, in a
                        // launch of several steps, of the current species' range
                        // (the species differ in cost per slot: a range's last
                        // chunks stay small whatever follows it)
                        long long done_est = (long long)(*(volatile unsigned long long*)A.head);
                        long long rend = total;
                        if (MULTI && done_est < nsp0 - g0) rend = min(total, nsp0 - g0);
                        else if (MULTI && done_est < nsp0 + nsp1 - g0) rend = min(total, nsp0 + nsp1 - g0);
                        long long rem = rend - done_est;
                        long long chunk = rem / (4 * nwarps_grid);
                        chunk = chunk < 32 ? 32 : (chunk > 1024 ? 1024 : chunk);
                        base = (long long)atomicAdd(A.head, (unsigned long long)chunk);
                        len = (base < total) ? min(chunk, total - base) : 0;
                    }
                    base = __shfl_sync(FULL, base, 0);
                    len = __shfl_sync(FULL, len, 0);
                    if (len <= 0) { input_done = true; break; }
                    cur = base; end = base + len;
                }
                int avail = int(min(end - cur, 32ll));
                int nn = __popc(need);
                int tk = min(avail, nn);
                int rk = __popc(need & lt);
                if (!has && rk < tk) {
                    long long v = g0 + cur + rk;
                    if (LEARN && A.spill_mode == 2) {
                        float4 a = A.lq_in_xw[v], b = A.lq_in_ps[v];
                        uint4 m1 = A.lq_in_m1[v];
                        float4 m2 = A.lq_in_m2[v];
                        const uint32_t pk = __float_as_uint(m2.w);
                        L.x = a.x; L.y = a.y; L.z = a.z; L.w = a.w;
                        L.px = b.x; L.py = b.y; L.pz = b.z; L.s = b.w;
                        L.sid_lo = m1.x; L.sid_hi = m1.y; L.ctr = m1.z;
                        L.species = int(pk & 3u); L.k = int((pk >> 2) & 63u); L.nsub = int(pk >> 16);
                        L.th = m2.x; L.tlo = m2.y;
                        L.slot = -1; L.alive = true; L.rvalid = false;
                        L.sw = (H->nswarm > 0) ? min(int(L.sid_hi >> 24), H->nswarm - 1) : 0;
                        const SpeciesHdr& S = H->sp[L.species];
                        const float E = kin_energy_exact(L.species, L.px, L.py, L.pz);
                        learned_outcome(L, K, S, S.proc[(pk >> 8) & 15u], E, A.lq_in_y[v], m1.w);
                        has = true;
                    } else if (A.spill_mode) {
                        float4 a = A.sp_in_xw[v], b = A.sp_in_ps[v];
                        uint4 m = A.sp_in_meta[v];
                        L.x = a.x; L.y = a.y; L.z = a.z; L.w = a.w;
                        L.px = b.x; L.py = b.y; L.pz = b.z; L.s = b.w;
                        L.sid_lo = m.x; L.sid_hi = m.y;
                        L.species = int(m.z & 3u); L.k = int(m.z >> 2);
                        L.th = __uint_as_float(m.w); L.tlo = 0.0f;
                        L.ctr = 0u; L.slot = -1;
                        has = true;
                    } else {
                        int sp; long long sl;
                        if (v < nsp0) { sp = 0; sl = v; }
                        else if (v < nsp0 + nsp1) { sp = 1; sl = v - nsp0; }
                        else { sp = 2; sl = v - nsp0 - nsp1; }
                        L.species = sp;
                        load_slot(L, A.in_xw[sp], A.in_ps[sp], A.in_meta[sp], sl);
                        dd_add(L.th, L.tlo, dt_hi, dt_lo);
                        L.slot = int(sl);
                        L.k = 0;
                        has = (L.ctr != PCL_DEAD_CTR);
                        // host-direct mode: a slot read dead from the host is dead in
                        // the device copy (which may hold an older particle there)
                        // and in the output arrays (which may differ from the input)
                        if (!has && A.hx_meta[sp]) {
                            A.meta[sp][sl].z = PCL_DEAD_CTR;
                            if (sl < A.hx_cap[sp]) A.hx_meta[sp][sl].z = PCL_DEAD_CTR;
                        }
                        if (has) atomicAdd(&tal[T_LSTART + 0], 1u);
                    }
                    if (has && !(LEARN && A.spill_mode == 2)) {
                        L.rvalid = false; L.alive = true; L.nsub = 0;
                        L.sw = (H->nswarm > 0) ? min(int(L.sid_hi >> 24), H->nswarm - 1) : 0;
                        L.r = setr(H->sp[L.species], K, kin_energy(L.species, L.px, L.py, L.pz), L.sw);
                    }
                }
                cur += tk;
                need = __ballot_sync(FULL, !has);
            }
        }
        if (__ballot_sync(FULL, has) == 0u) {
            // no work in this warp; the stack is empty because it is drained first
            if (input_done && (!EVENT || (*cs_n == 0 && (!MULTI || *hd_n == 0)))) break;
            continue;
        }

        // ---------------- one sub-step per busy lane, and the step boundary in the
        // same iteration when the sub-step used up the clock
        int fin = 0;  // 1: survives the launch, 2: removed
        bool park = false;
        if (has) {
            const SpeciesHdr& S = H->sp[L.species];
            bool boundary = true;
            if (L.alive && dd_val(L.th, L.tlo) > kEpsT && L.nsub < kSubstepCap) {
                float tnext = L.s / L.r;
                // trem > tnext with the low word (th - tnext is exact near the decision)
                bool coll = __fadd_rn(__fsub_rn(L.th, tnext), L.tlo) > 0.0f;
                float h = coll ? tnext : dd_val(L.th, L.tlo);
                if (!coll) L.s -= h * L.r;
                if (!GENERAL) push<false>(L, S, K, h);
                else push_general(L, S, K, h, dt_hi);
                if (coll) dd_add(L.th, L.tlo, -tnext, 0.0f);
                else { L.th = 0.0f; L.tlo = 0.0f; }
                L.nsub += 1;
                if (EVENT) park = coll && L.alive;
                else if (coll && L.alive) collide<LEARN>(L, K, S);
                // advance1!'s loop ends once the clock is spent (mixed_population.jl:66)
                boundary = !park && !(dd_val(L.th, L.tlo) > kEpsT);
            } else if (L.nsub >= kSubstepCap) {
                err(K, PCL_E_SUBSTEP_CAP);
                L.th = 0.0f; L.tlo = 0.0f;
            }
            if (park) {
                // collided later, in a batch
            } else if (!L.alive) {
                fin = 2;
            } else if (boundary) {
                float E = kin_energy(L.species, L.px, L.py, L.pz);
                if (E < S.cut) {  // droplow! (population.jl:273-284)
                    fin = 2;
                } else {
                    atomicAdd(&tal[T_LEND + 3 * L.k + L.species], 1u);
                    if (L.k + 1 >= nsteps) {
                        fin = 1;
                    } else {
                        L.k += 1;
                        L.nsub = 0;
                        dd_add(L.th, L.tlo, dt_hi, dt_lo);  // remainder below eps carries over (mixed_population.jl:65)
                        L.r = setr(S, K, E, L.sw);  // advance_init! of the next step
                        if (MULTI && L.species == PCL_PHOTON && (!GENERAL || (S.wall_coord < 0 && !S.frozen))) {
                            // A photon's collision-free whole steps in this
                            // iteration, each exactly as its own iteration would
                            // run it (the same clock decision, decrement, push and
                            // clock reset): no force acts on it and its energy, so
                            // its rate bound (setr!) and the droplow! outcome, do
                            // not change in flight, whatever the field.  The step
                            // that collides, the launch's last step, and every
                            // step of photons with a wall (whose crossings are
                            // recorded per sub-step) or not pushed at all are
                            // left to the loop.
                            const int k0 = L.k;
                            while (L.k + 1 < nsteps && dd_val(L.th, L.tlo) > kEpsT) {
                                const float tn = L.s / L.r;
                                if (__fadd_rn(__fsub_rn(L.th, tn), L.tlo) > 0.0f) break;
                                const float hh = dd_val(L.th, L.tlo);
                                L.s -= hh * L.r;
                                push<false>(L, S, K, hh);
                                L.th = 0.0f; L.tlo = 0.0f;
                                dd_add(L.th, L.tlo, dt_hi, dt_lo);
                                L.k += 1;
                            }
                            if (L.k > k0) {  // live at the end of steps k0 .. L.k - 1
                                atomicAdd(&tal[T_FLY + k0], 1u);
                                atomicAdd(&tal[T_FLY + L.k], 0xffffffffu);
                            }
                        }
                    }
                }
            }
        }

        if (EVENT) {
            // park the colliding particles; if the stash is full (its parked
            // collisions and held particles; possible with several steps per
            // launch, where lanes keep particles across steps) the rest stay
            // in their lanes and collide at the start of the next iteration.
            // A.stash entries are in use: parked collisions from the bottom,
            // held particles from the top of all kCollStash, and together at
            // most A.stash, so the two never meet
            const unsigned pm = __ballot_sync(FULL, park);
            if (pm) {
                __syncwarp();
                const int base = *cs_n;
                const int space = A.stash - base - (MULTI ? *hd_n : 0);
                const int rank = __popc(pm & lt);
                if (park) {
                    if (rank < space) {
                        park_lane(L, cs + size_t(base + rank) * 5);
                        has = false;
                    } else {
                        pend = true;
                    }
                }
                __syncwarp();
                if (lane == 0) *cs_n = base + min(__popc(pm), space);
                __syncwarp();
            }
        }

        // ---------------- finish: appended secondaries reserve slots per species
        unsigned am = __ballot_sync(FULL, fin == 1 && L.slot < 0);
        while (am) {
            int leader = __ffs(am) - 1;
            int lsp = __shfl_sync(FULL, L.species, leader);
            unsigned grp = __ballot_sync(FULL, fin == 1 && L.slot < 0 && L.species == lsp);
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&ctl->n[lsp], (unsigned long long)__popc(grp));
            base = __shfl_sync(FULL, base, leader);
            if (grp & (1u << lane)) {
                long long slot = (long long)base + __popc(grp & lt);
                if (slot < A.cap[lsp]) {
                    put_slot(A, lsp, slot, make_float4(L.x, L.y, L.z, L.w), make_float4(L.px, L.py, L.pz, L.s),
                             make_uint4(L.sid_lo, L.sid_hi, L.ctr, __float_as_uint(-dd_val(L.th, L.tlo))));
                } else {
                    err(K, PCL_E_CAPACITY);
                }
            }
            am &= ~grp;
        }
        if (fin == 1 && L.slot >= 0) {
            put_slot(A, L.species, L.slot, make_float4(L.x, L.y, L.z, L.w), make_float4(L.px, L.py, L.pz, L.s),
                     make_uint4(L.sid_lo, L.sid_hi, L.ctr, __float_as_uint(-dd_val(L.th, L.tlo))));
        } else if (fin == 2 && L.slot >= 0) {
            A.meta[L.species][L.slot].z = PCL_DEAD_CTR;
            if (A.hx_meta[L.species] && L.slot < A.hx_cap[L.species]) A.hx_meta[L.species][L.slot].z = PCL_DEAD_CTR;
            atomicAdd(&tal[T_DEAD + L.species], 1u);
        }
        if (fin) has = false;
    }

    // ---------------- flush block tallies
    __syncthreads();
    // photons flown through whole steps: T_FLY is a difference array over the
    // steps (+1 at the first step flown, -1 after the last; modulo 2^32)
    for (int j = threadIdx.x; j < nsteps - 1; j += blockDim.x) {
        uint32_t f = 0;
        for (int k = 0; k <= j; ++k) f += tal[T_FLY + k];
        tal[T_LEND + 3 * j + PCL_PHOTON] += f;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < T_WORDS; i += blockDim.x) {
        uint32_t v = tal[i];
        // the particles that start step k >= 1 of the launch are those that
        // ended step k - 1 (every boundary but the last ends one step and
        // starts the next); only loaded slots count at step 0
        const int ks = i - T_LSTART;
        if (ks >= 1) {
            const int e = T_LEND + 3 * (ks - 1);
            v = ks < nsteps ? tal[e] + tal[e + 1] + tal[e + 2] : 0u;
        }
        if (!v) continue;
        unsigned long long vv = v;
        if (i < T_NULL) atomicAdd(&ctl->coll[i / 16][i % 16], vv);
        else if (i < T_SPAWN) atomicAdd(&ctl->nulls[i - T_NULL], vv);
        else if (i < T_DEAD) atomicAdd(&ctl->spawned[i - T_SPAWN], vv);
        else if (i < T_ERR) atomicAdd(&ctl->dead[i - T_DEAD], vv);
        else if (i < T_LEND) atomicAdd(&ctl->err[i - T_ERR], vv);
        else if (i < T_LSTART) atomicAdd(&ctl->live_end[(i - T_LEND) / 3][(i - T_LEND) % 3], vv);
        else if (i < T_FLY) atomicAdd(&ctl->live_start[i - T_LSTART], vv);
    }
}

// The step kernel is instantiated for 2, 3 and 4 resident 256-thread blocks
// per SM (register budgets 128, 85 and 64); the launch shape is a tunable.
// Instantiations: the classic kernels in 2, 3 and 4 blocks per SM, the event
// kernel in 3 (its stash), each with or without the learned samplers'
// suspend/resume (LEARN); the general kernel (position-dependent field, wall
// crossings; learned samplers included) in 3, where it needs no register
// spills; the event kernels (plain, learned, general) have a second instance
// for launches of several steps (MULTI).  Code a launch does not use stays out
// of its kernel.
static void (*step_kernel(int minb, bool general, bool event, bool learn, bool multi))(StepArgs) {
    if (general) {
        if (!event) return k_step<3, true, false, true, false>;
        if (learn) return multi ? k_step<3, true, true, true, true> : k_step<3, true, true, true, false>;
        return multi ? k_step<3, true, true, false, true> : k_step<3, true, true, false, false>;
    }
    if (learn) {
        if (!event) return k_step<3, true, false, true, false>;
        return multi ? k_step<3, false, true, true, true> : k_step<3, false, true, true, false>;
    }
    if (event) return multi ? k_step<3, false, true, false, true> : k_step<3, false, true, false, false>;
    return (minb == 2)   ? k_step<2, false, false, false, false>
           : (minb == 3) ? k_step<3, false, false, false, false>
                         : k_step<4, false, false, false, false>;
}

cudaError_t launch_step(int minb, int grid, int threads, size_t smem, cudaStream_t stream, const StepArgs& A) {
    void (*kern)(StepArgs) = step_kernel(minb, A.general != 0, A.event != 0, A.learn != 0, A.nsteps > 1);
    // the shared-memory attribute is set outside stream capture (prepare_step
    // runs first); during capture the launch is only recorded
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(stream, &cs);
    if (e != cudaSuccess) return e;
    if (cs == cudaStreamCaptureStatusNone) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, threads, smem, stream>>>(A);
    return cudaGetLastError();
}

// Launch without touching the kernel's attributes (prepare_step ran first):
// setting an attribute between launches of a pipeline can hold the host back.
cudaError_t launch_step_prepared(int minb, int grid, int threads, size_t smem, cudaStream_t stream,
                                 const StepArgs& A) {
    step_kernel(minb, A.general != 0, A.event != 0, A.learn != 0, A.nsteps > 1)<<<grid, threads, smem, stream>>>(A);
    return cudaGetLastError();
}

cudaError_t prepare_step(int minb, size_t smem, bool general, bool event, bool learn) {
    for (bool multi : {false, true}) {
        cudaError_t e = cudaFuncSetAttribute(step_kernel(minb, general, event, learn, multi),
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Launch prologue: snapshot the work space and clear per-launch counters.
__global__ void k_begin(Control* ctl, long long cap0, long long cap1, long long cap2) {
    int t = threadIdx.x;
    const long long cap[3] = {cap0, cap1, cap2};
    if (t < 3) {
        unsigned long long n = ctl->n[t];
        if ((long long)n > cap[t]) n = (unsigned long long)cap[t];
        ctl->n[t] = n;
        ctl->n_start[t] = n;
        ctl->dead[t] = 0;
    }
    if (t == 0) { ctl->head = 0; ctl->spill_n = 0; ctl->timeout = 0; ctl->launch_seq += 1u; }
    for (int i = t; i < PCL_MAX_STEPS_PER_LAUNCH * 3; i += blockDim.x) ctl->live_end[i / 3][i % 3] = 0;
    for (int i = t; i < PCL_MAX_STEPS_PER_LAUNCH; i += blockDim.x) ctl->live_start[i] = 0;
}

// Spill-pass prologue: the spill queue written by the previous pass becomes
// the input of the next.
__global__ void k_begin_spill(Control* ctl, unsigned long long* in_n, unsigned long long* out_n) {
    if (threadIdx.x == 0) {   // out_n == nullptr: the pass appends to a queue that keeps its contents
        if (out_n) *out_n = 0;
        ctl->head = 0;
    }
    (void)in_n;
}

// ------------------------------------------------------------ compaction -
// repack! (population.jl:229-259) as an order-preserving stream compaction
// into the other buffer: count live slots per tile, scan the tile counts,
// scatter.  gridDim.y = species.
constexpr int kTile = 2048;



__global__ void k_compact_count(CompactArgs C) {
    const int sp = blockIdx.y;
    const long long n = (long long)C.n[sp];
    const long long t0 = (long long)blockIdx.x * kTile;
    if (t0 >= n) return;
    unsigned int cnt = 0;
    for (long long i = t0 + threadIdx.x; i < min(n, t0 + kTile); i += blockDim.x)
        cnt += (C.smeta[sp][i].z != PCL_DEAD_CTR) ? 1u : 0u;
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    __shared__ unsigned int ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += ws[w];
        C.tile_cnt[sp][blockIdx.x] = s;
    }
}

__global__ void k_compact_scan(CompactArgs C) {
    const int sp = blockIdx.x;
    const long long n = (long long)C.n[sp];
    const int nt = int((n + kTile - 1) / kTile);
    __shared__ unsigned long long carry;
    __shared__ unsigned long long wsum[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nt; base += blockDim.x) {
        int i = base + threadIdx.x;
        unsigned long long v = (i < nt) ? C.tile_cnt[sp][i] : 0ull;
        // block exclusive scan
        unsigned long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            unsigned long long w = (threadIdx.x < (blockDim.x >> 5)) ? wsum[threadIdx.x] : 0ull;
            for (int o = 1; o < 32; o <<= 1) {
                unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            wsum[threadIdx.x] = w;
        }
        __syncthreads();
        unsigned long long wpre = (threadIdx.x >= 32) ? wsum[(threadIdx.x >> 5) - 1] : 0ull;
        unsigned long long incl = x + wpre;
        if (i < nt) C.tile_off[sp][i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) C.n_out[sp] = carry;
}

__global__ void k_compact_scatter(CompactArgs C) {
    const int sp = blockIdx.y;
    const long long n = (long long)C.n[sp];
    const long long t0 = (long long)blockIdx.x * kTile;
    if (t0 >= n) return;
    __shared__ unsigned int wcnt[32];
    __shared__ unsigned long long run;
    if (threadIdx.x == 0) run = C.tile_off[sp][blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (long long b = t0; b < min(n, t0 + kTile); b += blockDim.x) {
        long long i = b + threadIdx.x;
        bool live = false;
        uint4 m;
        if (i < n && i < t0 + kTile) { m = C.smeta[sp][i]; live = (m.z != PCL_DEAD_CTR); }
        unsigned bal = __ballot_sync(0xffffffffu, live);
        if (lane == 0) wcnt[w] = __popc(bal);
        __syncthreads();
        unsigned int pre = 0, tot = 0;
        for (int q = 0; q < nw; ++q) { if (q < w) pre += wcnt[q]; tot += wcnt[q]; }
        if (live) {
            unsigned long long d = run + pre + __popc(bal & ((1u << lane) - 1u));
            C.dxw[sp][d] = C.sxw[sp][i];
            C.dps[sp][d] = C.sps[sp][i];
            C.dmeta[sp][d] = m;
        }
        __syncthreads();
        if (threadIdx.x == 0) run += tot;
        __syncthreads();
    }
}

// ------------------------------------------------------------- moments ---
// Double-float accumulation (hi + lo, ~48-bit significand) on the FP32 pipes:
// GB300 runs FP64 arithmetic at a small fraction of its FP32 rate, and a
// reduction of FP32 state in plain FP64 per particle is bound by it.
// (hi, lo) += a
__device__ __forceinline__ void df_acc(float& hi, float& lo, float a) {
    float s, e;
    two_sum(hi, a, s, e);
    e = __fadd_rn(e, lo);
    fast_two_sum(s, e, hi, lo);
}
// (hi, lo) += a b, the product split exactly into p + pe (fma)
__device__ __forceinline__ void df_acc_prod(float& hi, float& lo, float a, float b) {
    const float p = __fmul_rn(a, b), pe = __fmaf_rn(a, b, -p);
    float s, e;
    two_sum(hi, p, s, e);
    e = __fadd_rn(__fadd_rn(e, pe), lo);
    fast_two_sum(s, e, hi, lo);
}
// (hi, lo) += (bh, bl)
__device__ __forceinline__ void df_acc2(float& hi, float& lo, float bh, float bl) {
    float s, e;
    two_sum(hi, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, bl));
    fast_two_sum(s, e, hi, lo);
}

// Population moments (nactives, weight, meanenergy, spread, posvar;
// population.jl:89-223): sum w, sum w E, sum w x, y, z, sum w x^2, y^2, z^2,
// max E and the live count.  Per particle in FP32 (E = p^2 / (sqrt(1 + p^2)
// + 1), the step's cancellation-free form, with IEEE square root and division;
// products split exactly), summed per thread and per warp in double-float,
// and across warps in FP64.
__global__ void k_moments(const float4* xw, const float4* ps, const uint4* meta, long long n, int species,
                          double* out) {
    float hi[8] = {0, 0, 0, 0, 0, 0, 0, 0}, lo[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float emax = 0.0f;
    unsigned long long live = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        // the three records are loaded together, before the dead-slot test, so
        // their latencies overlap
        const uint4 m = meta[i];
        const float4 a = xw[i], b = ps[i];
        if (m.z == PCL_DEAD_CTR) continue;
        const float E = kin_energy_exact(species, b.x, b.y, b.z);
        const float w = a.w;
        df_acc(hi[0], lo[0], w);
        df_acc_prod(hi[1], lo[1], w, E);
        df_acc_prod(hi[2], lo[2], w, a.x);
        df_acc_prod(hi[3], lo[3], w, a.y);
        df_acc_prod(hi[4], lo[4], w, a.z);
        const float c[3] = {a.x, a.y, a.z};
#pragma unroll
        for (int q = 0; q < 3; ++q) {   // w c^2: c^2 = p + pe exactly, then w p exactly and w pe in FP32
            const float p = __fmul_rn(c[q], c[q]), pe = __fmaf_rn(c[q], c[q], -p);
            df_acc_prod(hi[5 + q], lo[5 + q], w, p);
            df_acc(hi[5 + q], lo[5 + q], __fmul_rn(w, pe));
        }
        emax = fmaxf(emax, E);
        live += 1;
    }
    for (int o = 16; o; o >>= 1) {
        for (int q = 0; q < 8; ++q) {
            const float bh = __shfl_xor_sync(0xffffffffu, hi[q], o), bl = __shfl_xor_sync(0xffffffffu, lo[q], o);
            df_acc2(hi[q], lo[q], bh, bl);
        }
        emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        live += __shfl_xor_sync(0xffffffffu, live, o);
    }
    if ((threadIdx.x & 31) == 0) {
        for (int q = 0; q < 8; ++q) atomicAdd(&out[q], double(hi[q]) + double(lo[q]));
        atomicMax(reinterpret_cast<unsigned long long*>(&out[8]),
                  (unsigned long long)__double_as_longlong(double(emax)));
        atomicAdd(reinterpret_cast<unsigned long long*>(&out[9]), live);
    }
}

// Energy spectrum of the live particles, as the reference's scripts build one
// with StatsBase.fit(Histogram, E, edges[, weights]) (scripts/beam.jl:137-147,
// scripts/swarm.jl:149-158): bin i counts edges[i] <= E < edges[i+1] (device
// energy units, FP64 from the FP32 momentum, as the host computes it from the
// downloaded state); energies outside [edges[0], edges[nb]) are not counted.  swarm >= 0 keeps the particles of
// that swarm (top 8 bits of the stream id) only.  Per-block shared bins, one
// global atomic per non-empty bin.
__global__ void k_energy_hist(const float4* xw, const float4* ps, const uint4* meta, const unsigned long long* nslots,
                              long long cap, int species, int swarm, const double* edges, int nb,
                              unsigned long long* counts, double* wsum) {
    extern __shared__ double hsh[];
    double* se = hsh;                 // [nb + 1] edges
    double* sw = hsh + nb + 1;        // [nb] weights other than 1
    unsigned int* sc = reinterpret_cast<unsigned int*>(sw + nb);   // [nb] counts
    unsigned int* s1 = sc + nb;       // [nb] counts of weight-1 particles (most populations)
    float* sf = reinterpret_cast<float*>(s1 + nb);                 // [nb + 1] edges rounded to FP32
    for (int i = threadIdx.x; i <= nb; i += blockDim.x) { se[i] = edges[i]; sf[i] = float(edges[i]); }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) { sw[i] = 0.0; sc[i] = 0u; s1[i] = 0u; }
    __syncthreads();
    const long long n = min((long long)*nslots, cap);
    const double lo = se[0], hi = se[nb];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const uint4 m = meta[i];
        const float4 b = ps[i];
        const float w = xw[i].w;      // loaded with the others, so the latencies overlap
        if (m.z == PCL_DEAD_CTR) continue;
        if (swarm >= 0 && int(m.y >> 24) != swarm) continue;
        // the bin from the FP32 energy and FP32 edges (GB300's FP64 rate is a
        // small fraction of its FP32 rate); the FP64 energy decides whenever
        // the FP32 one lies within 1e-6 (relative) of an edge it was compared
        // with, a margin far above both roundings
        const float Ef = kin_energy_exact(species, b.x, b.y, b.z);
        const float tol = 1e-6f * Ef;
        const float flo = sf[0], fhi = sf[nb];
        bool near = fabsf(Ef - flo) <= tol || fabsf(Ef - fhi) <= tol;
        int a = 0, z = nb;            // se[a] <= E < se[z]
        if (!near && (Ef >= flo && Ef < fhi)) {
            while (z - a > 1) {
                const int mid = (a + z) >> 1;
                const float d = Ef - sf[mid];
                near = near || fabsf(d) <= tol;
                if (d >= 0.0f) a = mid; else z = mid;
            }
        } else if (!near) {
            continue;                 // clearly outside [edges[0], edges[nb])
        }
        if (near) {
            const double p2 = double(b.x) * b.x + double(b.y) * b.y + double(b.z) * b.z;
            const double E = (species == PCL_PHOTON) ? sqrt(p2) : p2 / (sqrt(1.0 + p2) + 1.0);
            if (!(E >= lo && E < hi)) continue;
            a = 0; z = nb;
            while (z - a > 1) {
                const int mid = (a + z) >> 1;
                if (E >= se[mid]) a = mid; else z = mid;
            }
        }
        atomicAdd(&sc[a], 1u);
        // a weight of exactly 1 is counted in integers (a shared FP64 atomic is
        // a compare-and-swap loop); other weights are summed in FP64
        if (w == 1.0f) atomicAdd(&s1[a], 1u);
        else atomicAdd(&sw[a], double(w));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        if (sc[i]) {
            atomicAdd(&counts[i], (unsigned long long)sc[i]);
            atomicAdd(&wsum[i], sw[i] + double(s1[i]));
        }
    }
}

// FP64 moments per swarm of a batched context: out[sw][6] = {live, sum w,
// sum w E, sum w z, sum w z^2, sum w x^2 + y^2}; lanes of one warp are grouped
// by swarm before the atomics.
// Per-swarm moments: live count, sum w, sum w E, sum w z, sum w z^2,
// sum w (x^2 + y^2).  Per-particle values in FP32, sums in FP64: warp groups
// of the same swarm combine by shuffles, each block accumulates in shared
// memory and writes one partial row; k_swarm_reduce adds the rows.
__global__ void k_swarm_moments(const float4* xw, const float4* ps, const uint4* meta, long long n, int species,
                                int nswarm, double* partial) {
    extern __shared__ double acc[];
    const int len = 6 * nswarm;
    for (int i = threadIdx.x; i < len; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    // the warp's running sums of its current swarm, in double-float (a shared
    // FP64 atomic is a compare-and-swap loop on GB300): flushed to shared
    // memory when the swarm changes and at the end
    float rh[6] = {0, 0, 0, 0, 0, 0}, rl[6] = {0, 0, 0, 0, 0, 0};
    int cur = -1;
    auto flush = [&]() {
        if (cur >= 0 && (threadIdx.x & 31) == 0)
            for (int q = 0; q < 6; ++q) atomicAdd(&acc[6 * cur + q], double(rh[q]) + double(rl[q]));
        for (int q = 0; q < 6; ++q) { rh[q] = 0.0f; rl[q] = 0.0f; }
        cur = -1;
    };
    for (long long i0 = (long long)blockIdx.x * blockDim.x; i0 < n; i0 += (long long)gridDim.x * blockDim.x) {
        long long i = i0 + threadIdx.x;
        bool live = false;
        int sw = 0;
        float v[6] = {0, 0, 0, 0, 0, 0};
        if (i < n) {
            uint4 m = meta[i];
            if (m.z != PCL_DEAD_CTR) {
                live = true;
                sw = min(int(m.y >> 24), nswarm - 1);
                float4 a = xw[i], b = ps[i];
                const float E = kin_energy(species, b.x, b.y, b.z);
                const float w = a.w;
                v[0] = 1.0f; v[1] = w; v[2] = w * E; v[3] = w * a.z; v[4] = w * a.z * a.z;
                v[5] = w * (a.x * a.x + a.y * a.y);
            }
        }
        const unsigned FULL = 0xffffffffu;
        unsigned act = __ballot_sync(FULL, live);
        if (!act) continue;
        const int sw0 = __shfl_sync(FULL, sw, __ffs(act) - 1);
        if (__all_sync(FULL, !live || sw == sw0)) {
            // the usual case (swarms are contiguous): one butterfly sum per value,
            // added to the warp's running sums
            if (sw0 != cur) { flush(); cur = sw0; }
            for (int q = 0; q < 6; ++q) {
                float t = v[q];
                for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
                df_acc(rh[q], rl[q], t);
            }
        } else {
            flush();
            if (!live) continue;
            unsigned grp = __match_any_sync(act, sw);
            int leader = __ffs(grp) - 1;
            for (int q = 0; q < 6; ++q) {
                double tot = 0.0;
                for (unsigned g = grp; g; g &= g - 1) tot += double(__shfl_sync(grp, v[q], __ffs(g) - 1));
                if ((threadIdx.x & 31) == leader) atomicAdd(&acc[6 * sw + q], tot);
            }
        }
    }
    flush();
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += blockDim.x) partial[(size_t)blockIdx.x * len + i] = acc[i];
}

// One warp per value: its lanes sum every 32nd block's partial, then a
// butterfly adds the lanes (a thread walking all blocks' rows alone was bound
// by the latency of its dependent loads).
__global__ void k_swarm_reduce(const double* partial, int nblocks, int len, double* out) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= len) return;
    double s = 0.0;
    for (int b = lane; b < nblocks; b += 32) s += partial[(size_t)b * len + i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[i] = s;
}

// ------------------------------------------------------- sampler test ----
// Test hook behind pcl_test_sampler: force table position j for n primaries.
__global__ void k_test_sampler(StepArgs A, int species, int j, long long n, const float* p_in,
                               const uint32_t* sid, float* out_p, float* out_s, int* out_kind,
                               uint32_t* out_ctr) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(smem + A.blob_bytes);
    __shared__ uint32_t tal[T_WORDS];
    for (int i = threadIdx.x; i < T_WORDS; i += blockDim.x) tal[i] = 0u;
    bool ok = stage_blob(smem, A.blob, A.blob_bytes, mbar);
    if (__syncthreads_or(!ok)) return;
    const BlobHdr* H = reinterpret_cast<const BlobHdr*>(smem);
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float capbuf[8];
    int ncap = 0;
    KCtx K;
    K.H = H; K.blob = reinterpret_cast<const float*>(smem); K.stk = nullptr; K.top = nullptr; K.tal = tal;
    K.A = &A; K.cap = capbuf; K.ncap = &ncap;
    Lane L;
    L.x = L.y = L.z = 0.0f; L.w = 1.0f; L.th = 0.0f; L.tlo = 0.0f; L.k = 0; L.s = 0.0f;
    L.px = p_in[3 * i]; L.py = p_in[3 * i + 1]; L.pz = p_in[3 * i + 2];
    L.sid_lo = sid[2 * i]; L.sid_hi = sid[2 * i + 1]; L.ctr = 0u; L.rvalid = false;
    L.species = species; L.alive = true; L.slot = -1; L.nsub = 0; L.sw = 0;
    const SpeciesHdr& S = H->sp[species];
    float E = kin_energy(species, L.px, L.py, L.pz);
    L.r = setr(S, K, E, 0);
    const DevProc& P = S.proc[j];
    sample_process(L, K, S, P, E, 0u);
    for (int q = 0; q < 3; ++q) out_kind[3 * i + q] = -1;
    if (L.alive) {
        out_p[9 * i + 0] = L.px; out_p[9 * i + 1] = L.py; out_p[9 * i + 2] = L.pz;
        out_s[3 * i] = L.s; out_kind[3 * i] = species;
    }
    // secondaries: species per process kind
    int ks[2] = {-1, -1};
    switch (P.kind) {
        case PCL_PROC_MOLLER: case PCL_PROC_RBEB: case PCL_PROC_COMPTON: case PCL_PROC_KN_COMPTON:
        case PCL_PROC_PHOTOELECTRIC: case PCL_PROC_BHABHA: ks[0] = PCL_ELECTRON; break;
        case PCL_PROC_SELTZER_BERGER: ks[0] = PCL_PHOTON; break;
        case PCL_PROC_BETHE_HEITLER: ks[0] = PCL_ELECTRON; ks[1] = PCL_POSITRON; break;
        case PCL_PROC_ANNIHILATION: ks[0] = PCL_PHOTON; ks[1] = PCL_PHOTON; break;
        default: break;
    }
    for (int c = 0; c < ncap && c < 2; ++c) {
        out_p[9 * i + 3 * (c + 1) + 0] = capbuf[4 * c + 0];
        out_p[9 * i + 3 * (c + 1) + 1] = capbuf[4 * c + 1];
        out_p[9 * i + 3 * (c + 1) + 2] = capbuf[4 * c + 2];
        out_s[3 * i + c + 1] = capbuf[4 * c + 3];
        out_kind[3 * i + c + 1] = ks[c];
    }
    out_ctr[i] = L.ctr;
}

// ------------------------------------------------- variance reduction ---
// The particle's next stream word (the draw a Lane would take at counter ctr).
__device__ __forceinline__ uint32_t stream_word(uint32_t ctr, uint32_t lo, uint32_t hi, uint32_t k0, uint32_t k1) {
    uint32_t a = ctr >> 2, b = lo, c = hi, d = 0u;
    philox4x32_10(a, b, c, d, k0, k1);
    const uint32_t sh = ctr & 3u;
    return sh == 0u ? a : (sh == 1u ? b : (sh == 2u ? c : d));
}

// roulette! (population.jl:291-311): keep a live particle with probability
// pkeep (one draw from its stream) and divide its weight by pkeep, else
// remove it.
__global__ void k_roulette(float4* xw, uint4* meta, long long n, float pkeep, uint32_t k0, uint32_t k1,
                           unsigned long long* dead) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        uint4 m = meta[i];
        if (m.z == PCL_DEAD_CTR) continue;
        const float u = bits_to_u(stream_word(m.z, m.x, m.y, k0, k1));
        if (u < pkeep) {
            xw[i].w = xw[i].w / pkeep;
            meta[i].z = m.z + 1u;
        } else {
            meta[i].z = PCL_DEAD_CTR;
            atomicAdd(dead, 1ull);
        }
    }
}

// f(E) of a table of nt nodes (tab: energies E_i ascending, values v_i,
// slopes (v_{i+1} - v_i) / (E_{i+1} - E_i) in FP64, then the energies
// rounded to FP32), linear in E between nodes and constant beyond the ends.
// The interval is found by bisection over the FP32 energies (at most 12
// halvings for 4096 nodes) and corrected with FP64 comparisons, so it is the
// FP64 interval; then one FP64 multiply-add: GB300's FP64 rate is a small
// fraction of its FP32 rate, and the division it saves dominated the cost.
__device__ __forceinline__ double table_fn(const double* tab, int nt, double e) {
    const double* tE = tab;
    const double* tV = tab + nt;
    const double* tS = tab + 2 * nt;
    const float* tF = reinterpret_cast<const float*>(tab + 3 * nt);
    if (!(e > tE[0])) return tV[0];
    if (!(e < tE[nt - 1])) return tV[nt - 1];
    const float ef = float(e);
    int lo = 0, hi = nt - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tF[mid] <= ef) lo = mid; else hi = mid;
    }
    while (lo > 0 && e < tE[lo]) --lo;
    while (lo < nt - 2 && !(e < tE[lo + 1])) ++lo;
    return __fma_rn(__dsub_rn(e, tE[lo]), tS[lo], tV[lo]);
}

// roulette!(f, popl) (population.jl:291-305) with f of the kinetic energy
// given as a table (energies in units of m_e c^2): keep with probability
// q = f(E) (one draw), dividing the weight by q, else remove; q <= 0
// removes, q >= 1 keeps.  E from the FP32 momentum with IEEE operations.
__global__ void k_roulette_fn(float4* xw, const float4* ps, uint4* meta, long long n, int species, const double* tab,
                              int nt, uint32_t k0, uint32_t k1, unsigned long long* dead) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        uint4 m = meta[i];
        if (m.z == PCL_DEAD_CTR) continue;
        const float4 q4 = ps[i];
        const float q = float(table_fn(tab, nt, double(kin_energy_exact(species, q4.x, q4.y, q4.z))));
        const float u = bits_to_u(stream_word(m.z, m.x, m.y, k0, k1));
        if (u < q) {
            xw[i].w = xw[i].w / q;
            meta[i].z = m.z + 1u;
        } else {
            meta[i].z = PCL_DEAD_CTR;
            atomicAdd(dead, 1ull);
        }
    }
}

// roulette! with a keep probability per swarm (batched swarms: the swarm is
// the top 8 bits of the stream id); pkeep >= 1 leaves a swarm untouched and
// takes no draw.
__global__ void k_roulette_swarms(float4* xw, uint4* meta, long long n, const float* pkeep, int nswarm, uint32_t k0,
                                  uint32_t k1, unsigned long long* dead) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        uint4 m = meta[i];
        if (m.z == PCL_DEAD_CTR) continue;
        const float q = pkeep[min(int(m.y >> 24), nswarm - 1)];
        if (!(q < 1.0f)) continue;
        const float u = bits_to_u(stream_word(m.z, m.x, m.y, k0, k1));
        if (u < q) {
            xw[i].w = xw[i].w / q;
            meta[i].z = m.z + 1u;
        } else {
            meta[i].z = PCL_DEAD_CTR;
            atomicAdd(dead, 1ull);
        }
    }
}

// Live particles per swarm (the top 8 bits of the stream id; every particle
// counts as swarm 0 when nswarm is 1), added into counts[0..nswarm), over the
// min(*nslots, cap) slots of the species (read on the device, so that the
// launch needs no host read-back).  A warp whose live particles share one
// swarm adds them with one shared atomic.
__global__ void k_swarm_count(const uint4* meta, const unsigned long long* nslots, long long cap, int nswarm,
                              unsigned int* counts) {
    __shared__ unsigned int h[256];
    const long long n = min((long long)*nslots, cap);
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0u;
    __syncthreads();
    const unsigned FULL = 0xffffffffu;
    const long long n32 = (n + 31) / 32 * 32;   // whole warps stay in the loop together
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n32;
         i += (long long)gridDim.x * blockDim.x) {
        int sw = -1;
        if (i < n) {
            const uint4 m = meta[i];
            if (m.z != PCL_DEAD_CTR) sw = min(int(m.y >> 24), nswarm - 1);
        }
        const unsigned act = __ballot_sync(FULL, sw >= 0);
        if (!act) continue;
        const int sw0 = __shfl_sync(FULL, sw, __ffs(act) - 1);
        if (__all_sync(FULL, sw < 0 || sw == sw0)) {
            if ((threadIdx.x & 31) == 0) atomicAdd(&h[sw0], unsigned(__popc(act)));
        } else {
            const unsigned grp = __match_any_sync(FULL, sw);
            if (sw >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&h[sw], unsigned(__popc(grp)));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nswarm; i += blockDim.x)
        if (h[i]) atomicAdd(&counts[i], h[i]);
}

// RouletteCallback (callback.jl:210-227) per swarm on the device: a swarm with
// n > cap live particles gets roulette!(cap / n) (the keep probability rounded
// to FP32 as in k_roulette_swarms), with n from k_swarm_count.  A block with
// no swarm over the cap returns before it reads a particle.
__global__ void k_roulette_cap(float4* xw, uint4* meta, const unsigned long long* nslots, long long slot_cap,
                               const unsigned int* counts, int nswarm, unsigned long long cap, uint32_t k0,
                               uint32_t k1) {
    const long long n = min((long long)*nslots, slot_cap);
    // each swarm's keep probability once per block (an FP64 quotient, which
    // GB300 runs at a small fraction of its FP32 rate); 2 = under the cap
    __shared__ float qs[256];
    int over = 0;
    for (int i = threadIdx.x; i < nswarm; i += blockDim.x) {
        const unsigned int cnt = counts[i];
        over |= (cnt > cap);
        qs[i] = (cnt > cap) ? float(double(cap) / double(cnt)) : 2.0f;
    }
    if (!__syncthreads_or(over)) return;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const uint4 m = meta[i];
        if (m.z == PCL_DEAD_CTR) continue;
        const float q = qs[min(int(m.y >> 24), nswarm - 1)];
        if (q > 1.0f) continue;
        const float u = bits_to_u(stream_word(m.z, m.x, m.y, k0, k1));
        if (u < q) {
            xw[i].w = xw[i].w / q;
            meta[i].z = m.z + 1u;
        } else {
            meta[i].z = PCL_DEAD_CTR;
        }
    }
}

// split! (population.jl:318-335): divide a live particle's weight by 1 + p and
// add Poisson(p) copies of it (number by inversion with one draw from its
// stream; the reference draws it from Distributions.jl).  The inversion sums
// the pmf in Float64 from e = exp(-p) (computed on the host), with
// correctly rounded operations that the compiler cannot contract, so the sum
// passes every uniform below 1 and matches a host computation bit for bit.
// Copy j gets the stream id of words (2(j%2), 2(j%2)+1) of Philox block
// (ctr, sid, 2 + j/2) of its parent and a fresh counter; in swarm mode
// (nswarm > 0) its top 8 bits stay the parent's swarm, as for any secondary.
// x, p, w, s and the step clock are copied.
// One particle of split!: weight / (1 + p), Poisson(p) copies (above), u the
// particle's draw and e = exp(-p).
__device__ __forceinline__ void split_one(float4* xw, float4* ps, uint4* meta, long long i, uint4 m, long long cap,
                                          float p, float u, double e, int nswarm, uint32_t k0, uint32_t k1,
                                          unsigned long long* nslots, unsigned long long* lost) {
    const double pd = double(p);
    float4 a = xw[i];
    a.w = a.w / (1.0f + p);
    xw[i] = a;
    const uint32_t ctr0 = m.z;
    meta[i].z = m.z + 1u;
    int k = 0;
    double P = e, F = e;
    const double ud = double(u);
    while (ud > F && k < 1024) {
        ++k;
        P = __dmul_rn(P, __ddiv_rn(pd, double(k)));
        F = __dadd_rn(F, P);
    }
    if (k == 0) return;
    const float4 b = ps[i];
    for (int j = 0; j < k; ++j) {
        uint32_t c0 = ctr0, c1 = m.x, c2 = m.y, c3 = 2u + uint32_t(j >> 1);
        philox4x32_10(c0, c1, c2, c3, k0, k1);
        uint32_t lo = (j & 1) ? c2 : c0, hi = (j & 1) ? c3 : c1;
        if (nswarm > 0) hi = (hi & 0x00FFFFFFu) | (m.y & 0xFF000000u);
        const unsigned long long q = atomicAdd(nslots, 1ull);
        if ((long long)q < cap) {
            xw[q] = a;
            ps[q] = b;
            meta[q] = make_uint4(lo, hi, 0u, m.w);
        } else {
            atomicAdd(lost, 1ull);
        }
    }
}

__global__ void k_split(float4* xw, float4* ps, uint4* meta, long long n, long long cap, float p, double e,
                        int nswarm, uint32_t k0, uint32_t k1, unsigned long long* nslots, unsigned long long* lost) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const uint4 m = meta[i];
        if (m.z == PCL_DEAD_CTR) continue;
        const float u = bits_to_u(stream_word(m.z, m.x, m.y, k0, k1));
        split_one(xw, ps, meta, i, m, cap, p, u, e, nswarm, k0, k1, nslots, lost);
    }
}

// split!(f, popl) (population.jl:316-331) with the mean number of copies a
// function of the kinetic energy, given as a table as for k_roulette_fn
// (values in [0, 64]); exp(-p) is the device's FP64 exp.  A particle draws no
// copy when u <= exp(-p), i.e. -ln u >= p: where the FP32 logarithm (within a
// few ulp) clears p by a relative 1e-5, that outcome is certain and the FP64
// exponential is skipped (e = 1 gives the same k = 0), so the copies are
// those of the exact test.
__global__ void k_split_fn(float4* xw, float4* ps, uint4* meta, long long n, long long cap, int species,
                           const double* tab, int nt, int nswarm, uint32_t k0, uint32_t k1,
                           unsigned long long* nslots, unsigned long long* lost) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const uint4 m = meta[i];
        if (m.z == PCL_DEAD_CTR) continue;
        const float4 q4 = ps[i];
        const float p = float(table_fn(tab, nt, double(kin_energy_exact(species, q4.x, q4.y, q4.z))));
        const float u = bits_to_u(stream_word(m.z, m.x, m.y, k0, k1));
        const bool none = -logf(u) > p * 1.00001f + 1e-6f;
        split_one(xw, ps, meta, i, m, cap, p, u, none ? 1.0 : exp(-double(p)), nswarm, k0, k1, nslots, lost);
    }
}

// ------------------------------------------------ learned-sampler data --
// Training data: samples of the table sampler of process j at nT energies
// a_g = -1 + 2 g / (nT - 1), T = 10^(6 + 2 a_g) eV, primary along z, each
// sample histogrammed (nbins over [hmin, hmax)) in the network's output
// variable: ln(k / T) of the photon (bremsstrahlung) or v = (1 - e0 / eps) /
// (1 - 2 e0) of the secondary (Moller).
__global__ void k_learn_hist(StepArgs A, int species, int j, int kind, int nT, long long per_T, int nbins,
                             float hmin, float hmax, unsigned long long sid_base, unsigned int* hist) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(smem + A.blob_bytes);
    __shared__ uint32_t tal[T_WORDS];
    for (int i = threadIdx.x; i < T_WORDS; i += blockDim.x) tal[i] = 0u;
    bool ok = stage_blob(smem, A.blob, A.blob_bytes, mbar);
    if (__syncthreads_or(!ok)) return;
    const BlobHdr* H = reinterpret_cast<const BlobHdr*>(smem);
    float capbuf[8];
    int ncap = 0;
    KCtx K;
    K.H = H; K.blob = reinterpret_cast<const float*>(smem); K.stk = nullptr; K.top = nullptr; K.tal = tal;
    K.A = &A; K.cap = capbuf; K.ncap = &ncap;
    const SpeciesHdr& S = H->sp[species];
    const DevProc& P = S.proc[j];
    const long long total = (long long)nT * per_T;
    const float scale = float(nbins) / (hmax - hmin);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int g = int(i / per_T);
        const float a = (nT > 1) ? -1.0f + 2.0f * float(g) / float(nT - 1) : 0.0f;
        const float E0 = exp10f(6.0f + 2.0f * a) / 510998.95f;
        Lane L;
        L.x = L.y = L.z = 0.0f; L.w = 1.0f; L.th = 0.0f; L.tlo = 0.0f; L.k = 0; L.s = 0.0f;
        L.px = 0.0f; L.py = 0.0f; L.pz = sqrtf(E0 * (E0 + 2.0f));
        const unsigned long long sid = sid_base + (unsigned long long)i;
        L.sid_lo = uint32_t(sid); L.sid_hi = uint32_t(sid >> 32); L.ctr = 0u; L.rvalid = false;
        L.species = species; L.alive = true; L.slot = -1; L.nsub = 0; L.sw = 0; L.r = 0.0f;
        const float E = kin_energy_exact(species, 0.0f, 0.0f, L.pz);
        ncap = 0;
        sample_process(L, K, S, P, E, 0u);
        if (ncap < 1) continue;
        const float cx = capbuf[0], cy = capbuf[1], cz = capbuf[2];
        float h;
        if (kind == PCL_LEARN_SB) {
            h = 1.0f - logf(sqrtf(cx * cx + cy * cy + cz * cz) / E) / sb_ymin(K, P, E);
        } else {
            const float p2 = cx * cx + cy * cy + cz * cz;
            const float eps = p2 / (sqrtf(1.0f + p2) + 1.0f) / E;
            const float e0 = P.p[0] / E;
            h = (1.0f - e0 / eps) / (1.0f - 2.0f * e0);
        }
        int b = int(floorf((h - hmin) * scale));
        b = min(max(b, 0), nbins - 1);
        atomicAdd(&hist[(size_t)g * nbins + b], 1u);
    }
}

// Network inputs of the suspended collisions: (a, 2u - 1).
__global__ void k_learn_x(const float4* ps, const float4* m2, const unsigned long long* n_dev, long long cap,
                          float* X) {
    const long long n = min((long long)*n_dev, cap);   // the queue counter can pass its capacity
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 b = ps[i];
        float4 q = m2[i];
        int sp = int(__float_as_uint(q.w) & 3u);
        X[2 * i] = learn_a(kin_energy_exact(sp, b.x, b.y, b.z));
        X[2 * i + 1] = 2.0f * q.z - 1.0f;
    }
}

// Output of the network attached to each suspended collision's process:
// Y[i] = Yk[which[species][j] * stride + i].
__global__ void k_learn_pick(const float4* m2, const unsigned long long* n_dev, long long cap, const float* Yk,
                             long long stride, LearnPick which, float* Y) {
    const long long n = min((long long)*n_dev, cap);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint32_t pk = __float_as_uint(m2[i].w);
        int sp = int(pk & 3u), j = int((pk >> 8) & 15u);
        int w = which.net[sp * 16 + j];
        Y[i] = Yk[(long long)max(w, 0) * stride + i];
    }
}

// ------------------------------------------ energy-draw cost (test hook) --
// The secondary-energy draw alone, for timing the table samplers against the
// networks: primary i of n at E_i = 10^(4 + 4 (i + 1/2) / n) eV along z, with
// stream id sid_base + i.
__device__ __forceinline__ float draw_grid_energy(long long i, long long n) {
    return exp10f(4.0f + 4.0f * (float(i) + 0.5f) / float(n)) / 510998.95f;
}

__device__ __forceinline__ void draw_lane(Lane& L, int species, unsigned long long sid, float E) {
    L.x = L.y = L.z = 0.0f; L.w = 1.0f; L.th = 0.0f; L.tlo = 0.0f; L.k = 0; L.s = 0.0f;
    L.px = 0.0f; L.py = 0.0f; L.pz = sqrtf(E * (E + 2.0f));
    L.sid_lo = uint32_t(sid); L.sid_hi = uint32_t(sid >> 32); L.ctr = 0u; L.rvalid = false;
    L.species = species; L.alive = true; L.slot = -1; L.nsub = 0; L.sw = 0; L.r = 0.0f;
}

// Table path: k / T (Seltzer-Berger) or eps (Moller) from the table sampler's
// energy draw; draws[i] = uniforms it consumed.
__global__ void k_draw_table(StepArgs A, int species, int j, int kind, long long n, unsigned long long sid_base,
                             float* out, uint32_t* draws) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(smem + A.blob_bytes);
    __shared__ uint32_t tal[T_WORDS];
    for (int i = threadIdx.x; i < T_WORDS; i += blockDim.x) tal[i] = 0u;
    bool ok = stage_blob(smem, A.blob, A.blob_bytes, mbar);
    if (__syncthreads_or(!ok)) return;
    KCtx K;
    K.H = reinterpret_cast<const BlobHdr*>(smem); K.blob = reinterpret_cast<const float*>(smem); K.stk = nullptr;
    K.top = nullptr; K.tal = tal; K.A = &A; K.cap = nullptr; K.ncap = nullptr;
    const DevProc& P = K.H->sp[species].proc[j];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float E = draw_grid_energy(i, n);
        Lane L;
        draw_lane(L, species, sid_base + (unsigned long long)i, E);
        out[i] = (kind == PCL_LEARN_SB) ? sb_k(L, K, P, E) / E : moller_eps(L, K, P, E);
        draws[i] = L.ctr;
    }
}

// Network path, before the network: its inputs (a, 2u - 1), one uniform each.
__global__ void k_draw_net_x(long long n, unsigned long long sid_base, uint32_t k0, uint32_t k1, float* X) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float E = draw_grid_energy(i, n);
        Lane L;
        draw_lane(L, 0, sid_base + (unsigned long long)i, E);
        const float u = bits_to_u(next_bits(L, k0, k1));
        X[2 * i] = learn_a(E);
        X[2 * i + 1] = 2.0f * u - 1.0f;
    }
}

// Network path, after the network: its output mapped to k / T or eps as the
// step's learned samplers map it (learned_outcome).
__global__ void k_draw_net_map(StepArgs A, int species, int j, int kind, long long n, const float* Y, float* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(smem + A.blob_bytes);
    bool ok = stage_blob(smem, A.blob, A.blob_bytes, mbar);
    if (__syncthreads_or(!ok)) return;
    KCtx K;
    K.H = reinterpret_cast<const BlobHdr*>(smem); K.blob = reinterpret_cast<const float*>(smem); K.stk = nullptr;
    K.top = nullptr; K.tal = nullptr; K.A = &A; K.cap = nullptr; K.ncap = nullptr;
    const DevProc& P = K.H->sp[species].proc[j];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float E = draw_grid_energy(i, n);
        const float v = fminf(fmaxf(Y[i], 0.0f), 1.0f);
        if (kind == PCL_LEARN_SB) {
            out[i] = expf(fminf((1.0f - v) * sb_ymin(K, P, E), -1e-6f));
        } else {
            const float e0 = P.p[0] / E;
            out[i] = e0 / (1.0f - v * (1.0f - 2.0f * e0));
        }
    }
}

// Shared-memory bytes of k_step for a block of `threads`.
size_t step_smem_bytes(int blob_bytes, int threads, bool event) {
    int nw = threads / 32;
    size_t b = size_t(blob_bytes) + size_t(nw) * kWarpStack * 3 * 16 + size_t(nw) * 4 + T_WORDS * 4 + 64;
    if (event) b += 16 + size_t(nw) * kCollStash * 5 * 16 + size_t(nw) * 8;
    return (b + 15) & ~size_t(15);
}

}  // namespace pcl
