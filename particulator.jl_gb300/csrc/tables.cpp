// Host-side (FP64) table builders: the init path of the reference, restated so
// that the shared library can produce every table the device step consumes.
//
//   BinaryIntervals / chebnodes / chebval / precheb / chebeval / chebdiff /
//   chebfit ............................................ src/cheby.jl:15-227
//   collision_table_from_processes, compratebound ....... src/collision_table.jl:115-167
//   LogLinRange ......................................... src/util.jl:60-127
//   totalcs of every process ............................ the per-process files cited below
//   SeltzerBerger table builder (findcumvalues, scaledcs) src/seltzer.jl:23-64,163-231
//   ContinuumLoss energy_loss, ChebContinuumLoss ......... src/continuum.jl:6-139
//
// The reference evaluates these once at set-up in Float64; so do we.  Where
// the reference relies on a third-party routine the restatement is noted:
// LinearAlgebra `\` (an n x n LU solve with partial pivoting) and BSplineKit
// order-2 interpolation (piecewise-linear interpolant, its exact piecewise
// quadratic antiderivative, Newton inversion to rtol 1e-6).
#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>
#include <numeric>
#include <limits>

#include "physconst.h"
#include "../../include/particulator_gb300.h"

namespace pcl {
using namespace si;

// ---------------------------------------------------------------- helpers --
// Julia's max(a, b) for Float64 propagates NaN (used by several totalcs).
static inline double jmax(double a, double b) {
    if (std::isnan(a) || std::isnan(b)) return std::numeric_limits<double>::quiet_NaN();
    return a > b ? a : b;
}

// Binary intervals (cheby.jl:15-36): interval 0 = (0, xmax 2^-k), interval
// i >= 1 = (xmax 2^(i-k-1), xmax 2^(i-k)).
struct BinaryIntervals {
    int k;
    double xmax;
    void interval(int i, double& l, double& r) const {
        if (i == 0) {
            double l1, r1;
            interval(1, l1, r1);
            l = 0.0;
            r = l1;
            return;
        }
        double lf = std::ldexp(1.0, i - k - 1);
        l = lf * xmax;
        r = 2.0 * lf * xmax;
    }
};

// chebval (cheby.jl:57-81): T_0..T_{n-1}(xi)
static inline void chebval(double xi, int n, double* t) {
    t[0] = 1.0;
    if (n > 1) t[1] = xi;
    for (int j = 2; j < n; ++j) t[j] = 2.0 * xi * t[j - 1] - t[j - 2];
}

// precheb (cheby.jl:127-143)
static inline void precheb(double x, const BinaryIntervals& b, int n, int& i, double* t) {
    double x1 = x / b.xmax;
    int l = 0;
    double s = std::frexp(x1, &l);
    i = (x1 == 0.0) ? 0 : l + b.k;
    double xi;
    if (i > 0) {
        xi = 4.0 * s - 3.0;
    } else {
        xi = std::ldexp(1.0, b.k + 1) * x1 - 1.0;
        i = 0;
    }
    chebval(xi, n, t);
}

// chebeval (cheby.jl:111-125); a is [n][k+1] column-major with stride `ld`
// between intervals and `st` between terms.
static inline double chebeval(double x, const BinaryIntervals& b, const double* a, int n,
                              int st, int ld) {
    int i;
    double t[PCL_MAX_ORDER];
    precheb(x, b, n, i, t);
    double s = 0.0;
    for (int j = 0; j < n; ++j) s += a[j * st + i * ld] * t[j];
    return s;
}

// chebdiff (cheby.jl:153-203)
static inline double chebdiff(double x, const BinaryIntervals& b, const double* a, int n,
                              int st, int ld) {
    double x1 = x / b.xmax;
    int lexp = 0;
    double s = std::frexp(x1, &lexp);
    int i = (x1 == 0.0) ? 0 : lexp + b.k;
    double xi;
    if (i > 0) {
        xi = 4.0 * s - 3.0;
    } else {
        xi = std::ldexp(1.0, b.k + 1) * x1 - 1.0;
        i = 0;
    }
    double l, r;
    b.interval(i, l, r);
    double u0 = 1.0, u1 = 2.0 * xi;
    double df = a[1 * st + i * ld];
    for (int j = 3; j <= n; ++j) {
        df += (j - 1) * u1 * a[(j - 1) * st + i * ld];
        double u2 = 2.0 * xi * u1 - u0;
        u0 = u1;
        u1 = u2;
    }
    return 2.0 * df / (r - l);
}

// Dense n x n solve with partial pivoting (restates LinearAlgebra `\` for the
// square collocation matrix of chebfit, cheby.jl:222).  A is row-major.
static void lu_solve(int n, double* A, double* bvec) {
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[r * n + c]) > std::fabs(A[piv * n + c])) piv = r;
        if (piv != c) {
            for (int k = 0; k < n; ++k) std::swap(A[c * n + k], A[piv * n + k]);
            std::swap(bvec[c], bvec[piv]);
        }
        for (int r = c + 1; r < n; ++r) {
            double f = A[r * n + c] / A[c * n + c];
            A[r * n + c] = f;
            for (int k = c + 1; k < n; ++k) A[r * n + k] -= f * A[c * n + k];
            bvec[r] -= f * bvec[c];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = bvec[r];
        for (int k = r + 1; k < n; ++k) s -= A[r * n + k] * bvec[k];
        bvec[r] = s / A[r * n + r];
    }
}

// chebfit (cheby.jl:211-227): out is [n][k+1] column-major (term fastest).
template <class F>
static void chebfit(F&& f, const BinaryIntervals& b, int n, double* out) {
    for (int i = 0; i <= b.k; ++i) {
        double l, r;
        b.interval(i, l, r);
        double A[PCL_MAX_ORDER * PCL_MAX_ORDER], fx[PCL_MAX_ORDER];
        for (int m = 0; m < n; ++m) {
            // chebnodes (cheby.jl:42-44)
            double x = (l + r) / 2 + (r - l) / 2 * std::cos((2 * m + 1) * pi / (2 * n));
            fx[m] = f(x);
            double xi = (2 * x - (l + r)) / (r - l);
            double t[PCL_MAX_ORDER];
            chebval(xi, n, t);
            for (int j = 0; j < n; ++j) A[m * n + j] = t[j];
        }
        lu_solve(n, A, fx);
        for (int j = 0; j < n; ++j) out[j + n * i] = fx[j];
    }
}

// --------------------------------------------------------------- speed ---
// speed(::Type{Electron}, eng) (electron.jl:47), positron.jl:34, photon.jl:46
static inline double speed(int species, double eng) {
    if (species == PCL_PHOTON) return c;
    double q = mc2 / (mc2 + eng);
    return c * std::sqrt(1 - q * q);
}

// ----------------------------------------------------------- totalcs -----
// moller.jl:40-57
static double totalcs_moller(int Z, double tcut, double eng) {
    double x = tcut / eng;
    if (x > 1) return 0.0;
    double g = 1 + eng / mc2;
    double b2 = (g * g - 1) / (g * g);
    double A = ((g - 1) * (g - 1) / (g * g)) * (0.5 - x) + 1 / x - 1 / (1 - x) -
               ((2 * g - 1) / (g * g)) * std::log((1 - x) / x);
    return jmax(0.0, 2 * pi * r_e * r_e * Z * A / (g - 1) / b2);
}

// relativistic_coulomb.jl:58-75
static double totalcs_coulomb(double Z, double K) {
    K += 1e-4 * eV;
    double a = 1.3413 * std::pow(Z, -1.0 / 3.0) * a_0;
    double g = 1 + K / (m_e * c * c);
    double p = std::sqrt(K * (K + 2 * (m_e * c * c))) / c;
    double beta = p / (g * m_e * c);
    double al = hbar * hbar / (4 * p * p * a * a);
    double b2 = beta * beta;
    return (pi * r_e * r_e * Z * Z / (b2 * b2 * g * g) *
            ((1 + al * b2) / (al * (1 + al)) + b2 * std::log(al / (1 + al))));
}

// rbeb.jl:127-150
static double rbeb_sigmaI(double T, double B, double U) {
    double t1 = T / mc2, b1 = B / mc2, u1 = U / mc2;
    double bt2 = 1 - 1 / ((1 + t1) * (1 + t1));
    double bb2 = 1 - 1 / ((1 + b1) * (1 + b1));
    double bu2 = 1 - 1 / ((1 + u1) * (1 + u1));
    double t = T / B;
    double al = alpha;
    double al4 = al * al * al * al;
    return (2 * a_0 * a_0 * pi * al4 / (b1 * (bb2 + bt2 + bu2)) *
            (1 - 1 / t + (b1 * b1 * (t - 1)) / (2 * (1 + t1) * (1 + t1)) -
             ((1 + 2 * t1) * std::log(t)) / ((1 + t) * (1 + t1) * (1 + t1)) -
             ((t * t - 1) * (bt2 - std::log(bt2) + std::log(2 * b1 * (1 - bt2)))) / (2 * t * t)));
}

// rbeb.jl:117-120 (Julia's `false * x` is a strong zero)
static double totalcs_rbeb(double B, double U, double N, double T) {
    if (!(T > B)) return 0.0;
    return N * rbeb_sigmaI(T, B, U);
}

// seltzer.jl:217-231 (linear interpolation of the tabulated cross section in log T)
static double totalcs_sb(const double* le, const double* tcs, int ne, double K) {
    double lK = std::log(K);
    // searchsortedlast
    int i = int(std::upper_bound(le, le + ne, lK) - le);  // 1-based index of last <= lK
    if (i == 0) return 0.0;
    if (i >= ne) return std::numeric_limits<double>::quiet_NaN();  // reference reads past the table
    double w = (le[i] - lK) / (le[i] - le[i - 1]);
    return w * tcs[i - 1] + (1 - w) * tcs[i];
}

// compton.jl:34-47
static double totalcs_kn(int Z, double eng) {
    double x = 2 * eng / mc2;
    double sigma = (2 * pi * r_e * r_e * (1 / x) *
                    ((1 - 4 / x - 8 / (x * x)) * std::log(1 + x) + 0.5 + 8 / x -
                     1 / ((1 + x) * (1 + x)) / 2));
    return Z * sigma;
}

// compton.jl:59-112 (G4KleinNishinaCompton empirical fit).  For Z <= 1 the
// reference uses an undefined `keV` (compton.jl:89); Geant4's 40 keV is used.
static double totalcs_compton(int Z, double eng) {
    const double barn = 1e-28;
    const double a = 20.0, b = 230.0, cc = 440.0;
    const double d1 = 2.7965e-1 * barn, d2 = -1.8300e-1 * barn, d3 = 6.7527 * barn,
                 d4 = -1.9798e+1 * barn;
    const double e1 = 1.9756e-5 * barn, e2 = -1.0205e-2 * barn, e3 = -7.3913e-2 * barn,
                 e4 = 2.7079e-2 * barn;
    const double f1 = -3.9178e-7 * barn, f2 = 6.8241e-5 * barn, f3 = 6.0480e-5 * barn,
                 f4 = 3.0274e-4 * barn;
    double Zd = Z;
    double p1Z = Zd * (d1 + e1 * Zd + f1 * Zd * Zd);
    double p2Z = Zd * (d2 + e2 * Zd + f2 * Zd * Zd);
    double p3Z = Zd * (d3 + e3 * Zd + f3 * Zd * Zd);
    double p4Z = Zd * (d4 + e4 * Zd + f4 * Zd * Zd);
    double T0 = 15.0e3 * eV;
    if (Z <= 1) T0 = 40.0e3 * eV;
    double X = std::max(eng, T0) / mc2;
    double sigma = p1Z * std::log(1 + 2 * X) / X +
                   (p2Z + p3Z * X + p4Z * X * X) / (1 + a * X + b * X * X + cc * X * X * X);
    if (eng < T0) {
        double dT0 = 1e3 * eV;
        X = (T0 + dT0) / mc2;
        double sigma1 = p1Z * std::log(1.0 + 2.0 * X) / X +
                        (p2Z + p3Z * X + p4Z * X * X) / (1.0 + a * X + b * X * X + cc * X * X * X);
        double c1 = -T0 * (sigma1 - sigma) / (sigma * dT0);
        double c2 = 0.150;
        if (Zd > 1.5) c2 = 0.375 - 0.0556 * std::log(Zd);
        double y = std::log(eng / T0);
        sigma *= std::exp(-y * (c1 + c2 * y));
    }
    return sigma;
}

// photo_electric.jl:54-58; left[n] J, coeffs [n][4] row-major (SI)
static double totalcs_pe(const double* left, const double* coeffs, int n, double eng) {
    int j = int(std::upper_bound(left, left + n, eng) - left);  // searchsortedlast
    if (j == 0) return 0.0;
    double s = 0.0;
    for (int i = 1; i <= 4; ++i) s += std::pow(eng, -double(i)) * coeffs[(j - 1) * 4 + (i - 1)];
    return s;
}

// bethe_heitler.jl:28-80
static double totalcs_bh(int Z, double eng) {
    if (eng < 2 * mc2) return 0.0;
    const double mb = 1e-34;
    const double lim = 1.5e6 * eV;
    const double a0 = 8.7842e+2 * mb, a1 = -1.9625e+3 * mb, a2 = 1.2949e+3 * mb,
                 a3 = -2.0028e+2 * mb, a4 = 1.2575e+1 * mb, a5 = -2.8333e-1 * mb;
    const double b0 = -1.0342e+1 * mb, b1 = 1.7692e+1 * mb, b2 = -8.2381 * mb,
                 b3 = 1.3063 * mb, b4 = -9.0815e-2 * mb, b5 = 2.3586e-3 * mb;
    const double c0 = -4.5263e+2 * mb, c1 = 1.1161e+3 * mb, c2 = -8.6749e+2 * mb,
                 c3 = 2.1773e+2 * mb, c4 = -2.0467e+1 * mb, c5 = 6.5372e-1 * mb;
    double eng1 = std::max(eng, lim);
    double x = std::log(eng1 / mc2);
    double x2 = x * x, x3 = x2 * x, x4 = x3 * x, x5 = x4 * x;
    double F1 = a0 + a1 * x + a2 * x2 + a3 * x3 + a4 * x4 + a5 * x5;
    double F2 = b0 + b1 * x + b2 * x2 + b3 * x3 + b4 * x4 + b5 * x5;
    double F3 = c0 + c1 * x + c2 * x2 + c3 * x3 + c4 * x4 + c5 * x5;
    double Zd = Z;
    double sigma = (Zd + 1) * (F1 * Zd + F2 * Zd * Zd + F3);
    if (eng < lim) {
        double q = (eng - 2 * mc2) / (lim - 2 * mc2);
        sigma = sigma * q * q;
    }
    return sigma;
}

// bhaba.jl:84-91
static inline void bhabha_bs(double y, double& B1, double& B2, double& B3, double& B4) {
    double u = 1 - 2 * y;
    B1 = 2 - y * y;
    B2 = u * (3 + y * y);
    B3 = u * u + u * u * u;
    B4 = u * u * u;
}

// bhaba.jl:35-49
static double totalcs_bhabha(int Z, double tcut, double eng) {
    double g = 1 + eng / mc2;
    double beta = std::sqrt((g * g - 1) / (g * g));
    double x = tcut / eng;
    double y = 1 / (g + 1);
    double B1, B2, B3, B4;
    bhabha_bs(y, B1, B2, B3, B4);
    double A = (1 / x - 1) / (beta * beta) + B1 * std::log(x) + B2 * (1 - x) -
               B3 * (1 - x * x) / 2 + B4 * (1 - x * x * x) / 3;
    return jmax(0.0, 2 * pi * r_e * r_e * Z * A / (g - 1));
}

// anihilation.jl:25-32
static double totalcs_annihilation(double Z, double eng) {
    double g = 1 + eng / mc2;
    double s = std::sqrt(g * g - 1);
    double A = ((g * g + 4 * g + 1) / (g * g - 1) * std::log(g + s) - (g + 3) / s) / (g + 1);
    return Z * pi * r_e * r_e * A;
}

static double proc_Z(const pcl_process& p) {
    return (p.Z == 0) ? p.param[0] : double(p.Z);
}

static double totalcs(const pcl_process& p, double E) {
    switch (p.kind) {
        case PCL_PROC_MOLLER: return totalcs_moller(p.Z, p.param[0], E);
        case PCL_PROC_RBEB: return totalcs_rbeb(p.param[0], p.param[1], p.param[2], E);
        case PCL_PROC_SELTZER_BERGER: return totalcs_sb(p.aux0, p.aux1, p.naux, E);
        case PCL_PROC_REL_COULOMB: return totalcs_coulomb(proc_Z(p), E);
        case PCL_PROC_COMPTON: return totalcs_compton(p.Z, E);
        case PCL_PROC_KN_COMPTON: return totalcs_kn(p.Z, E);
        case PCL_PROC_PHOTOELECTRIC: return totalcs_pe(p.aux0, p.aux1, p.naux, E);
        case PCL_PROC_BETHE_HEITLER: return totalcs_bh(p.Z, E);
        case PCL_PROC_BHABHA: return totalcs_bhabha(p.Z, p.param[0], E);
        case PCL_PROC_ANNIHILATION: return totalcs_annihilation(proc_Z(p), E);
        default: return std::numeric_limits<double>::quiet_NaN();
    }
}

static bool proc_valid_for(const pcl_process& p, int species) {
    switch (p.kind) {
        case PCL_PROC_MOLLER:
        case PCL_PROC_RBEB:
        case PCL_PROC_SELTZER_BERGER:
            return species == PCL_ELECTRON;
        case PCL_PROC_REL_COULOMB:
            return species == PCL_ELECTRON || species == PCL_POSITRON;
        case PCL_PROC_COMPTON:
        case PCL_PROC_KN_COMPTON:
        case PCL_PROC_PHOTOELECTRIC:
        case PCL_PROC_BETHE_HEITLER:
            return species == PCL_PHOTON;
        case PCL_PROC_BHABHA:
        case PCL_PROC_ANNIHILATION:
            return species == PCL_POSITRON;
        default:
            return false;
    }
}

// ------------------------------------------------ Seltzer-Berger build ----
// Piecewise-linear interpolant through (x[m], p[m]) and its exact antiderivative
// C(x) = int_{x0}^{x} itp: this is what BSplineKit.interpolate(x, p,
// BSplineOrder(2)) and integral(...) represent (seltzer.jl:164-173).
struct LinCum {
    const double* x;
    const double* p;
    int n;
    std::vector<double> C;  // C at the data points
    LinCum(const double* x_, const double* p_, int n_) : x(x_), p(p_), n(n_), C(n_) {
        C[0] = 0.0;
        for (int m = 0; m + 1 < n; ++m) C[m + 1] = C[m] + 0.5 * (p[m] + p[m + 1]) * (x[m + 1] - x[m]);
    }
    int seg(double v) const {
        int m = int(std::upper_bound(x, x + n, v) - x) - 1;
        if (m < 0) m = 0;
        if (m > n - 2) m = n - 2;
        return m;
    }
    double itp(double v) const {
        int m = seg(v);
        double h = x[m + 1] - x[m];
        double s = (v - x[m]) / h;
        return p[m] + (p[m + 1] - p[m]) * s;
    }
    double cum(double v) const {
        int m = seg(v);
        double h = x[m + 1] - x[m];
        double d = v - x[m];
        return C[m] + p[m] * d + 0.5 * (p[m + 1] - p[m]) * d * d / h;
    }
};

// findcumvalues! (seltzer.jl:163-192)
static bool findcumvalues(const double* x, const double* p, int n, const double* pcum, int ncum,
                          double xmin, double xmax, double* out, double rtol = 1e-6) {
    for (int m = 0; m < n; ++m)
        if (!(p[m] > 0)) return false;  // @assert all(itp.(knots(itp)) .> 0)
    LinCum L(x, p, n);
    double cum0 = L.cum(std::max(xmin, x[0]));
    double cum1 = L.cum(std::min(xmax, x[n - 1]));
    double span = cum1 - cum0;
    // knots of the antiderivative: the data points with the end points repeated
    std::vector<double> knt;
    knt.push_back(x[0]);
    knt.push_back(x[0]);
    for (int m = 0; m < n; ++m) knt.push_back(x[m]);
    knt.push_back(x[n - 1]);
    knt.push_back(x[n - 1]);
    std::vector<double> fk(knt.size());
    for (size_t m = 0; m < knt.size(); ++m) fk[m] = (L.cum(knt[m]) - cum0) / span;
    for (int i = 0; i < ncum; ++i) {
        // searchsortedlast(fknt, pcum[i]) -> 1-based j
        int j = int(std::upper_bound(fk.begin(), fk.end(), pcum[i]) - fk.begin());
        int ja = std::max(1, j), jb = std::min(int(knt.size()), j + 1);
        double xs = 0.5 * (knt[ja - 1] + knt[jb - 1]);
        double dx = std::numeric_limits<double>::infinity();
        for (int it = 0; it < 200 && std::fabs(dx / xs) > rtol; ++it) {
            double f = (L.cum(xs) - cum0) / span;
            double df = L.itp(xs) / span;
            dx = (f - pcum[i]) / df;
            xs = xs - dx;
        }
        out[i] = xs;
    }
    return true;
}

// scaledcs (seltzer.jl:201-211)
static double scaledcs(const double* logk, const double* s, int n, double lmin, double lmax) {
    LinCum L(logk, s, n);
    return L.cum(std::min(lmax, logk[n - 1])) - L.cum(std::max(lmin, logk[0]));
}

// LinRange(start, stop, len)[i] for 0-based i (Julia's lerp form)
static inline double linrange(double a, double b, int len, int i) {
    double d = double(len - 1);
    return (a * (d - i) + b * i) / d;
}

}  // namespace pcl

using namespace pcl;

// ------------------------------------------------------------- C ABI ------
extern "C" int pcl_sb_build(int Z, int nx, int ny, const double* x, const double* y,
                            const double* value, int ncum, double gamma_min, double gamma_max,
                            double energy_scale, double* log_energy, double* totalcs_out,
                            double* data) {
    if (nx < 2 || ny < 2 || ncum < 2 || !x || !y || !value || !log_energy || !totalcs_out || !data)
        return PCL_ERR_INVALID;
    std::vector<double> logk(nx), pcum(ncum);
    for (int m = 0; m < nx; ++m) logk[m] = std::log(x[m]);
    for (int i = 0; i < ncum; ++i) pcum[i] = linrange(0.0, 1.0, ncum, i);
    for (int i = 0; i < ny; ++i) log_energy[i] = std::log(std::exp(y[i]) * energy_scale);
    for (int i = 0; i < ny; ++i) {
        double T1 = std::exp(log_energy[i]);
        double q = 1 + T1 / si::mc2;
        double beta = std::sqrt(1 - 1 / (q * q));
        const double* row = value + size_t(i) * nx;
        double lmin = std::log(gamma_min / T1), lmax = std::log(gamma_max / T1);
        if (!findcumvalues(logk.data(), row, nx, pcum.data(), ncum, lmin, lmax,
                           data + size_t(i) * ncum))
            return PCL_ERR_NUMERIC;
        totalcs_out[i] = (double(Z) * Z / (beta * beta)) * 1e-31 *
                         scaledcs(logk.data(), row, nx, lmin, lmax);
    }
    return PCL_OK;
}

extern "C" int pcl_totalcs(const pcl_process* proc, int64_t n, const double* energy, double* out) {
    if (!proc || (n > 0 && (!energy || !out))) return PCL_ERR_INVALID;
    if (proc->kind == PCL_PROC_SELTZER_BERGER && (!proc->aux0 || !proc->aux1 || proc->naux < 2))
        return PCL_ERR_INVALID;
    if (proc->kind == PCL_PROC_PHOTOELECTRIC && (!proc->aux0 || !proc->aux1 || proc->naux < 1))
        return PCL_ERR_INVALID;
    if (proc->kind < PCL_PROC_MOLLER || proc->kind > PCL_PROC_ANNIHILATION) return PCL_ERR_UNSUPPORTED;
    for (int64_t i = 0; i < n; ++i) out[i] = totalcs(*proc, energy[i]);
    return PCL_OK;
}

extern "C" int pcl_build_collision_table(int species, int nproc, const pcl_process* procs,
                                         double Fdt, double safety, int nintervals, int order,
                                         double max_energy, double* rate, double* ratebound,
                                         int32_t* perm) {
    if (species < 0 || species >= PCL_NSPECIES) return PCL_ERR_INVALID;
    if (nproc < 0 || nproc > PCL_MAX_PROC || order < 1 || order > PCL_MAX_ORDER ||
        nintervals < 1 || nintervals > PCL_MAX_INTERVALS || !(max_energy > 0))
        return PCL_ERR_INVALID;
    if (nproc > 0 && (!procs || !rate || !perm)) return PCL_ERR_INVALID;
    if (!ratebound) return PCL_ERR_INVALID;
    for (int j = 0; j < nproc; ++j) {
        if (!proc_valid_for(procs[j], species)) return PCL_ERR_UNSUPPORTED;
        if (procs[j].kind == PCL_PROC_SELTZER_BERGER && (!procs[j].aux0 || !procs[j].aux1))
            return PCL_ERR_INVALID;
        if (procs[j].kind == PCL_PROC_PHOTOELECTRIC && (!procs[j].aux0 || !procs[j].aux1))
            return PCL_ERR_INVALID;
    }
    BinaryIntervals b{nintervals, max_energy};
    const int nI = nintervals + 1;
    // a[k, j, i] column-major (collision_table.jl:128), unsorted for now
    std::vector<double> a(size_t(order) * nproc * nI);
    for (int j = 0; j < nproc; ++j) {
        const pcl_process& P = procs[j];
        std::vector<double> fit(size_t(order) * nI);
        chebfit([&](double eng) { return P.coef * speed(species, eng) * totalcs(P, eng); }, b, order,
                fit.data());
        for (int i = 0; i < nI; ++i)
            for (int k = 0; k < order; ++k) a[k + order * (j + nproc * i)] = fit[k + order * i];
    }
    // compratebound (collision_table.jl:152-167)
    {
        std::vector<double> rb(size_t(order) * nI);
        const int st = 1, ld = order * nproc;
        chebfit(
            [&](double eng) {
                if (nproc == 0) return 0.0;
                double df = 0.0, f = 0.0;
                for (int j = 0; j < nproc; ++j) df += chebdiff(eng, b, a.data() + order * j, order, st, ld);
                for (int j = 0; j < nproc; ++j) f += chebeval(eng, b, a.data() + order * j, order, st, ld);
                double g = (species == PCL_PHOTON) ? 0.0 : 1 + eng / (si::m_e * si::c * si::c);
                return f + g * g * g * speed(species, eng) * Fdt * std::fabs(df) * safety;
            },
            b, order, rb.data());
        std::memcpy(ratebound, rb.data(), sizeof(double) * rb.size());
    }
    if (nproc == 0) return PCL_OK;
    // Order processes by their peak rate over LogLinRange(log(1e-2 eV), log(0.9999 max), 1e5),
    // descending (collision_table.jl:138-145).  Julia's maximum propagates NaN and
    // sortperm(rev=true) puts NaN keys first; ties keep ascending index.
    const int NG = 100000;
    const double L1 = std::log(1e-2 * si::eV), L2 = std::log(0.9999 * max_energy);
    const double x0 = std::exp(L1);
    std::vector<double> key(nproc, -std::numeric_limits<double>::infinity());
    std::vector<char> isnan_key(nproc, 0);
    for (int g = 0; g < NG; ++g) {
        double eng = std::exp(linrange(L1, L2, NG, g)) - x0;
        double v1 = speed(species, eng);
        for (int j = 0; j < nproc; ++j) {
            double val = procs[j].coef * (totalcs(procs[j], eng) * v1);
            if (std::isnan(val)) isnan_key[j] = 1;
            else if (val > key[j]) key[j] = val;
        }
    }
    std::vector<int> p(nproc);
    std::iota(p.begin(), p.end(), 0);
    std::stable_sort(p.begin(), p.end(), [&](int u, int v) {
        if (isnan_key[u] != isnan_key[v]) return isnan_key[u] > isnan_key[v];
        if (isnan_key[u]) return false;
        return key[u] > key[v];
    });
    for (int jj = 0; jj < nproc; ++jj) {
        perm[jj] = p[jj];
        for (int i = 0; i < nI; ++i)
            for (int k = 0; k < order; ++k)
                rate[k + order * (jj + nproc * i)] = a[k + order * (p[jj] + nproc * i)];
    }
    return PCL_OK;
}

extern "C" int pcl_ratebound_split(int species, int order, int nproc, int nintervals, double xmax,
                                   const double* rate, double safety, double* A, double* B) {
    if (species < 0 || species >= PCL_NSPECIES || order < 1 || order > PCL_MAX_ORDER || nproc < 0 ||
        nproc > PCL_MAX_PROC || nintervals < 1 || nintervals > PCL_MAX_INTERVALS || !(xmax > 0) || !A || !B ||
        (nproc > 0 && !rate))
        return PCL_ERR_INVALID;
    BinaryIntervals b{nintervals, xmax};
    const int nI = nintervals + 1;
    for (int i = 0; i < nI; ++i)
        for (int k = 0; k < order; ++k) {
            double s = 0.0;
            for (int j = 0; j < nproc; ++j) s += rate[k + order * (j + nproc * i)];
            A[k + order * i] = s;
        }
    const int st = 1, ld = order * nproc;
    chebfit(
        [&](double eng) {
            if (nproc == 0 || species == PCL_PHOTON) return 0.0;
            double df = 0.0;
            for (int j = 0; j < nproc; ++j) df += chebdiff(eng, b, rate + order * j, order, st, ld);
            double g = 1 + eng / (si::m_e * si::c * si::c);
            return g * g * g * speed(species, eng) * std::fabs(df) * safety;
        },
        b, order, B);
    return PCL_OK;
}

// ---- continuum losses (continuum.jl:63-139) ----
namespace pcl {
static void x0x1(double C, double& x0, double& x1) {
    if (C < 10) { x0 = 1.6; x1 = 4.0; }
    else if (C < 10.5) { x0 = 1.7; x1 = 4.0; }
    else if (C < 11.0) { x0 = 1.8; x1 = 4.0; }
    else if (C < 11.5) { x0 = 1.9; x1 = 4.0; }
    else if (C < 12.25) { x0 = 2.0; x1 = 4.0; }
    else if (C < 13.804) { x0 = 2.0; x1 = 5.0; }
    else { x0 = 0.326 * C - 2.5; x1 = 5.0; }
}

static double energy_loss(double nel, double I, double Tcut, bool positron, double eng) {
    const double mc2_ = si::mc2;
    double tau = eng / mc2_;
    double tauc = Tcut / mc2_;
    double taumax = positron ? tau : tau / 2;
    double g = 1 + tau;
    double b2 = 1 - 1 / (g * g);
    double tup = std::min(tauc, taumax);
    double F;
    if (positron) {
        double y = 1 / (2 + tau);
        F = (std::log(tau * tup) -
             (tup * tup / tau) * (tau * 2 * tup - 3 * tup * tup * y / 2 -
                                  (tup - tup * tup * tup / 3) * y * y -
                                  (tup * tup / 2 - tau * tup * tup * tup / 3 + tup * tup * tup * tup / 4) *
                                      y * y * y));
    } else {
        F = (-1 - b2 + std::log((tau - tup) * tup) + tau / (tau - tup) +
             (tup * tup / 2 + (2 * tau + 1) * std::log(1 - tup / tau)) / (g * g));
    }
    const double ln10 = std::log(10.0);
    double x = std::log(g * g * b2) / ln10 / 2;
    double hnup = si::hbar * si::c * std::sqrt(4 * si::pi * nel * si::r_e);
    double C = 1 + 2 * std::log(I / hnup);
    double xa = C / ln10 / 2;
    const double m = 3;
    double x0, x1;
    x0x1(C, x0, x1);
    double a = 2 * ln10 * (xa - x) / std::pow(x1 - x0, m);
    double delta;
    if (x < x0) delta = 0.0;
    else if (x < x1) delta = 2 * ln10 * x - C + a * std::pow(x1 - x, m);
    else delta = 2 * ln10 * x - C;
    return (2 * si::pi * si::r_e * si::r_e * mc2_ * nel / b2) *
           (std::log((2 * (g + 1)) / ((I / mc2_) * (I / mc2_))) + F - delta);
}
}  // namespace pcl

extern "C" int pcl_build_continuum_loss(double nel, double I, double Tcut, double Tmax, int n,
                                        int* k_out, double* xmax_out, double* ec, double* pc,
                                        int cap) {
    if (!(nel > 0) || !(I > 0) || !(Tcut > 0) || !(Tmax > Tcut) || n < 1 || n > PCL_MAX_ORDER ||
        !k_out || !xmax_out || !ec || !pc)
        return PCL_ERR_INVALID;
    int k = int(std::ceil(std::log2(Tmax / Tcut)));
    if (k < 1 || k > PCL_MAX_INTERVALS) return PCL_ERR_INVALID;
    if (cap < n * (k + 1)) return PCL_ERR_INVALID;
    BinaryIntervals b{k, std::ldexp(1.0, k) * Tcut};
    chebfit([&](double x) { return energy_loss(nel, I, Tcut, false, x); }, b, n, ec);
    chebfit([&](double x) { return energy_loss(nel, I, Tcut, true, x); }, b, n, pc);
    *k_out = k;
    *xmax_out = b.xmax;
    return PCL_OK;
}
