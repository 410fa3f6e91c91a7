"""Independent numpy restatement of the reference's table-building init path
(test infrastructure only), used to check the library's C++ builders.

  totalcs of each process ........ moller.jl:40-57, relativistic_coulomb.jl:58-75,
                                   seltzer.jl:217-231, rbeb.jl:117-150, compton.jl:34-112,
                                   photo_electric.jl:54-58, bethe_heitler.jl:28-80,
                                   bhaba.jl:35-49, anihilation.jl:25-32
  chebfit / chebnodes / interval . cheby.jl:15-44, 211-227 (LinearAlgebra `\\` -> numpy.linalg.solve)
  compratebound / sort ........... collision_table.jl:115-167
  SeltzerBerger builder .......... seltzer.jl:23-64, 163-211 (BSplineKit order 2 -> linear
                                   interpolant, exact quadratic antiderivative, Newton)
  energy_loss .................... continuum.jl:63-139
PARITY UNPINNED: checked against the reference by reading only.
"""
from __future__ import annotations

import math

import numpy as np

c = 299792458.0
eV = e = 1.6021766208e-19
m_e = 9.10938356e-31
hbar = 1.0545718001391127e-34
alpha = 0.0072973525664
eps0 = 8.854187817620389e-12
mc2 = m_e * c ** 2
r_e = e ** 2 / (m_e * c ** 2) / (4 * math.pi * eps0)
a_0 = hbar / (m_e * c * alpha)


def speed(photon: bool, E):
    if photon:
        return c * np.ones_like(E)
    return c * np.sqrt(1 - (mc2 / (mc2 + E)) ** 2)


def jmax0(A):
    """Julia's max(0, A) (NaN propagates)."""
    return np.where(np.isnan(A), np.nan, np.maximum(0.0, A))


def cs_moller(Z, tcut, E):
    with np.errstate(all="ignore"):
        x = tcut / E
        g = 1 + E / mc2
        b2 = (g ** 2 - 1) / g ** 2
        A = ((g - 1) ** 2 / g ** 2) * (0.5 - x) + 1 / x - 1 / (1 - x) - ((2 * g - 1) / g ** 2) * np.log((1 - x) / x)
        out = jmax0(2 * np.pi * r_e ** 2 * Z * A / (g - 1) / b2)
        return np.where(x > 1, 0.0, out)


def cs_coulomb(Z, K):
    K = K + 1e-4 * eV
    a = 1.3413 * Z ** (-1 / 3) * a_0
    g = 1 + K / (m_e * c ** 2)
    p = np.sqrt(K * (K + 2 * (m_e * c ** 2))) / c
    beta = p / (g * m_e * c)
    al = hbar ** 2 / (4 * p ** 2 * a ** 2)
    return (np.pi * r_e ** 2 * Z ** 2 / (beta ** 4 * g ** 2) *
            ((1 + al * beta ** 2) / (al * (1 + al)) + beta ** 2 * np.log(al / (1 + al))))


def cs_sb(le, tcs, K):
    lK = np.log(K)
    i = np.searchsorted(le, lK, side="right")  # searchsortedlast (1-based)
    out = np.zeros_like(K)
    ok = (i > 0) & (i < len(le))
    ii = i[ok]
    w = (le[ii] - lK[ok]) / (le[ii] - le[ii - 1])
    out[ok] = w * tcs[ii - 1] + (1 - w) * tcs[ii]
    return out


def cs_compton(Z, E):
    barn = 1e-28
    a, b, cc = 20.0, 230.0, 440.0
    d = np.array([2.7965e-1, -1.8300e-1, 6.7527, -1.9798e+1]) * barn
    ee = np.array([1.9756e-5, -1.0205e-2, -7.3913e-2, 2.7079e-2]) * barn
    f = np.array([-3.9178e-7, 6.8241e-5, 6.0480e-5, 3.0274e-4]) * barn
    p = Z * (d + ee * Z + f * Z ** 2)
    T0 = 15.0e3 * eV if Z > 1 else 40.0e3 * eV

    def sig(X):
        return p[0] * np.log(1 + 2 * X) / X + (p[1] + p[2] * X + p[3] * X ** 2) / (1 + a * X + b * X ** 2 + cc * X ** 3)
    X = np.maximum(E, T0) / mc2
    sigma = sig(X)
    low = E < T0
    if np.any(low):
        X1 = (T0 + 1e3 * eV) / mc2
        s1 = sig(X1)
        c1 = -T0 * (s1 - sigma[low]) / (sigma[low] * 1e3 * eV)
        c2 = 0.375 - 0.0556 * np.log(Z) if Z > 1.5 else 0.15
        with np.errstate(all="ignore"):
            y = np.log(E[low] / T0)
            sigma[low] = sigma[low] * np.exp(-y * (c1 + c2 * y))
    return sigma


def cs_pe(left, coeffs, E):
    j = np.searchsorted(left, E, side="right")
    out = np.zeros_like(E)
    ok = j > 0
    jj = j[ok] - 1
    for i in range(1, 5):
        out[ok] += E[ok] ** (-i) * coeffs[jj, i - 1]
    return out


def cs_bh(Z, E):
    mb = 1e-34
    lim = 1.5e6 * eV
    A = np.array([8.7842e+2, -1.9625e+3, 1.2949e+3, -2.0028e+2, 1.2575e+1, -2.8333e-1]) * mb
    B = np.array([-1.0342e+1, 1.7692e+1, -8.2381, 1.3063, -9.0815e-2, 2.3586e-3]) * mb
    Cc = np.array([-4.5263e+2, 1.1161e+3, -8.6749e+2, 2.1773e+2, -2.0467e+1, 6.5372e-1]) * mb
    x = np.log(np.maximum(E, lim) / mc2)
    xp = np.stack([x ** k for k in range(6)])
    F1, F2, F3 = A @ xp, B @ xp, Cc @ xp
    sigma = (Z + 1) * (F1 * Z + F2 * Z * Z + F3)
    sigma = np.where(E < lim, sigma * ((E - 2 * mc2) / (lim - 2 * mc2)) ** 2, sigma)
    return np.where(E < 2 * mc2, 0.0, sigma)


def cs_bhabha(Z, tcut, E):
    with np.errstate(all="ignore"):
        g = 1 + E / mc2
        beta = np.sqrt((g ** 2 - 1) / g ** 2)
        x = tcut / E
        y = 1 / (g + 1)
        B1, B2, B3, B4 = 2 - y ** 2, (1 - 2 * y) * (3 + y ** 2), (1 - 2 * y) ** 2 + (1 - 2 * y) ** 3, (1 - 2 * y) ** 3
        A = (1 / x - 1) / beta ** 2 + B1 * np.log(x) + B2 * (1 - x) - B3 * (1 - x ** 2) / 2 + B4 * (1 - x ** 3) / 3
        return jmax0(2 * np.pi * r_e ** 2 * Z * A / (g - 1))


def cs_annihilation(Z, E):
    with np.errstate(all="ignore"):
        g = 1 + E / mc2
        A = ((g ** 2 + 4 * g + 1) / (g ** 2 - 1) * np.log(g + np.sqrt(g ** 2 - 1)) - (g + 3) / np.sqrt(g ** 2 - 1)) / (g + 1)
        return Z * np.pi * r_e ** 2 * A


def totalcs(proc, E):
    """proc: a particulator_gb300 process object (fields read only)."""
    n = type(proc).__name__
    E = np.asarray(E, dtype=float)
    if n == "Moller":
        return cs_moller(proc.Z, proc.tcut, E)
    if n == "RelativisticCoulomb":
        return cs_coulomb(float(proc.Z), E)
    if n == "SeltzerBerger":
        return cs_sb(proc.log_energy, proc.totalcs, E)
    if n in ("Compton",):
        return cs_compton(proc.Z, E)
    if n == "PhotoElectric":
        return cs_pe(proc.left_energy, proc.coeffs, E)
    if n == "BetheHeitler":
        return cs_bh(proc.Z, E)
    if n == "Bhaba":
        return cs_bhabha(proc.Z, proc.tcut, E)
    if n == "PositronAnihilation":
        return cs_annihilation(float(proc.Z), E)
    raise NotImplementedError(n)


def interval(k, xmax, i):
    if i == 0:
        return 0.0, interval(k, xmax, 1)[0]
    l = 2.0 ** (i - k - 1)
    return l * xmax, 2 * l * xmax


def chebval(xi, n):
    t = [np.ones_like(xi), xi]
    while len(t) < n:
        t.append(2 * xi * t[-1] - t[-2])
    return np.stack(t[:n], axis=-1)


def chebfit(f, k, xmax, n):
    """a[n, k+1]"""
    a = np.zeros((n, k + 1))
    for i in range(k + 1):
        l, r = interval(k, xmax, i)
        x = np.array([(l + r) / 2 + (r - l) / 2 * math.cos((2 * m + 1) * math.pi / (2 * n)) for m in range(n)])
        xi = (2 * x - (l + r)) / (r - l)
        a[:, i] = np.linalg.solve(chebval(xi, n), f(x))
    return a


def precheb(x, k, xmax, n):
    x1 = np.asarray(x, dtype=float) / xmax
    s, l = np.frexp(x1)
    i = np.where(x1 == 0, 0, l + k)
    xi = np.where(i > 0, 4 * s - 3, 2.0 ** (k + 1) * x1 - 1)
    i = np.where(i > 0, i, 0)
    return i, chebval(xi, n)


def chebeval(x, k, xmax, a):
    i, t = precheb(x, k, xmax, a.shape[0])
    return np.sum(a[:, i].T * t, axis=-1)


def chebdiff(x, k, xmax, a):
    n = a.shape[0]
    i, t = precheb(x, k, xmax, n)
    xi = t[..., 1] if n > 1 else np.zeros_like(np.asarray(x, float))
    l = np.array([interval(k, xmax, int(q))[0] for q in np.atleast_1d(i)])
    r = np.array([interval(k, xmax, int(q))[1] for q in np.atleast_1d(i)])
    u0, u1 = np.ones_like(xi), 2 * xi
    df = a[1, i]
    for j in range(3, n + 1):
        df = df + (j - 1) * u1 * a[j - 1, i]
        u0, u1 = u1, 2 * xi * u1 - u0
    return 2 * df / (r - l)


def collision_table(processes, particle_is_photon, lepton, Fdt, safety=1.1, nintervals=32, order=3,
                    max_energy=1e3 * eV * 2 ** 18):
    """Unsorted fits a[order, nproc, k+1], the rate bound rb[order, k+1] and the
    sort permutation of collision_table_from_processes."""
    k = nintervals
    n = len(processes)
    a = np.zeros((order, n, k + 1))
    for j, (cf, p) in enumerate(processes):
        a[:, j, :] = chebfit(lambda E: cf * speed(particle_is_photon, E) * totalcs(p, E), k, max_energy, order)

    def rbf(E):
        if n == 0:
            return np.zeros_like(E)
        df = sum(chebdiff(E, k, max_energy, a[:, j, :]) for j in range(n))
        f = sum(chebeval(E, k, max_energy, a[:, j, :]) for j in range(n))
        g = (1 + E / (m_e * c ** 2)) if lepton else 0.0
        return f + g ** 3 * speed(particle_is_photon, E) * Fdt * np.abs(df) * safety
    rb = chebfit(rbf, k, max_energy, order)
    L1, L2 = math.log(1e-2 * eV), math.log(0.9999 * max_energy)
    NG = 100000
    L = (L1 * (NG - 1 - np.arange(NG)) + L2 * np.arange(NG)) / (NG - 1)
    eng = np.exp(L) - math.exp(L1)
    v1 = speed(particle_is_photon, eng)
    keys = []
    for cf, p in processes:
        with np.errstate(all="ignore"):
            vals = cf * (totalcs(p, eng) * v1)
        keys.append(np.nan if np.any(np.isnan(vals)) else np.max(vals))
    order_idx = sorted(range(n), key=lambda j: (0 if np.isnan(keys[j]) else 1, -(keys[j] if not np.isnan(keys[j]) else 0), j))
    return a, rb, np.array(order_idx)


def sb_build(Z, x, y, value, ncum=1000, gamma_min=1e2 * eV, gamma_max=5e7 * eV, energy_scale=1e6 * eV):
    """SeltzerBerger(d, Z; ...) -> (log_energy, totalcs, data[ncum, ne])."""
    le = np.log(np.exp(y) * energy_scale)
    logk = np.log(x)
    pcum = np.linspace(0.0, 1.0, ncum)
    data = np.zeros((ncum, len(y)))
    tcs = np.zeros(len(y))
    for i in range(len(y)):
        T1 = math.exp(le[i])
        beta = math.sqrt(1 - 1 / (1 + T1 / mc2) ** 2)
        p = value[i]
        h = np.diff(logk)
        Cp = np.concatenate([[0.0], np.cumsum(0.5 * (p[1:] + p[:-1]) * h)])

        def cum(v):
            m = np.clip(np.searchsorted(logk, v, side="right") - 1, 0, len(logk) - 2)
            d = v - logk[m]
            return Cp[m] + p[m] * d + 0.5 * (p[m + 1] - p[m]) * d * d / h[m]

        def itp(v):
            m = np.clip(np.searchsorted(logk, v, side="right") - 1, 0, len(logk) - 2)
            return p[m] + (p[m + 1] - p[m]) * (v - logk[m]) / h[m]
        lmin, lmax = math.log(gamma_min / T1), math.log(gamma_max / T1)
        c0 = cum(max(lmin, logk[0]))
        c1 = cum(min(lmax, logk[-1]))
        knt = np.concatenate([[logk[0]] * 2, logk, [logk[-1]] * 2])
        fk = (cum(knt) - c0) / (c1 - c0)
        for q, pc in enumerate(pcum):
            j = int(np.searchsorted(fk, pc, side="right"))
            ja, jb = max(1, j), min(len(knt), j + 1)
            xs = 0.5 * (knt[ja - 1] + knt[jb - 1])
            dx = math.inf
            it = 0
            while it < 200 and (xs == 0 and dx != 0 or xs != 0 and abs(dx / xs) > 1e-6):
                f = (cum(xs) - c0) / (c1 - c0)
                df = itp(xs) / (c1 - c0)
                dx = (f - pc) / df
                xs = xs - dx
                it += 1
                if xs == 0 and dx == 0:
                    break
            data[q, i] = xs
        tcs[i] = (Z ** 2 / beta ** 2) * 1e-31 * (c1 - c0)
    return le, tcs, data


def energy_loss(nel, I, Tcut, positron, E):
    tau = E / mc2
    tauc = Tcut / mc2
    tmax = tau if positron else tau / 2
    g = 1 + tau
    b2 = 1 - 1 / g ** 2
    tup = np.minimum(tauc, tmax)
    with np.errstate(all="ignore"):
        if positron:
            y = 1 / (2 + tau)
            F = (np.log(tau * tup) - (tup ** 2 / tau) * (tau * 2 * tup - 3 * tup ** 2 * y / 2 - (tup - tup ** 3 / 3) * y ** 2
                                                        - (tup ** 2 / 2 - tau * tup ** 3 / 3 + tup ** 4 / 4) * y ** 3))
        else:
            F = (-1 - b2 + np.log((tau - tup) * tup) + tau / (tau - tup)
                 + (tup ** 2 / 2 + (2 * tau + 1) * np.log(1 - tup / tau)) / g ** 2)
    ln10 = math.log(10)
    x = np.log(g ** 2 * b2) / ln10 / 2
    hnup = hbar * c * math.sqrt(4 * math.pi * nel * r_e)
    C = 1 + 2 * math.log(I / hnup)
    xa = C / ln10 / 2
    x0, x1 = ((1.6, 4.0) if C < 10 else (1.7, 4.0) if C < 10.5 else (1.8, 4.0) if C < 11 else (1.9, 4.0) if C < 11.5
              else (2.0, 4.0) if C < 12.25 else (2.0, 5.0) if C < 13.804 else (0.326 * C - 2.5, 5.0))
    a = 2 * ln10 * (xa - x) / (x1 - x0) ** 3
    delta = np.where(x < x0, 0.0, np.where(x < x1, 2 * ln10 * x - C + a * (x1 - x) ** 3, 2 * ln10 * x - C))
    return (2 * math.pi * r_e ** 2 * mc2 * nel / b2) * (np.log((2 * (g + 1)) / (I / mc2) ** 2) + F - delta)
