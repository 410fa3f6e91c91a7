"""Host table builders (C++ in the library) against the independent numpy
restatement in oracle/tables_ref.py, plus properties the reference relies on."""
import numpy as np
import pytest

from oracle import tables_ref as ref


@pytest.fixture(scope="module")
def comp(pcl):
    return pcl.workloads.air_composition()


def _grid():
    return np.exp(np.linspace(np.log(1.5e3), np.log(2.5e8), 400)) * ref.eV


def test_totalcs_every_process(pcl, comp):
    E = _grid()
    procs = (pcl.workloads.electron_processes(comp) + pcl.workloads.photon_processes(comp)
             + pcl.workloads.positron_processes(comp))
    for _, p in procs:
        got = pcl.totalcs(p, E)
        want = ref.totalcs(p, E)
        both = np.isfinite(want)
        assert np.array_equal(np.isfinite(got), both), type(p).__name__
        np.testing.assert_allclose(got[both], want[both], rtol=1e-11, atol=1e-40, err_msg=type(p).__name__)


def test_known_cross_section_values(pcl):
    """Published values the formulas must reproduce: Klein-Nishina per electron at
    1 MeV is 0.2112 b (L&L 86); BH vanishes below 2 m c^2."""
    kn = pcl.KleinNishinaCompton(1)
    assert abs(pcl.totalcs(kn, 1e6 * ref.eV) / 1e-28 - 0.2112) < 5e-4
    assert pcl.totalcs(pcl.BetheHeitler(7), 1.0e6 * ref.eV) == 0.0
    assert pcl.totalcs(pcl.Moller(7, 1e4 * ref.eV), 1.5e4 * ref.eV) == 0.0  # x = tcut/E > 1/2 -> max(0, <0)


def test_sb_table_matches_restatement(pcl):
    sb = pcl.SeltzerBerger(7)
    _, x, y, value = pcl.data.read_g4_2dvector(pcl.data.sb_path(7))
    le, tcs, data = ref.sb_build(7, x, y, value)
    np.testing.assert_allclose(sb.log_energy, le, rtol=1e-15)
    np.testing.assert_allclose(sb.totalcs, tcs, rtol=1e-12)
    np.testing.assert_allclose(sb.table(), data, rtol=1e-9, atol=1e-9)
    # inverse CDF: monotone in pcum, ends at the integration limits
    t = sb.table()
    assert np.all(np.diff(t, axis=0) >= -1e-12)
    # pcum = 1 -> upper limit min(log(gamma_max / T), log 1) (seltzer.jl:184)
    T = np.exp(sb.log_energy)
    np.testing.assert_allclose(t[-1], np.minimum(np.log(5e7 * ref.eV / T), 0.0), atol=1e-9)


@pytest.mark.parametrize("which", ["electron", "photon", "positron"])
def test_collision_table_matches_restatement(pcl, comp, which):
    co = pcl.co
    Fdt = co.elementary_charge * 5e5 * 1e-12
    procs = {"electron": pcl.workloads.electron_processes(comp),
             "photon": pcl.workloads.photon_processes(comp),
             "positron": pcl.workloads.positron_processes(comp)}[which]
    sp = {"electron": pcl.Electron, "photon": pcl.Photon, "positron": pcl.Positron}[which]
    F = 0.0 if sp == pcl.Photon else Fdt
    tab = pcl.collision_table_from_processes(procs, sp, F, safety=1.15)
    a, rb, perm = ref.collision_table(procs, sp == pcl.Photon, sp != pcl.Photon, F, safety=1.15)
    assert list(tab.perm) == list(perm)
    got = tab.rate_array()
    np.testing.assert_allclose(got, a[:, perm, :], rtol=1e-9, atol=1e-6 * np.abs(a).max())
    np.testing.assert_allclose(tab.ratebound.reshape(-1, tab.order).T, rb, rtol=1e-9, atol=1e-6 * np.abs(rb).max())


def test_positron_table_order_reference_quirk(pcl, comp):
    """Bhabha and annihilation cross sections are NaN at E = 0; Julia's
    sortperm(rev=true) puts NaN keys first (collision_table.jl:141-145)."""
    tab = pcl.collision_table_from_processes(pcl.workloads.positron_processes(comp), pcl.Positron, 0.0)
    names = [type(p).__name__ for p in tab.proc]
    assert names == ["Bhaba", "Bhaba", "PositronAnihilation", "PositronAnihilation", "RelativisticCoulomb",
                     "RelativisticCoulomb"]


def test_ratebound_bounds_rates(pcl, comp):
    """ratebound >= sum of rates on a dense grid above the cut (the null-collision
    method's requirement, collisions.jl:156-161)."""
    co = pcl.co
    Fdt = co.elementary_charge * 5e5 * 1e-12
    tab = pcl.collision_table_from_processes(pcl.workloads.electron_processes(comp), pcl.Electron, Fdt, safety=1.15)
    for E in np.exp(np.linspace(np.log(1e4), np.log(2e8), 600)) * co.eV:
        s = sum(tab.rate_at(j, E) for j in range(tab.nproc))
        assert tab.ratebound_at(E) >= s * (1 - 1e-12), E / co.eV


def test_chebfit_exact_on_polynomials(pcl):
    """An order-n fit reproduces polynomials of degree < n to rounding."""
    k, xmax, n = 10, 1.0, 3
    a = ref.chebfit(lambda x: 3 * x * x - 2 * x + 0.5, k, xmax, n)
    x = np.linspace(1e-6, 0.999, 200)
    np.testing.assert_allclose(ref.chebeval(x, k, xmax, a), 3 * x * x - 2 * x + 0.5, rtol=1e-12, atol=1e-12)


def test_continuum_loss_matches_restatement(pcl, comp):
    co = pcl.co
    nel = 14 * comp["N2"] + 16 * comp["O2"]
    cl = pcl.ChebContinuumLoss.build(pcl.ContinuumLoss(nel, 85.7 * co.eV, 1e4 * co.eV), 2.6e8 * co.eV, 3)
    k, xmax = cl.bints.k, cl.bints.xmax
    assert abs(xmax - 2 ** k * 1e4 * co.eV) < 1e-30
    ec = ref.chebfit(lambda E: ref.energy_loss(nel, 85.7 * co.eV, 1e4 * co.eV, False, E), k, xmax, 3)
    pc = ref.chebfit(lambda E: ref.energy_loss(nel, 85.7 * co.eV, 1e4 * co.eV, True, E), k, xmax, 3)
    np.testing.assert_allclose(cl.ec.reshape(k + 1, 3).T, ec, rtol=1e-10)
    np.testing.assert_allclose(cl.pc.reshape(k + 1, 3).T, pc, rtol=1e-10)
    # restricted stopping power of 1 MeV electrons in air: ~0.16 MeV/m (below the 0.2 MeV/m total)
    f = cl.force_magnitude(pcl.Electron, 1e6 * co.eV) / (1e6 * co.eV)
    assert 0.12 < f < 0.2


def test_moller_total_cs_integrates_the_differential(pcl):
    """The Moller total cross section above the cut (moller.jl:40-56, a closed
    form) equals the integral over eps = T2 / T in [tcut / T, 1/2] of the
    published Moller differential cross section per atom,
    2 pi r_e^2 Z / (beta^2 (gamma - 1)) [((gamma - 1) / gamma)^2
    + (1 / eps) (1 / eps - (2 gamma - 1) / gamma^2)
    + (1 / (1 - eps)) (1 / (1 - eps) - (2 gamma - 1) / gamma^2)],
    integrated numerically here: a check of the restated closed form against
    the physics it stands for, independent of any restatement."""
    from scipy.integrate import quad
    co = pcl.co
    for Z in (7, 8):
        for tcut_ev in (1e3, 1e4):
            m = pcl.Moller(Z, tcut_ev * co.eV)
            for T_ev in (2.5e3, 3e4, 1e6, 3e7, 1e9):
                if tcut_ev / T_ev >= 0.5:
                    continue
                g = 1.0 + T_ev * co.eV / co.electron_mc2
                b2 = (g * g - 1.0) / (g * g)
                q = (2.0 * g - 1.0) / (g * g)
                f = lambda e: ((g - 1.0) / g) ** 2 + (1.0 / e) * (1.0 / e - q) + (1.0 / (1.0 - e)) * (1.0 / (1.0 - e) - q)
                integral, err = quad(f, tcut_ev / T_ev, 0.5, epsabs=0.0, epsrel=1e-12, limit=200)
                want = 2.0 * np.pi * co.r_e ** 2 * Z * integral / (b2 * (g - 1.0))
                got = pcl.totalcs(m, T_ev * co.eV)
                assert abs(got - want) <= 1e-9 * want, (Z, tcut_ev, T_ev, got, want)


def test_coulomb_total_cs_integrates_the_differential(pcl):
    """The screened relativistic Coulomb total cross section
    (relativistic_coulomb.jl:58-75, a closed form) equals pi r_e^2 Z^2 /
    (beta^4 gamma^2) times the integral over x = sin^2(theta / 2) in [0, 1] of
    (1 - beta^2 x) / (x + alpha)^2, the density its sampler draws from
    (relativistic_coulomb.jl:27-52), integrated numerically here in
    y = ln(x + alpha) (with the reference's 1e-4 eV added to the energy)."""
    from scipy.integrate import quad
    co = pcl.co
    for Z in (7, 8):
        c = pcl.RelativisticCoulomb(Z)
        for K_ev in (1e2, 1e4, 1e6, 1e8):
            K = K_ev * co.eV + 1e-4 * co.eV
            mc2 = co.electron_mass * co.c ** 2
            a = 1.3413 * Z ** (-1.0 / 3.0) * co.a_0
            g = 1.0 + K / mc2
            p = np.sqrt(K * (K + 2.0 * mc2)) / co.c
            b = p / (g * co.electron_mass * co.c)
            al = co.hbar ** 2 / (4.0 * p * p * a * a)
            # y = ln(x + alpha) spreads the peak of width alpha at x = 0
            integral, err = quad(lambda y: (1.0 - b * b * (np.exp(y) - al)) * np.exp(-y), np.log(al),
                                 np.log1p(al), epsabs=0.0, epsrel=1e-12, limit=400)
            want = np.pi * co.r_e ** 2 * Z ** 2 / (b ** 4 * g ** 2) * integral
            got = pcl.totalcs(c, K_ev * co.eV)
            assert abs(got - want) <= 1e-8 * want, (Z, K_ev, got, want)


def test_bhabha_total_cs_integrates_the_differential(pcl):
    """The Bhabha total cross section above the cut (bhaba.jl:34-48, a closed
    form) equals the integral over eps in [tcut / T, 1] of the published
    differential form 2 pi r_e^2 Z / (gamma - 1) [1 / (beta^2 eps^2) - B1 / eps
    + B2 - B3 eps + B4 eps^2], y = 1 / (gamma + 1), B1 = 2 - y^2,
    B2 = (1 - 2y)(3 + y^2), B3 = (1 - 2y)^2 + (1 - 2y)^3, B4 = (1 - 2y)^3,
    integrated numerically here in ln(eps)."""
    from scipy.integrate import quad
    co = pcl.co
    for Z in (7, 8):
        for tcut_ev in (1e3, 1e4):
            b = pcl.Bhabha(Z, tcut_ev * co.eV)
            for T_ev in (2e4, 3e5, 1e7, 1e9):
                g = 1.0 + T_ev * co.eV / co.electron_mc2
                b2 = (g * g - 1.0) / (g * g)
                y = 1.0 / (g + 1.0)
                u = 1.0 - 2.0 * y
                B1, B2, B3, B4 = 2.0 - y * y, u * (3.0 + y * y), u * u + u ** 3, u ** 3
                f = lambda e: 1.0 / (b2 * e * e) - B1 / e + B2 - B3 * e + B4 * e * e
                # in t = ln(eps), so that the 1 / eps^2 peak at the cut is resolved
                integral, err = quad(lambda t: f(np.exp(t)) * np.exp(t), np.log(tcut_ev / T_ev), 0.0,
                                     epsabs=0.0, epsrel=1e-12, limit=200)
                want = 2.0 * np.pi * co.r_e ** 2 * Z * integral / (g - 1.0)
                got = pcl.totalcs(b, T_ev * co.eV)
                assert abs(got - want) <= 1e-9 * want, (Z, tcut_ev, T_ev, got, want)


def test_klein_nishina_total_cs_integrates_the_differential(pcl):
    """The Klein-Nishina total cross section (compton.jl:34-47, a closed form)
    equals Z times the Klein-Nishina differential cross section per electron,
    d sigma / d Omega = (r_e^2 / 2) P^2 (P + 1 / P - sin^2 theta) with
    P = 1 / (1 + k (1 - cos theta)), k = E / (m_e c^2), integrated over the
    sphere numerically here."""
    from scipy.integrate import quad
    co = pcl.co
    for Z in (7, 8):
        c = pcl.KleinNishinaCompton(Z)
        for E_ev in (1e3, 1e5, 1e6, 1e8):
            k = E_ev * co.eV / co.electron_mc2

            def f(mu):
                P = 1.0 / (1.0 + k * (1.0 - mu))
                return P * P * (P + 1.0 / P - (1.0 - mu * mu))
            integral, err = quad(f, -1.0, 1.0, epsabs=0.0, epsrel=1e-12, limit=200)
            want = Z * 2.0 * np.pi * 0.5 * co.r_e ** 2 * integral
            got = pcl.totalcs(c, E_ev * co.eV)
            assert abs(got - want) <= 1e-7 * want, (Z, E_ev, got, want)


def _rbeb_bracket(w, t, t1, b1, bt2):
    """The bracket of the relativistic binary-encounter-Bethe differential
    cross section in w = W / B (Kim, Santos and Parente, Phys. Rev. A 62,
    052710 (2000); rbeb.jl:102-113)."""
    return (b1 ** 2 / (1 + t1) ** 2 + 1 / (t - w) ** 2 + 1 / (1 + w) ** 2
            - (1 + 2 * t1) * (1 / (t - w) + 1 / (1 + w)) / ((1 + t) * (1 + t1) ** 2)
            + (1 / (t - w) ** 3 + 1 / (1 + w) ** 3) * (-bt2 - np.log(2 * b1) + np.log(bt2 / (1 - bt2))))


def test_rbeb_total_cs_integrates_the_differential(pcl):
    """The RBEB total ionization cross section (rbeb.jl:119-146, a closed form)
    equals N times the integral of the RBEB differential cross section over
    w = W / B in [0, (T / B - 1) / 2], integrated numerically here, for an N2
    and an O2 orbital from 100 eV to 100 MeV."""
    from scipy.integrate import quad
    co = pcl.co
    mc2 = co.electron_mc2
    for B_ev, U_ev, N in ((15.58, 54.91, 2), (543.8, 796.2, 4)):
        r = pcl.RBEB(B_ev * co.eV, U_ev * co.eV, N)
        for T_ev in (1e2, 1e3, 1e4, 1e6, 1e8):
            if T_ev <= B_ev:
                continue
            t1, b1, u1 = T_ev * co.eV / mc2, B_ev * co.eV / mc2, U_ev * co.eV / mc2
            bt2, bb2, bu2 = (1 - 1 / (1 + t1) ** 2, 1 - 1 / (1 + b1) ** 2, 1 - 1 / (1 + u1) ** 2)
            t = T_ev / B_ev
            pref = 2 * co.a_0 ** 2 * np.pi * co.fine_structure ** 4 / (b1 * (bb2 + bt2 + bu2))
            integral, err = quad(lambda y: _rbeb_bracket(np.expm1(y), t, t1, b1, bt2) * np.exp(y), 0.0,
                                 np.log1p((t - 1) / 2), epsabs=0.0, epsrel=1e-12, limit=400)
            want = N * pref * integral
            got = pcl.totalcs(r, T_ev * co.eV)
            assert abs(got - want) <= 1e-8 * want, (B_ev, T_ev, got, want)


def test_annihilation_total_cs_integrates_the_differential(pcl):
    """The two-photon annihilation total cross section (anihilation.jl:24-32,
    Heitler's closed form) equals Z pi r_e^2 / ((gamma + 1) (gamma^2 - 1)) times
    the integral over the photon energy fraction eps in [eps_min, 1 - eps_min]
    of S(eps) = -(gamma + 1)^2 + (gamma^2 + 4 gamma + 1) / eps - 1 / eps^2,
    eps_min = (1 - sqrt((gamma - 1) / (gamma + 1))) / 2 (the differential form
    of the GEANT4 Physics Reference Manual), integrated numerically here."""
    from scipy.integrate import quad
    co = pcl.co
    for Z in (7, 8):
        a = pcl.PositronAnihilation(Z)
        for T_ev in (1e3, 1e5, 1e6, 1e8):
            g = 1.0 + T_ev * co.eV / co.electron_mc2
            e0 = 0.5 * (1.0 - np.sqrt((g - 1.0) / (g + 1.0)))
            S = lambda e: -(g + 1.0) ** 2 + (g * g + 4.0 * g + 1.0) / e - 1.0 / (e * e)
            integral, err = quad(lambda t: S(np.exp(t)) * np.exp(t), np.log(e0), np.log1p(-e0),
                                 epsabs=0.0, epsrel=1e-12, limit=400)
            want = Z * np.pi * co.r_e ** 2 * integral / ((g + 1.0) * (g * g - 1.0))
            got = pcl.totalcs(a, T_ev * co.eV)
            assert abs(got - want) <= 1e-8 * want, (Z, T_ev, got, want)
