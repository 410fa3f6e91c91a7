"""The recipe of the grown mixed avalanche (data/rrea_mixed_0.5MVm.json) and
its sampler: the growth stopped through PopulationTargetCallback, the species
mix had settled, and a draw keeps the recorded fractions, spectra and angles."""
import numpy as np


def test_recipe_records_a_settled_growth(pcl):
    rec = pcl.workloads.rrea_recipe()
    g = rec["growth"]
    assert g["seed_electrons"] == 10_000 and g["dt_s"] == 1e-12 and g["roulette"] is None
    assert g["stop"]["callback"] == "PopulationTargetCallback"
    assert g["live_at_stop"][0] >= g["stop"]["n"] and not g["errors"]
    h = np.asarray(rec["history"])
    # the step before the stop was still below the target
    assert h[-2, 1] < g["stop"]["n"] <= h[-1, 1]
    ratio = np.asarray(rec["settling"]["photon_per_electron_last_4_outputs"])
    assert np.ptp(ratio) / ratio.mean() < 0.01
    fr = [rec["species"][k]["fraction"] for k in ("electron", "photon", "positron")]
    assert abs(sum(fr) - 1) < 1e-12 and min(fr) > 0
    for k in ("electron", "photon", "positron"):
        d = rec["species"][k]
        assert d["outside_histogram"] == 0
        assert sum(c[2] for c in d["cells"]) == d["count"]


def test_sample_keeps_fractions_and_spectra(pcl):
    rec = pcl.workloads.rrea_recipe()
    n = 1 << 18
    st = pcl.workloads.rrea_mixed_state(n, seed=3)
    counts = [len(st[s].w) for s in (pcl.Electron, pcl.Photon, pcl.Positron)]
    assert sum(counts) == n
    assert counts == pcl.workloads.rrea_species_counts(n)
    le = np.asarray(rec["log10_energy_eV_edges"])
    for sp, name in ((pcl.Electron, "electron"), (pcl.Photon, "photon")):
        a = st[sp]
        E = pcl.kinenergy(sp, a.p) / pcl.co.eV
        assert E.min() >= rec["growth"]["cuts_eV"][name]
        d = rec["species"][name]
        assert abs(E.mean() / d["mean_energy_eV"] - 1) < 0.02
        # the log-energy histogram of the draw against the recipe's marginal (3 sigma per bin)
        want = np.zeros(len(le) - 1)
        for iE, ic, c in d["cells"]:
            want[iE] += c
        want *= len(E) / want.sum()
        got, _ = np.histogram(np.log10(E), le)
        big = want > 50
        assert np.all(np.abs(got[big] - want[big]) <= 3 * np.sqrt(want[big]) + 1)
        pn = np.linalg.norm(a.p, axis=1)
        np.testing.assert_allclose(pn, pcl.momentum_norm_from_kin(sp, E * pcl.co.eV), rtol=1e-12)
        assert np.all(a.w == 1.0)
    # same seed, same draw
    again = pcl.workloads.rrea_mixed_state(n, seed=3)
    np.testing.assert_array_equal(again[pcl.Photon].p, st[pcl.Photon].p)
