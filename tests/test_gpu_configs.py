"""The benchmark configurations at their stated sizes (or, for the 100k-step
512^3 run, the same loop on a shorter horizon): the FP32 path against the
FP64 path on the 256^3 workload for 10k steps with FP64 reductions every
100 steps, and the coarsening loop that records R-bar(t) and the particle
count.  Bounds are written next to each check."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_fp32_against_fp64_256cubed_10k_steps_reduced_every_100():
    """256^3 periodic, ~6400 lognormal spheres (median R 5, sigma 0.3) at
    solid fraction 0.3, dt = 0.8 of the limit, 10 000 steps; both precisions
    reduced in FP64 on the device every 100 steps."""
    from phasefield_coarsening_gb300 import validate
    r = validate.compare(None, "spheres256_lognormal5_vf30", steps=10000, seed=0, every=100)
    m = r["series_max"]
    print({k: v for k, v in r.items() if k != "series"})
    assert len(r["series"]) == 100 and m["nonfinite"] == 0
    # mean particle radius within 0.5 % of FP64 (measured ~1e-6), same count
    assert r["rbar_rel_err"] <= 5e-3
    assert r["count_fp32"] == r["count_fp64"]
    # FP64 conserves solute to round-off at every reduction
    assert m["mass_drift_fp64"] <= 1e-13
    # FP32 storage drops increments below half an ulp of c: a slow drift,
    # ~7e-8 after 10k steps; ppf_mass_project removes it where it matters
    assert m["mass_drift_fp32"] <= 2e-7
    # phase fraction and free energy at every reduction
    assert m["solid_fraction_diff"] <= 1e-6
    assert m["free_energy_rel_diff"] <= 1e-5
    # interface position (solid-volume difference over the interface area, cells)
    assert abs(r["interface_shift_cells"]) <= 1e-3
    for k in ("max_abs_etaS", "max_abs_etaL", "max_abs_c"):
        assert r[k] <= 2e-3, k


def test_coarsening_loop_records_rbar_and_count():
    """The long run's loop (512^3 statistics: solid fraction 0.2, median R 4)
    on a 128^3 grid for 3000 steps, observed every 1000: R-bar, count and
    solid fraction are recorded, solute is conserved, the free energy does
    not rise beyond FP32 noise, and the R-bar^3 fit is reported."""
    from phasefield_coarsening_gb300 import coarsen
    r = coarsen.run("spheres512_lognormal4_vf20", steps=3000, every=1000, shape=(128, 128, 128), autotune=False)
    s = r["series"]
    assert [p["step"] for p in s] == [0, 1000, 2000, 3000]
    assert all(p["nonfinite"] == 0 and p["count"] > 0 for p in s)
    assert r["mass_drift_max"] <= 2e-7
    # a gradient flow: the free energy falls while the initial interfaces
    # relax (2e-5 relative over the first 1000 steps) and then stays put; it
    # never rises by more than the FP32 storage noise of the state (the FP64
    # sum moves by a few parts in 1e8 per 1000 steps)
    for a, b in zip(s, s[1:]):
        assert b["free_energy"] <= a["free_energy"] + 1e-7 * abs(a["free_energy"])
    f = r["fit"]
    assert f["points"] == 4 and np.isfinite(f["k_rbar3_per_time"])
    # with the reference's constants the microstructure barely moves
    assert abs(f["rbar_rel_change"]) <= 1e-3
