"""GPU parity of the fused step (through the C-ABI) against the oracle and
the reference's golden vectors, plus size-independent properties at full
size.  Tolerances are written next to each check."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import phasefield_coarsening_gb300 as ppf
from helpers import golden_cases, golden_dt, load_golden, smooth_state

pytestmark = pytest.mark.gpu

DT08 = 0.8 / (6.0 * 1e-14)       # 0.8 of the explicit limit dx^2/(6 DL)


def run_gpu(state, nsteps, bc=0, precision="f64", dt=0.0, c_only_from=None):
    shape = state[0].shape
    with ppf.Simulation(shape, ppf.params_default(dt=dt), bc=bc, precision=precision) as s:
        s.upload(*state)
        if c_only_from is None or c_only_from >= nsteps:
            s.step(nsteps)
        else:
            if c_only_from > 0:
                s.step(c_only_from)
            s.step_c_only(nsteps - c_only_from)
        out = s.download()
        st = s.reduce()
    return out, st


def maxabs(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))))


def test_fp64_parity_64cubed_1000_steps():
    """20 spheres R~U[4,8] on 64^3, periodic, dt = 0.8 of the limit, 1000
    steps: max-abs field error <= 1e-10 against the reference's FP64 step."""
    from phasefield_coarsening_gb300 import ic
    eS, eL, c, _ = ic.workload("spheres64_uniform4to8", seed=0)
    (gS, gL, gc), st = run_gpu((eS, eL, c), 1000, bc=0, dt=DT08)
    oS, oL, oc, sums = oracle.run(eS, eL, c, 1000, bc=0, params=oracle.reference_params(dt=DT08))
    errs = [maxabs(gS, oS), maxabs(gL, oL), maxabs(gc, oc)]
    print("fp64 1000-step max-abs errors", errs)
    assert max(errs) <= 1e-10
    np.testing.assert_allclose([st["sum_dc2"], st["sum_detaS2"], st["sum_detaL2"]], sums, rtol=1e-6)


@pytest.mark.parametrize("name", golden_cases())
def test_fp64_matches_reference_golden(name):
    d, meta = load_golden(name)
    etaL = d["in_etaL"] if meta["fix_etaL"] else np.ones_like(d["in_etaL"])
    state = (d["in_etaS"], etaL, d["in_c"])
    done = 0
    with ppf.Simulation(meta["shape"], ppf.params_default(dt=golden_dt(meta)), bc=meta["bc"]) as s:
        s.upload(*state)
        for k, row in enumerate(d["saves"]):
            it = int(row[0])
            full = max(0, min(it + 1, meta["n_iter_init"]) - done)
            if full:
                s.step(full)
            if it + 1 - done - full > 0:
                s.step_c_only(it + 1 - done - full)
            done = it + 1
            out = s.download()
            st = s.reduce()
            for f, arr in zip(("etaS", "etaL", "c"), out):
                # FP64 on both sides; the GPU contracts to FMAs and uses
                # reciprocals, so a few ulp per step
                assert maxabs(arr, d[f"out{k + 1}_{f}"]) <= 1e-12, (name, f)
            # the reference prints the sums with 5 significant digits
            np.testing.assert_allclose([st["sum_dc2"], st["sum_detaS2"], st["sum_detaL2"]], row[1:4], rtol=6e-5)


SHAPES = [(1, 1, 1), (2, 3, 4), (5, 7, 9), (13, 17, 19), (9, 10, 65), (33, 9, 130), (3, 70, 7)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("bc", [0, 1])
def test_fp64_shapes_and_bcs(shape, bc):
    st = smooth_state(shape, seed=sum(shape) + bc)
    (gS, gL, gc), g = run_gpu(st, 25, bc=bc)
    oS, oL, oc, sums = oracle.run(*st, 25, bc=bc)
    assert max(maxabs(gS, oS), maxabs(gL, oL), maxabs(gc, oc)) <= 1e-12
    # atol: on a 1-cell grid every neighbour is the cell itself and dc is
    # pure round-off in the reference's form (~1e-19), exactly 0 in flux form
    np.testing.assert_allclose([g["sum_dc2"], g["sum_detaS2"], g["sum_detaL2"]], sums, rtol=1e-8, atol=1e-30)


@pytest.mark.parametrize("bc", [0, 1])
def test_fp64_c_only_steps(bc):
    st = smooth_state((11, 12, 13), seed=7)
    (gS, gL, gc), g = run_gpu(st, 12, bc=bc, c_only_from=5)
    oS, oL, oc, sums = oracle.run(*st, 12, bc=bc, n_iter_init=5)
    assert max(maxabs(gS, oS), maxabs(gL, oL), maxabs(gc, oc)) <= 1e-12
    assert abs(g["sum_dc2"] - sums[0]) <= 1e-8 * sums[0]
    # sweep_fields_c leaves detaS/detaL alone: their sums are the last full step's
    _, _, _, s5 = oracle.run(*st, 5, bc=bc)
    np.testing.assert_allclose([g["sum_detaS2"], g["sum_detaL2"]], s5[1:], rtol=1e-8)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("bc", [0, 1])
def test_observables_match_oracle(precision, bc):
    st = smooth_state((20, 24, 70), seed=5)
    with ppf.Simulation(st[0].shape, bc=bc, precision=precision) as s:
        s.upload(*st)
        s.step(3)
        out = s.download()
        g = s.reduce()
    o = oracle.observe(*out, bc=bc)
    rt = 1e-12 if precision == "f64" else 2e-6     # f32: density in float, sum in double
    assert abs(g["mass"] - o["mass"]) <= 1e-13 * abs(o["mass"])   # c summed in double in both
    assert abs(g["solid"] - o["solid"]) <= rt * abs(o["solid"])
    assert g["solid_cells"] == o["solid_cells"]
    assert abs(g["free_energy"] - o["free_energy"]) <= rt * abs(o["free_energy"]) + 1e-6
    assert g["nonfinite"] == 0 and g["cells"] == 20 * 24 * 70 and g["steps"] == 3


def test_fp32_against_fp64_oracle_64cubed():
    """FP32 storage + arithmetic vs the FP64 oracle, 64^3 spheres, 500 steps.
    Field error bound 2e-5 (float c has a 6e-8 ulp near 1); solid fraction
    and mass agree to 1e-6 relative."""
    from phasefield_coarsening_gb300 import ic
    eS, eL, c, _ = ic.workload("spheres64_uniform4to8", seed=0)
    (gS, gL, gc), g = run_gpu((eS, eL, c), 500, bc=0, precision="f32", dt=DT08)
    oS, oL, oc, _ = oracle.run(eS, eL, c, 500, bc=0, params=oracle.reference_params(dt=DT08))
    errs = [maxabs(gS, oS), maxabs(gL, oL), maxabs(gc, oc)]
    o = oracle.observe(oS, oL, oc, bc=0)
    print("fp32 vs fp64 after 500 steps: max-abs", errs, "mass rel", (g["mass"] - o["mass"]) / o["mass"])
    assert max(errs) <= 2e-5
    assert abs(g["mass"] - o["mass"]) <= 1e-6 * o["mass"]
    assert abs(g["solid"] - o["solid"]) <= 1e-6 * o["solid"]


@pytest.mark.parametrize("shape", [(16, 32, 64), (17, 33, 70)])
@pytest.mark.parametrize("bc", [0, 1])
def test_fp32_full_and_partial_tiles_against_fp64_oracle(shape, bc):
    """The FP32 step on a domain whose tiles all lie inside (nx, ny multiples
    of 64 and 16: the launch without per-cell domain tests) and on one with
    partial tiles, 100 steps at dt = 0.8 of the limit, against the FP64
    oracle: max-abs field error <= 2e-5 (as for 64^3), mass to 1e-6."""
    st = smooth_state(shape, seed=21 + bc)
    (gS, gL, gc), g = run_gpu(st, 100, bc=bc, precision="f32", dt=DT08)
    oS, oL, oc, _ = oracle.run(*st, 100, bc=bc, params=oracle.reference_params(dt=DT08))
    errs = [maxabs(gS, oS), maxabs(gL, oL), maxabs(gc, oc)]
    assert max(errs) <= 2e-5, errs
    o = oracle.observe(oS, oL, oc, bc=bc)
    assert abs(g["mass"] - o["mass"]) <= 1e-6 * abs(o["mass"])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_solute_conserved_at_256cubed(precision):
    """Sum c is conserved by the flux form (phasefield.c:374-384): FP64 to
    1e-13 relative after 20 steps; FP32 storage rounds c + dc per cell
    (random, ~3e-8), bound 1e-8 relative."""
    st = smooth_state((256, 256, 256), seed=1)
    m0 = st[2].sum()
    with ppf.Simulation((256, 256, 256), precision=precision) as s:
        s.upload(*st)
        g0 = s.reduce()
        s.step(20)
        g1 = s.reduce()
    tol = 1e-13 if precision == "f64" else 1e-8
    if precision == "f64":
        assert abs(g0["mass"] - m0) <= 1e-13 * m0
    assert abs(g1["mass"] - g0["mass"]) <= tol * g0["mass"]


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_periodic_translation_equivariance(precision):
    """With periodic ghosts every cell does the same arithmetic wherever it
    sits, so rolling the input rolls the output bit for bit."""
    shape = (96, 80, 130)
    st = smooth_state(shape, seed=2)
    sh = (5, 17, 33)
    (a, _, ac), _ = run_gpu(st, 10, precision=precision)
    rolled = tuple(np.roll(x, sh, axis=(0, 1, 2)) for x in st)
    (b, _, bc_), _ = run_gpu(rolled, 10, precision=precision)
    assert np.array_equal(np.roll(a, sh, axis=(0, 1, 2)), b)
    assert np.array_equal(np.roll(ac, sh, axis=(0, 1, 2)), bc_)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_pure_solid_is_stationary(precision):
    shape = (8, 9, 70)
    cs = 0.4760325047801147
    st = (np.ones(shape), np.zeros(shape), np.full(shape, cs))
    (a, b, c), g = run_gpu(st, 50, precision=precision)
    ref = np.float32(cs) if precision == "f32" else cs
    assert np.all(a == 1.0) and np.all(b == 0.0) and np.all(c == ref)
    assert g["sum_dc2"] == 0.0 and g["sum_detaS2"] == 0.0


def test_uniform_state_is_a_pointwise_ode():
    """Laplacians vanish, dc = 0, and each cell follows the 1x1x1 system."""
    shape = (6, 7, 66)
    st = (np.full(shape, 0.7), np.full(shape, 0.4), np.full(shape, 0.8))
    (a, b, c), _ = run_gpu(st, 30, bc=1)
    one = oracle.run(np.full((1, 1, 1), 0.7), np.full((1, 1, 1), 0.4), np.full((1, 1, 1), 0.8), 30, bc=1)
    assert maxabs(a, one[0][0, 0, 0]) <= 1e-14 and maxabs(b, one[1][0, 0, 0]) <= 1e-14
    assert np.all(c == 0.8)


def test_nonfinite_cells_are_reported():
    st = list(smooth_state((8, 8, 8), seed=9))
    st[2] = st[2].copy()
    st[2][3, 4, 5] = np.nan
    with ppf.Simulation((8, 8, 8)) as s:
        s.upload(*st)
        g = s.reduce()
    assert g["nonfinite"] == 1


def test_state_errors():
    with ppf.Simulation((4, 4, 4)) as s:
        with pytest.raises(ppf.PPFError) as e:
            s.step(1)
        assert e.value.code == -4
        with pytest.raises(ppf.PPFError):
            s.download()
        with pytest.raises(ValueError):
            s.upload(np.zeros((4, 4, 5)), np.zeros((4, 4, 4)), np.zeros((4, 4, 4)))


@pytest.mark.parametrize("name", ["periodic_8x10x12", "noflux_conly_6x6x6", "etaL_bug_6x7x8",
                                  "converged_uniform_6x6x6"])
def test_ppf_program_matches_reference_run(name, tmp_path):
    """The `ppf` program on the reference's own input: same output files,
    same convergence lines (phasefield.c:240, :248, :267)."""
    d, meta = load_golden(name)
    inp = str(tmp_path / f"{name}.h5")
    ppf.write_fields(inp, d["in_etaS"], d["in_etaL"], d["in_c"])
    cmd = [ppf.EXE_PATH, inp, "--bc", "periodic" if meta["bc"] == 0 else "noflux", "--steps",
           str(meta["n_iter"]), "--save", str(meta["n_save"]), "--init", str(meta["n_iter_init"]),
           "--dt", repr(golden_dt(meta))]
    if not meta["fix_etaL"]:
        cmd.append("--ref-etaL-bug")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    outs = [ln for ln in r.stdout.splitlines() if ln]
    assert [os.path.basename(o) for o in outs] == meta["outputs"]
    ref_lines = [ln for ln in meta["stderr"].splitlines() if ": c=" in ln or ln.startswith("Total steps")]
    my_lines = [ln for ln in r.stderr.splitlines() if ": c=" in ln or ln.startswith("Total steps")]
    assert len(my_lines) == len(ref_lines)
    for k, fn in enumerate(outs):
        got = ppf.read_fields(fn)
        for f, arr in zip(("etaS", "etaL", "c"), got):
            assert maxabs(arr, d[f"out{k + 1}_{f}"]) <= 1e-12
    # identical text up to the last printed digit (sums agree to ~1e-14); the
    # stop (after n_iter, or at the first save with err < threshold) at the same step
    for a, b in zip(my_lines, ref_lines):
        assert a.split("\t")[0].split(":")[0] == b.split("\t")[0].split(":")[0]
    assert my_lines[-1].split(";")[0] == ref_lines[-1].split(";")[0]


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_launch_choices_are_bit_identical(precision):
    """The z chunk (uniform, or shorter chunks at the top of z), the unroll,
    the launch overlap and the way CTAs take work items (counter or
    round-robin) change only who computes a cell, never the arithmetic: every
    launch choice gives the same bits.  The last step's increment sums are
    summed per work item in item order, so for one z split they are the same
    bits whichever CTA took which item; another split groups the same terms
    differently."""
    shape = (40, 35, 70)
    st = smooth_state(shape, seed=12)
    ref, inc_of = None, {}
    # (the grid has whole tiles and edge tiles in x and y with either tile
    # shape: one launch over every tile, or two overlapping launches,
    # split = 0 / 1; the 32 x 32 tile shape, tile = 1, is FP32's only)
    t1 = 1 if precision == "f32" else 0
    for zc, roll, pdl, sched, zc2, tail, split, tile in [
            (None,) * 8, (1, 3, 1, 1, 0, 0, 1, 0), (1, 1, 0, 0, 0, 0, 0, 0), (7, 1, 0, 0, 0, 0, 1, 0),
            (7, 3, 1, 1, 0, 0, 0, 0), (40, 3, 0, 1, 0, 0, 1, 0), (40, 1, 1, 0, 0, 0, 0, 0), (13, 1, 1, 0, 0, 0, 1, 0),
            (13, 3, 0, 1, 0, 0, 0, 0), (2, 1, 1, 1, 0, 0, 0, 0), (12, 3, 1, 1, 4, 10, 1, 0), (12, 1, 1, 0, 4, 10, 0, 0),
            (9, 1, 0, 1, 2, 31, 1, 0), (16, 3, 1, 1, 5, 40, 0, 0), (7, 3, 1, 1, 0, 0, 1, t1), (7, 1, 0, 0, 0, 0, 0, t1),
            (13, 3, 1, 1, 5, 20, 1, t1), (40, 1, 1, 1, 0, 0, 0, t1)]:
        with ppf.Simulation(shape, bc=1, precision=precision) as s:
            if zc is not None:
                s.set_tune(zc, roll, pdl, sched, zc2, tail, split, tile)
            s.upload(*st)
            for _ in range(3):            # several launches: every launch resets the counter
                s.step(2)
            red = s.reduce()
            out = s.download()
            inc = (red["sum_dc2"], red["sum_detaS2"], red["sum_detaL2"])
        if ref is None:
            ref, ref_inc = out, inc
        else:
            for a, b in zip(out, ref):
                assert np.array_equal(a, b), (zc, roll, pdl, sched, zc2, tail, split, tile)
            np.testing.assert_allclose(inc, ref_inc, rtol=1e-13 if precision == "f64" else 1e-5)
            key = (zc, zc2, tail, split, tile)    # the same work items, summed in the same order
            if key in inc_of:
                assert inc == inc_of[key], (zc, roll, pdl, sched, zc2, tail, split, tile)
            inc_of[key] = inc


def test_fp64_has_one_tile_shape():
    with ppf.Simulation((8, 8, 8), precision="f64") as s:
        with pytest.raises(ppf.PPFError):
            s.set_tune(4, 1, 1, 1, 0, 0, 1, 1)
        s.set_tune(4, 1, 1, 1, 0, 0, 1, 0)
        assert s.get_tune()["tile"] == 0


def test_autotune_keeps_state_and_picks_a_valid_choice():
    shape = (64, 48, 130)
    st = smooth_state(shape, seed=13)
    with ppf.Simulation(shape, precision="f32") as s:
        s.upload(*st)
        s.step(3)
        before = s.download()
        t = s.autotune(trial_steps=3)
        after = s.download()
        assert t["roll"] in (1, 3) and 1 <= t["zc"] <= shape[0] and t["us_per_step"] > 0
        assert s.get_tune()["zc"] == t["zc"] and s.reduce()["steps"] == 3
        for a, b in zip(before, after):
            assert np.array_equal(a, b)
        s.step(4)
        got = s.download()
    ref = oracle.run(*st, 7, bc=0)
    assert max(float(np.abs(a - b).max()) for a, b in zip(got, ref[:3])) <= 1e-5


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_ppf_restart_continues_the_run_exactly(precision, tmp_path):
    """A run restarted from one of its own output files (--restart reads the
    /ppf_restart record: next iteration, dt, save number, error) writes the
    same later files, bit for bit, and the same convergence lines."""
    shape = (8, 10, 12)
    inp = str(tmp_path / "job.h5")
    ppf.write_fields(inp, *smooth_state(shape, seed=31))
    opts = ["--bc", "periodic", "--steps", "35", "--save", "10", "--dt", repr(DT08), "--precision", precision]
    r = subprocess.run([ppf.EXE_PATH, inp] + opts, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    outs = [ln for ln in r.stdout.splitlines() if ln]
    assert [os.path.basename(o) for o in outs] == ["job_1.h5", "job_2.h5", "job_3.h5"]
    rec = ppf.h5_read(outs[0], "ppf_restart").ravel()
    assert rec[0] == 11 and rec[1] == DT08 and rec[2] == 1
    # restart from the first save, dt taken from the record
    opts_r = [o for o in opts if o not in ("--dt", repr(DT08))] + ["--restart"]
    r2 = subprocess.run([ppf.EXE_PATH, outs[0]] + opts_r, capture_output=True, text=True, timeout=120)
    assert r2.returncode == 0, r2.stderr
    outs2 = [ln for ln in r2.stdout.splitlines() if ln]
    assert [os.path.basename(o) for o in outs2] == ["job_1_2.h5", "job_1_3.h5"]
    for a, b in zip(outs[1:], outs2):
        for x, y in zip(ppf.read_fields(a), ppf.read_fields(b)):
            assert np.array_equal(x, y)
        assert np.array_equal(ppf.h5_read(a, "ppf_restart"), ppf.h5_read(b, "ppf_restart"))
    conv = lambda t: [ln for ln in t.splitlines() if ": c=" in ln or ln.startswith("Total steps")]
    assert conv(r.stderr)[1:] == conv(r2.stderr)


def test_ppf_mass_project_option_keeps_the_solute_mass(tmp_path):
    """--mass-project (FP32 runs): every saved state holds the initial sum(c)
    to within a few units of 2^-24 (the projection's step)."""
    shape = (16, 20, 24)
    st = smooth_state(shape, seed=41)
    inp = str(tmp_path / "m.h5")
    ppf.write_fields(inp, *st)
    m0 = float(np.asarray(st[2], np.float32).astype(np.float64).sum())
    opts = ["--bc", "periodic", "--steps", "2001", "--save", "1000", "--dt", repr(DT08), "--precision", "f32"]
    r = subprocess.run([ppf.EXE_PATH, inp] + opts + ["--mass-project"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    outs = [ln for ln in r.stdout.splitlines() if ln]
    assert len(outs) == 2
    for fn in outs:
        c = ppf.read_fields(fn)[2]
        assert abs(c.sum() - m0) <= 4 * 2.0 ** -24       # within a few units of the projection's step
    r2 = subprocess.run([ppf.EXE_PATH, inp, "--precision", "f64", "--mass-project"], capture_output=True, text=True)
    assert r2.returncode != 0 and "f32" in r2.stderr
