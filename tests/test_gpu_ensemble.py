"""Ensembles: domains of different sizes stepped by one persistent launch
per time step (CUDA graph replays) must give exactly what each domain gives
on its own."""
import numpy as np
import pytest

import phasefield_coarsening_gb300 as ppf
from helpers import smooth_state

pytestmark = pytest.mark.gpu

SHAPES = [(24, 24, 24), (32, 40, 48), (16, 16, 70), (33, 17, 65), (48, 48, 48), (9, 30, 130)]


def _single(shape, state, steps, bc, precision, pieces=(37,)):
    with ppf.Simulation(shape, bc=bc, precision=precision) as s:
        s.upload(*state)
        for n in pieces:
            s.step(n)
        return s.download(), s.reduce()


@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("bc", ["periodic", "noflux"])
@pytest.mark.parametrize("sched,pdl,split,tile", [(1, 1, 1, 0), (0, 0, 1, 0), (1, 1, 0, 0), (1, 1, 1, 1),
                                                  (0, 1, 0, 1)])
def test_ensemble_equals_independent_domains(precision, bc, sched, pdl, split, tile):
    """With work items from the counter (1) or dealt round-robin (0); one
    launch over every tile (split 0) or whole and edge tiles as two launches,
    the edge-tile launch overlapping the whole-tile launch (pdl 1) or not;
    with 64 x 16 or 32 x 32 tiles (tile 0 / 1, the second FP32 only)."""
    if tile and precision == "f64":
        pytest.skip("FP64 has one tile shape")
    states = [smooth_state(sh, seed=30 + i) for i, sh in enumerate(SHAPES)]
    with ppf.Ensemble(SHAPES, bc=bc, precision=precision) as e:
        e.set_tune(8, 1, sched, pdl, split, tile)
        for d, st in enumerate(states):
            e.upload(d, *st)
        e.step(1)          # leaves every domain at buffer 1
        e.step(36)         # one direct step, two 16-step graph replays, the statistics step
        for d, (sh, st) in enumerate(zip(SHAPES, states)):
            got = e.download(d)
            gs = e.reduce(d)
            ref, rs = _single(sh, st, 37, bc, precision, pieces=(1, 36))
            for a, b in zip(got, ref):
                assert np.array_equal(a, b), (d, sh)
            # per-thread sums in the state's precision per work item, grouped
            # differently by the ensemble's work items
            np.testing.assert_allclose([gs["sum_dc2"], gs["sum_detaS2"], gs["sum_detaL2"]],
                                       [rs["sum_dc2"], rs["sum_detaS2"], rs["sum_detaL2"]],
                                       rtol=1e-12 if precision == "f64" else 1e-5)
            assert gs["steps"] == 37 and gs["mass"] == rs["mass"]


def test_ensemble_autotune_keeps_state_and_reupload():
    states = [smooth_state(sh, seed=50 + i) for i, sh in enumerate(SHAPES[:4])]
    with ppf.Ensemble(SHAPES[:4], precision="f32") as e:
        for d, st in enumerate(states):
            e.upload(d, *st)
        e.step(3)
        before = [e.download(d) for d in range(4)]
        t = e.autotune(trial_steps=2)
        assert t["roll"] in (1, 3) and t["zc"] >= 1
        for d in range(4):
            for a, b in zip(e.download(d), before[d]):
                assert np.array_equal(a, b)
        # a re-upload of one domain while the others are at buffer 1
        e.step(1)
        e.upload(2, *states[2])
        e.step(2)
        ref, _ = _single(SHAPES[2], states[2], 2, "periodic", "f32", pieces=(2,))
        for a, b in zip(e.download(2), ref):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_ensemble_batched_io_equals_per_domain_io(precision):
    """ppf_ensemble_upload_all / download_all (one conversion launch for all
    domains) give the per-domain calls' bits, before and after steps, and
    after an odd number of steps (state in the second buffer)."""
    states = [smooth_state(sh, seed=70 + i) for i, sh in enumerate(SHAPES)]
    with ppf.Ensemble(SHAPES, precision=precision) as a, ppf.Ensemble(SHAPES, precision=precision) as b:
        a.upload_all(states)
        for d, st in enumerate(states):
            b.upload(d, *st)
        for x, y in zip(a.download_all(), [b.download(d) for d in range(len(SHAPES))]):
            for p, q in zip(x, y):
                assert np.array_equal(p, q)
        for n in (5, 16):
            a.step(n)
            b.step(n)
            got = a.download_all()
            for d in range(len(SHAPES)):
                for p, q in zip(got[d], b.download(d)):
                    assert np.array_equal(p, q), (n, d)
            ra, rb = a.reduce(2), b.reduce(2)
            assert ra["sum_dc2"] == rb["sum_dc2"] and ra["steps"] == rb["steps"]
        # a fresh batched upload restarts every domain (increment sums cleared)
        a.upload_all(states)
        assert a.reduce(0)["sum_dc2"] == 0.0 and a.reduce(0)["steps"] == 0
