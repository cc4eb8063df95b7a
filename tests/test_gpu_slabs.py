"""Slabs on the GPU: a domain split into z slabs (one context each, one
ghost-plane exchange per step) against the undivided domain -- bit for bit,
both BCs and precisions, uneven slab heights, and after c-only-free
reuploads."""
import numpy as np
import pytest

import phasefield_coarsening_gb300 as ppf
from helpers import smooth_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("bc", ["periodic", "noflux"])
@pytest.mark.parametrize("nslabs", [1, 2, 3, 5])
def test_slabs_equal_the_undivided_domain(precision, bc, nslabs):
    shape = (23, 20, 70)
    st = smooth_state(shape, seed=32)
    with ppf.Simulation(shape, bc=bc, precision=precision) as s:
        s.upload(*st)
        s.step(12)
        ref = s.download()
        rst = s.reduce()
    with ppf.Slabs(shape, nslabs, bc=bc, precision=precision) as sl:
        sl.upload(*st)
        sl.step(7)
        sl.step(5)
        got = sl.download()
        gst = sl.reduce()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    assert gst["cells"] == rst["cells"] and gst["nonfinite"] == 0
    for k in ("mass", "solid", "free_energy"):
        assert abs(gst[k] - rst[k]) <= 1e-12 * abs(rst[k]) + 1e-300, k
    # the increment sums are per-thread sums in the state's precision per
    # work item, grouped differently by the slabs' work items
    rel = 1e-12 if precision == "f64" else 1e-5
    for k in ("sum_dc2", "sum_detaS2", "sum_detaL2"):
        assert abs(gst[k] - rst[k]) <= rel * abs(rst[k]) + 1e-300, k
