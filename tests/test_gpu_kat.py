"""Known answers derived from the equations (the reference has no tests of
its own): flat interfaces at the common-tangent compositions stay put;
reflection and axis permutation commute with the step (periodic and
no-flux); cells with etaS^2 + etaL^2 = 0 give the reference's NaNs."""
import numpy as np
import pytest

import oracle
import phasefield_coarsening_gb300 as ppf
from helpers import smooth_state
from phasefield_coarsening_gb300 import ic

pytestmark = pytest.mark.gpu
DT08 = 0.8 / (6.0 * 1e-14)


def slab(shape):
    cS, cL = ic.equilibrium_compositions()
    x = np.arange(shape[2])
    n = shape[2]
    # interfaces between grid points (a cell exactly at 0.5 would hide the crossing)
    e1 = 0.5 * (1 + np.tanh(2 * (x - n / 4 - 0.3) / 4.0)) * 0.5 * (1 - np.tanh(2 * (x - 3 * n / 4 - 0.3) / 4.0))
    eS = np.broadcast_to(e1, shape).copy()
    eL = 1 - eS
    h = eS ** 2 / (eS ** 2 + eL ** 2)
    return eS, eL, h * cS + (1 - h) * cL


def crossings(e):
    row = e[0, 0]
    return np.array([i + (0.5 - row[i]) / (row[i + 1] - row[i]) for i in range(len(row) - 1)
                     if (row[i] - 0.5) * (row[i + 1] - 0.5) < 0])


@pytest.mark.parametrize("precision,tol", [("f64", 1e-6), ("f32", 1e-4)])
def test_flat_interfaces_at_the_common_tangent_stay_put(precision, tol):
    shape = (4, 4, 64)
    st = slab(shape)
    with ppf.Simulation(shape, ppf.params_default(dt=DT08), bc="periodic", precision=precision) as s:
        s.upload(*st)
        s.step(8000)
        got = s.download()
    x0, x1 = crossings(st[0]), crossings(got[0])
    assert len(x0) == len(x1) == 2
    assert np.abs(x1 - x0).max() < tol
    if precision == "f64":
        ref = oracle.run(*st, 8000, bc=0, params=oracle.reference_params(dt=DT08))
        assert np.abs(crossings(ref[0]) - x1).max() < 1e-9


@pytest.mark.parametrize("bc", ["periodic", "noflux"])
def test_reflection_and_axis_permutation_commute_with_the_step(bc):
    shape = (10, 16, 16)
    st = smooth_state(shape, seed=23)
    ops = [(lambda a: a[:, :, ::-1], lambda a: a[:, :, ::-1]),       # x -> -x
           (lambda a: a[::-1], lambda a: a[::-1]),                   # z -> -z
           (lambda a: a.transpose(0, 2, 1), lambda a: a.transpose(0, 2, 1))]   # x <-> y
    with ppf.Simulation(shape, ppf.params_default(dt=DT08), bc=bc, precision="f64") as s:
        s.upload(*st)
        s.step(50)
        base = s.download()
        for fwd, back in ops:
            s.upload(*[np.ascontiguousarray(fwd(a)) for a in st])
            s.step(50)
            out = s.download()
            for a, b in zip(base, out):
                # summation order of the neighbours changes under the map: round-off only
                assert np.abs(a - back(b)).max() <= 1e-13


def test_zero_eta_cells_give_the_reference_nans():
    shape = (6, 7, 9)
    eS, eL, c = smooth_state(shape, seed=29)
    eS[2, 3, 4] = eL[2, 3, 4] = 0.0             # h = 0/0 in the reference's interpolation (:331)
    eS[4, 1, 7] = eL[4, 1, 7] = 0.0
    with ppf.Simulation(shape, bc="periodic", precision="f64") as s:
        s.upload(eS, eL, c)
        s.step(1)
        got = s.download()
        n = s.reduce()["nonfinite"]
    ref = oracle.run(eS, eL, c, 1, bc=0)
    for a, b in zip(got, ref[:3]):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        m = ~np.isnan(b)
        assert np.abs(a[m] - b[m]).max() <= 1e-12
    assert n == int(np.any([np.isnan(a) for a in got], axis=0).sum()) > 0
