"""The largest configuration's grid (512^3, 134 M cells): FP32 and FP64
contexts hold it, step it, conserve solute and analyse its particles."""
import numpy as np
import pytest

import phasefield_coarsening_gb300 as ppf

pytestmark = pytest.mark.gpu

N = 512
DT = 0.8 / (6.0 * 1e-14)


def big_state():
    """Smooth separable microstructure (cheap to build at 512^3)."""
    t = 2 * np.pi * np.arange(N) / N
    a, b = np.sin(6 * t + 0.3), np.cos(6 * t + 0.2)     # no grid plane on a zero
    eS = 0.5 * (1 + np.tanh(3 * a[:, None, None] * b[None, :, None] * a[None, None, :]))
    eL = 1.0 - eS
    c = 0.476 * eS + 0.999 * eL
    return eS, eL, c


@pytest.mark.parametrize("precision,steps,drift", [("f32", 40, 1e-7), ("f64", 4, 1e-13)])
def test_512_cubed(precision, steps, drift):
    st = big_state()
    with ppf.Simulation((N, N, N), ppf.params_default(dt=DT), bc="periodic", precision=precision) as s:
        s.upload(*st)
        r0 = s.reduce()
        p0 = s.particles(0.5)
        s.step(steps)
        r1 = s.reduce()
        p1 = s.particles(0.5)
    assert r1["nonfinite"] == 0 and r1["steps"] == steps
    assert abs(r1["mass"] / r0["mass"] - 1.0) < drift
    # the pattern's solid blocks: 12 sign regions per axis on the periodic torus
    # (the end regions join across the boundary), half of the 12^3 products
    # positive (the oracle's labeller gives the same on smaller grids)
    assert p0["count"] == 864
    # positive blocks touch along their edges, and relaxing the interfaces
    # joins them: fewer, never more, particles afterwards
    assert 1 <= p1["count"] <= 864
    assert r1["free_energy"] <= r0["free_energy"]
