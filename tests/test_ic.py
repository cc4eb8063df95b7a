"""Seeded synthetic microstructures."""
import math

import numpy as np

from phasefield_coarsening_gb300 import ic


def test_equilibrium_compositions_are_common_tangent():
    cs, cl = ic.equilibrium_compositions()
    assert abs(cs - 0.4760325047801147) < 1e-12 and abs(cl - 0.9990325047801147) < 1e-12
    A, CS, CL, cS0, cL0 = 1e9, -1e6, 1e7, 0.455, 0.978
    fS = lambda c: 0.5 * A * (c - cS0) ** 2 + CS
    fL = lambda c: 0.5 * A * (c - cL0) ** 2 + CL
    slope = A * (cs - cS0)
    assert abs(slope - A * (cl - cL0)) < 1e-3
    assert abs((fS(cs) - slope * cs) - (fL(cl) - slope * cl)) < 1e-3


def test_seeded_and_non_overlapping():
    rng1, rng2 = np.random.default_rng(4), np.random.default_rng(4)
    c1, r1 = ic.place_particles((48, 48, 48), rng1, ("uniform", 4.0, 8.0), count=20)
    c2, r2 = ic.place_particles((48, 48, 48), rng2, ("uniform", 4.0, 8.0), count=20)
    assert np.array_equal(c1, c2) and np.array_equal(r1, r2) and len(r1) == 20
    dims = np.array([48.0] * 3)
    for i in range(len(r1)):
        for j in range(i):
            d = c1[i] - c1[j]
            d -= dims * np.round(d / dims)
            assert math.sqrt(d @ d) >= r1[i] + r1[j] + 1.0 - 1e-9


def test_small_workload_fields():
    eS, eL, c, info = ic.generate((32, 32, 32), radius=("uniform", 4, 6), count=5, seed=1)
    assert info["particles"] == 5
    assert eS.min() >= 0 and eS.max() <= 1 and np.allclose(eS + eL, 1)
    assert abs(c.min() - 0.4760) < 2e-3 and abs(c.max() - 0.9990) < 2e-3
    assert 0.5 * info["sphere_fraction"] < (eS > 0.5).mean() < 1.5 * info["sphere_fraction"]


def test_volume_fraction_target():
    eS, eL, c, info = ic.generate((64, 64, 64), radius=("lognormal", 5.0, 0.3), vf=0.2, seed=2)
    assert abs(info["sphere_fraction"] - 0.2) < 0.02
