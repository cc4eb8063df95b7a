"""Shared helpers for the tests (golden fixture access, small states)."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    return d, meta


def golden_dt(meta):
    """The time step the case was built with (dx = 1, DL = 1e-14)."""
    dx, DL = 1.0, 1.0e-14
    return {"0.125*dx*dx/DL": 0.125 * dx * dx / DL, "0.8*dx*dx/(6.0*DL)": 0.8 * dx * dx / (6.0 * DL)}[meta["dt_expr"]]


def smooth_state(shape, seed=0):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    phase = np.zeros(shape)
    for _ in range(3):
        k = rng.integers(1, 3, size=3)
        ph = rng.random() * 2 * np.pi
        phase += np.sin(2 * np.pi * (k[0] * z / nz + k[1] * y / ny + k[2] * x / nx) + ph)
    etaS = 0.5 * (1 + np.tanh(phase))
    etaL = 1.0 - etaS + 0.02 * (rng.random(shape) - 0.5)
    h = etaS ** 2 / (etaS ** 2 + etaL ** 2)
    c = 0.476 * h + 0.999 * (1 - h) + 2e-3 * (rng.random(shape) - 0.5)
    return etaS, etaL, c
