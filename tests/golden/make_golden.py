"""Generate the golden vectors in tests/golden/ by running the reference
program itself.

The reference (jijn/phasefield_coarsening) has no tests and ships no
fixtures, so its own output on small seeded inputs is the pin: each case is
built with oracle/build_ref.py (the reference source with only its
compile-time grid/BC/step constants patched, see that file), fed an input
written with the oracle's HDF5 writer (oracle/hdf5_shim/h5ref.c), and its
output file and its stderr convergence line are stored next to the input in
one .npz.

Run from the repository root (needs the reference sources):
    python tests/golden/make_golden.py [case names]
"""
from __future__ import annotations

import json
import os
import re
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import oracle.build_ref as build_ref  # noqa: E402
from phasefield_coarsening_gb300 import build as pkg_build  # noqa: E402

SUMS_RE = re.compile(r"(\d+): c=\s*([0-9.eE+-]+); S=\s*([0-9.eE+-]+); L=\s*([0-9.eE+-]+)\s+iter: (\d+); err:\s*([0-9.eE+-]+)")


def smooth_random(shape, rng):
    """Smooth random fields: etaS in (0, 1) with interfaces, etaL near 1-etaS,
    c near the equilibrium compositions."""
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


# name: (shape, bc, n_iter, n_save, n_iter_init, dt_expr, fix_etaL, seed)
CASES = {
    "periodic_8x10x12": ((8, 10, 12), 0, 21, 20, None, None, True, 1),
    "noflux_8x10x12": ((8, 10, 12), 1, 21, 20, None, None, True, 2),
    "periodic_odd_5x7x9": ((5, 7, 9), 0, 31, 30, None, None, True, 3),
    "noflux_conly_6x6x6": ((6, 6, 6), 1, 16, 15, 10, None, True, 4),
    "periodic_dt08_8x8x8": ((8, 8, 8), 0, 41, 40, None, "0.8*dx*dx/(6.0*DL)", True, 5),
    "etaL_bug_6x7x8": ((6, 7, 8), 0, 11, 10, None, None, False, 6),
    # uniform liquid: every increment is zero, so the convergence test
    # (err < 1e-12 at a save, phasefield.c:247-250) stops the run at the first save
    "converged_uniform_6x6x6": ((6, 6, 6), 0, 51, 10, None, None, True, 7, "uniform"),
}


def make_case(name, spec, work):
    shape, bc, n_iter, n_save, n_init, dt_expr, fix, seed = spec[:8]
    from oracle import read_fields, write_fields      # the oracle's HDF5 subset: no product code
    rng = np.random.default_rng(seed)
    if len(spec) > 8 and spec[8] == "uniform":
        etaS, etaL, c = np.zeros(shape), np.ones(shape), np.full(shape, 0.95)
    else:
        etaS, etaL, c = smooth_random(shape, rng)
    inp = os.path.join(work, f"{name}.h5")
    write_fields(inp, etaS, etaL, c)
    exe = build_ref.build(*shape, bc=bc, n_iter=n_iter, n_save=n_save, n_iter_init=n_init, dt_expr=dt_expr,
                          fix_etaL=fix)
    r = build_ref.run(exe, inp)
    if r["rc"] != 0:
        raise RuntimeError(r["stderr"])
    outs = [ln.strip() for ln in r["stdout"].splitlines() if ln.strip()]
    saves = []
    for m in SUMS_RE.finditer(r["stderr"]):
        saves.append([int(m.group(1)), float(m.group(2)), float(m.group(3)), float(m.group(4)),
                      float(m.group(6))])
    arrays = {"in_etaS": etaS, "in_etaL": etaL, "in_c": c, "saves": np.array(saves)}
    for k, fn in enumerate(outs):
        oS, oL, oc = read_fields(fn if os.path.isabs(fn) else os.path.join(work, fn))
        arrays[f"out{k + 1}_etaS"], arrays[f"out{k + 1}_etaL"], arrays[f"out{k + 1}_c"] = oS, oL, oc
    meta = dict(shape=list(shape), bc=bc, n_iter=n_iter, n_save=n_save,
                n_iter_init=n_init if n_init is not None else 100000000, dt_expr=dt_expr or "0.125*dx*dx/DL",
                fix_etaL=fix, outputs=[os.path.basename(o) for o in outs], stderr=r["stderr"])
    arrays["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
    return meta


if __name__ == "__main__":
    pkg_build.build()
    work = tempfile.mkdtemp(prefix="ppf_golden_")
    try:
        for name, spec in CASES.items():
            if len(sys.argv) > 1 and name not in sys.argv[1:]:
                continue
            meta = make_case(name, spec, work)
            print(name, meta["outputs"])
    finally:
        shutil.rmtree(work)
