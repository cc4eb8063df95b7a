"""FP32 against FP64: run the same seeded microstructure with both step
precisions and report the field error, the particle statistics (count,
mean radius R-bar) and the solute mass drift.

    python -m phasefield_coarsening_gb300.validate --workload spheres256_lognormal5_vf30 --steps 10000
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import Simulation, params_default
from . import ic

DT08 = 0.8 / (6.0 * 1e-14)       # 0.8 of the explicit limit dx^2/(6 DL)


def compare(shape=None, workload="spheres64_uniform4to8", steps=1000, seed=0, dt=DT08, bc="periodic", every=None):
    """FP32 against FP64 after `steps`; with `every`, both runs are also
    reduced (FP64 sums on the device) every `every` steps and the series of
    mass drifts and solid-fraction / free-energy differences is returned."""
    eS, eL, c, info = ic.workload(workload, seed=seed, shape=shape)
    res = {"workload": workload, "grid": list(eS.shape), "steps": steps, "particles_initial": info["particles"]}
    sims = {p: Simulation(eS.shape, params_default(dt=dt), bc=bc, precision=p) for p in ("f64", "f32")}
    try:
        m0 = {}
        for p, s in sims.items():
            s.upload(eS, eL, c)
            m0[p] = s.reduce()["mass"]
        series = []
        done = 0
        every = every or steps
        while done < steps:
            n = min(every, steps - done)
            for s in sims.values():
                s.step(n)
            done += n
            r = {p: s.reduce() for p, s in sims.items()}
            series.append({
                "step": done,
                "mass_drift_fp64": (r["f64"]["mass"] - m0["f64"]) / m0["f64"],
                "mass_drift_fp32": (r["f32"]["mass"] - m0["f32"]) / m0["f32"],
                "solid_fraction_diff": (r["f32"]["solid"] - r["f64"]["solid"]) / r["f64"]["cells"],
                "free_energy_rel_diff": (r["f32"]["free_energy"] - r["f64"]["free_energy"]) /
                abs(r["f64"]["free_energy"]),
                "nonfinite": int(r["f32"]["nonfinite"] + r["f64"]["nonfinite"]),
            })
        out = {p: (s.download(), s.reduce(), s.particles(), m0[p]) for p, s in sims.items()}
    finally:
        for s in sims.values():
            s.close()
    (f64, s64, p64, m64), (f32, s32, p32, m32) = out["f64"], out["f32"]
    if len(series) > 1:
        res["series"] = series
        res["series_max"] = {k: max(abs(x[k]) for x in series) for k in series[0] if k != "step"}
    res.update({
        "max_abs_etaS": float(np.abs(f64[0] - f32[0]).max()),
        "max_abs_etaL": float(np.abs(f64[1] - f32[1]).max()),
        "max_abs_c": float(np.abs(f64[2] - f32[2]).max()),
        "rbar_fp64": p64["mean_radius"], "rbar_fp32": p32["mean_radius"],
        "rbar_rel_err": abs(p32["mean_radius"] - p64["mean_radius"]) / p64["mean_radius"],
        "count_fp64": p64["count"], "count_fp32": p32["count"],
        "solid_fraction_fp64": s64["solid"] / s64["cells"], "solid_fraction_fp32": s32["solid"] / s32["cells"],
        "free_energy_rel_err": abs(s32["free_energy"] - s64["free_energy"]) / abs(s64["free_energy"]),
        "mass_drift_fp64": (s64["mass"] - m64) / m64, "mass_drift_fp32": (s32["mass"] - m32) / m32,
        # interface position: solid-cell count difference over the interface area (cells)
        "interface_shift_cells": (p32["solid_volume"] - p64["solid_volume"]) / max(p64["interface_area"], 1.0),
    })
    return res


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", default="spheres64_uniform4to8", choices=sorted(ic.WORKLOADS))
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--every", type=int, default=None, help="reduce both runs every N steps")
    a = ap.parse_args()
    print(json.dumps(compare(None, a.workload, a.steps, a.seed, every=a.every)))
