"""Benchmark of the explicit phase-field step on GB300.

Workload: spheres256_lognormal5_vf30 -- a 256^3 periodic grid, seeded
non-overlapping spheres with lognormal radii (median 5 cells, sigma 0.3) at
solid fraction 0.3, tanh interfaces of width 4, c at the common-tangent
compositions +- 1e-3; dt = 0.8 of the explicit limit.  FP32 fused stencil.

One bench step = 100 explicit time steps followed by the FP64 reductions
(mass, phase fraction, free energy, last-step increment sums) read back to
the host.  value = cells * time steps / second over the K timed bench steps
(GLUPS), device-timed with CUDA events on the stream the kernels run on.
The state (2 x 3 x 67 MB) is larger than L2, so no flush is needed.

e2e: the same metric through the C-ABI with host buffers: each step uploads
the state from pinned host memory (ppf_upload), advances 100 steps,
reduces and downloads the state (ppf_download).  Two contexts on two
streams, one host thread each, take alternate steps, so that one's copies
over the host link overlap the other's stepping; wall clock over all steps.

--impl reference: the reference program itself (phasefield.c, serial build
with OpenMP on its three passes, oracle/build_ref.py) on the host cores,
same workload; each step is one run of 100 time steps (one bench step of
this arm) timed by the program's own loop timer.  Its input file is written
by the oracle's HDF5 code: the product library is never loaded there.

Extra sections of the default line: fp64 (the FP64 fused step, the
reference's precision, with its roofline against the measured FP64 FMA
rate), surrogate (the learned K-step network with the stencil corrector),
ensemble (64 domains in one persistent launch per time step).
--workload ensemble64 and --workload coarsen512 (512^3, R-bar(t) every 1000
steps for --steps x 1000 steps) print their own lines.

Multi-GPU: replicas only (one independent domain per rank), max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "sim-time per wall-s @256^3: surrogate vs plain stencil at <=1% R-bar err; GLUPS"
WORKLOAD = "spheres256_lognormal5_vf30"
DT_LIMIT = 1.0 / (6.0 * 1e-14)
DT = 0.8 * DT_LIMIT
INNER = 100
# host threads / contexts that take turns in the end-to-end measurement,
# and ensembles in the ensemble's (measured best: 3 contexts 202 GLUPS, 2
# ensembles with the batched upload/download 130 against 110 with 3)
E2E_CONTEXTS = 3
ENS_E2E_ENSEMBLES = 2
ALG_BYTES_F32 = 24          # read etaS, etaL, c + write 3, float


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float) -> float:
    """The largest of one float per rank (the job's time is its slowest
    rank's); the value itself when not running under torch.distributed."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_glups(world: int, cells: int, time_steps: int, seconds: float) -> float:
    """Whole-job lattice updates per second (replicas: every rank advances
    its own `cells`-cell domain by `time_steps`)."""
    return world * cells * time_steps / seconds / 1e9


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def host_link_gbs(pinned_src, pinned_dst):
    """Pinned host <-> device copy rates of this host (GB/s, best of 3 copies
    of one field array each way), which bound the end-to-end line."""
    import torch

    dev = torch.empty(pinned_src.numel(), dtype=pinned_src.dtype, device="cuda")
    out = {}
    for name, fn in (("h2d", lambda: dev.copy_(pinned_src.view(-1), non_blocking=True)),
                     ("d2h", lambda: pinned_dst.view(-1).copy_(dev, non_blocking=True))):
        best = None
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name] = round(dev.numel() * dev.element_size() / (best * 1e-3) / 1e9, 1)
    del dev
    return out


def read_profile_traffic():
    """dram bytes per launch of the f32 step from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", "step_f32_spheres256.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.startswith("dram_bytes_per_launch_256:"):
            try:
                return float(ln.split(":", 1)[1])
            except ValueError:
                return None
    return None


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline_sample(state, cells):
    """The reference program (or, where it cannot be built, the oracle
    restatement) on a bounded sample of the same workload."""
    import oracle.build_ref as br
    import __graft_entry__ as ge
    ncores = os.cpu_count() or 1
    try:
        exe = br.build(**ge.REF_BENCH)
        import oracle
        with tempfile.TemporaryDirectory() as td:
            inp = os.path.join(td, "in.h5")
            oracle.write_fields(inp, *state)      # the oracle's HDF5 writer: no product code
            r = br.run(exe, inp, threads=ncores, timeout=1200)
        if r["rc"] == 0 and r["loop_s"]:
            steps = ge.REF_BENCH["n_iter"]
            return {"value": cells * steps / r["loop_s"] / 1e9, "unit": "GLUPS", "cores": ncores,
                    "kind": "reference",
                    "sample": f"{steps} time steps of the 256^3 workload, reference phasefield.c serial build "
                              f"+ OpenMP on sweep_fields, gcc -O2, {ncores} threads"}
    except Exception as e:  # fall through to the port
        print(f"reference build unavailable ({e}); timing the oracle restatement", file=sys.stderr)
    import oracle
    steps = 5
    t0 = time.perf_counter()
    oracle.run(*state, steps, bc=0, params=oracle.reference_params(dt=DT))
    t = time.perf_counter() - t0
    return {"value": cells * steps / t / 1e9, "unit": "GLUPS", "cores": ncores, "kind": "port",
            "sample": f"{steps} time steps of the 256^3 workload, oracle restatement (C, OpenMP), {ncores} threads"}


# The configured network first: 32 hidden channels, K = 50 steps per call (BASELINE config 4);
# then two width-16 variants that are not the configured network (a cheaper layer, and K = 200).
SURROGATE_WEIGHTS = ("surrogate_w32_k50.npz", "surrogate_w16_k50.npz", "surrogate_w16_k200.npz")


def surrogate_section(state, shape):
    """The learned surrogate + stencil corrector against the plain FP32
    stencil on the same 256^3 state: simulated time per wall second of both
    arms (device-synchronised host clock around each cycle), the largest
    relative errors of mean particle radius, solid fraction and free energy
    over the run, the solute-mass drift, and the tensor throughput of one
    surrogate call.  One entry per committed trained network."""
    import numpy as np

    import phasefield_coarsening_gb300 as ppf
    from phasefield_coarsening_gb300 import surrogate as S

    cells = int(np.prod(shape))
    peak = None
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        peak = float(json.load(open(p)).get("bf16_tflops_sustained", 0)) or None
    out = []
    for name in SURROGATE_WEIGHTS:
        path = os.path.join(REPO, "phasefield_coarsening_gb300", "weights", name)
        if not os.path.exists(path):
            continue
        net = S.load(path)
        cfg = net.config
        res = S.compare_to_stencil(net, state, cycles=12, calls=10, corrector_steps=50, warmup=500)
        res.pop("trajectory")
        sim = ppf.Simulation(shape, ppf.params_default(dt=DT), "periodic", "f32")
        sim.upload(*state)
        net.advance(sim, 2)
        sim.sync()
        w0 = time.perf_counter()
        net.advance(sim, 10)
        sim.sync()
        call_s = (time.perf_counter() - w0) / 10
        sim.close()
        w = cfg["width"]
        chans = [16, w, w, w, w, w, 16]
        flop = 2 * 27 * sum(chans[i] * chans[i + 1] for i in range(6)) * cells
        # useful: the first layer's 5 real input channels, the last layer's 3 real outputs
        useful = 2 * 27 * (5 * w + 4 * w * w + w * 3) * cells
        tf = flop / call_s / 1e12
        tfu = useful / call_s / 1e12
        out.append({
            "weights": name, "width": w, "k_steps": cfg["k_steps"],
            "configured_network": w == 32 and cfg["k_steps"] == 50,
            "calls_per_cycle": 10, "corrector_steps": 50,
            "sim_time_per_wall_s": res["sim_time_per_wall_s"], "speedup_vs_stencil": round(res["speedup"], 3),
            "max_rel_err": res["max_rel_err"], "field_err_vs_change": res["field_err_vs_change"],
            "mass_drift": res["mass_drift"], "steps": res["steps"],
            "fallbacks": res["fallbacks"], "ms_per_call": round(call_s * 1e3, 3),
            "roofline": {"bound": "tensor", "achieved": round(tf, 1), "peak": peak, "unit": "TFLOP/s",
                         "frac": round(tf / peak, 4) if peak else None,
                         "flop_per_call": flop, "what": "executed BF16 MMA FLOPs of one call over its whole "
                                                       "duration (features, 6 convolutions, mass projection)",
                         "useful_flop_per_call": useful, "useful_achieved": round(tfu, 1),
                         "useful_frac": round(tfu / peak, 4) if peak else None},
        })
        net.close()
    return out


def run_ours(args):
    import numpy as np
    import torch

    import phasefield_coarsening_gb300 as ppf
    from phasefield_coarsening_gb300 import ic

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    eS, eL, c, info = ic.workload(WORKLOAD, seed=args.seed + rank)
    shape = eS.shape
    cells = int(np.prod(shape))
    sim = ppf.Simulation(shape, ppf.params_default(dt=DT), bc="periodic", precision="f32")
    # a real (non-NULL) stream shared by the kernels and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    sim.upload(eS, eL, c)
    if args.launch:
        # a fixed launch choice (z chunk, unroll), e.g. for a reproducible profile
        if len(args.launch) not in (2, 4):
            raise SystemExit("--launch takes ZC ROLL or ZC ROLL ZC2 TAIL")
        zc2, tail = (args.launch[2], args.launch[3]) if len(args.launch) == 4 else (0, 0)
        sim.set_tune(args.launch[0], args.launch[1], 1, 1, zc2, tail)
        tune = sim.get_tune()
    else:
        tune = sim.autotune(trial_steps=10)    # the project's launch autotuner (state is kept)

    def bench_step():
        sim.step(INNER)
        return sim.reduce()

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        bench_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    stats = None
    for k in range(args.steps):
        ev[k][0].record(stream)
        sim.step(INNER)
        ev[k][1].record(stream)
        stats = sim.reduce()
    t1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = t0.elapsed_time(t1)
    step_ms = sum(a.elapsed_time(b) for a, b in ev) / (args.steps * INNER)   # per f32 step launch
    total_ms = max_over_ranks(total_ms)
    value = job_glups(world, cells, INNER * args.steps, total_ms * 1e-3)

    # e2e through the C-ABI with pinned host buffers.  Every bench step
    # uploads its input from pinned host memory, steps, reduces and downloads
    # its result.  E2E_CONTEXTS contexts on their own streams, each driven by
    # its own host thread (the C-ABI's one-context-per-thread model; the calls
    # release the GIL), take turns at the bench steps, so that the host-link
    # copies of some overlap the others' stepping (measured on a GB300: 133,
    # 171 and 202 GLUPS with one, two and three contexts, 215 device-only).
    extra, streams = [], []
    for _ in range(E2E_CONTEXTS - 1):
        sx = ppf.Simulation(shape, ppf.params_default(dt=DT), bc="periodic", precision="f32")
        streams.append(torch.cuda.Stream())
        sx.set_stream(streams[-1].cuda_stream)
        sx.set_tune(tune["zc"], tune["roll"], tune["pdl"], tune["sched"], tune["zc2"], tune["tail"], tune["split"],
                    tune["tile"])
        extra.append(sx)
    host = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (eS, eL, c)]
    outh = [[torch.empty(shape, dtype=torch.float64).pin_memory() for _ in range(3)] for _ in range(E2E_CONTEXTS)]
    ptr_in = [h.data_ptr() for h in host]

    def e2e_worker(s, outp, n):
        ptr_out = [h.data_ptr() for h in outp]
        for _ in range(n):
            s.upload_from(*ptr_in)
            s.step(INNER)
            s.reduce()
            s.download_into(*ptr_out)

    def e2e_run(n):
        k = E2E_CONTEXTS
        ths = [threading.Thread(target=e2e_worker, args=(s, o, (n + k - 1 - i) // k))
               for i, (s, o) in enumerate(zip([sim] + extra, outh))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    e2e_run(max(E2E_CONTEXTS, args.warmup))
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    e2e_run(args.steps)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - w0
    for sx in extra:
        sx.close()
    e2e_s = max_over_ranks(e2e_s)
    e2e_value = job_glups(world, cells, INNER * args.steps, e2e_s)
    link = host_link_gbs(host[0], outh[0][0])

    if rank == 0:
        hbm, src = peaks()
        achieved = ALG_BYTES_F32 * cells / (step_ms * 1e-3) / 1e9
        traffic = read_profile_traffic()
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic: seeded spheres ({info['particles']} particles, sphere fraction "
                    f"{info['sphere_fraction']:.3f}), generated on the host",
            "config": {"workload": WORKLOAD, "grid": list(shape), "bc": "periodic", "dt": DT,
                       "time_steps_per_bench_step": INNER, "precision": "f32 storage and arithmetic, FP64 reductions",
                       "l2": "state 403 MB > 129 MB L2 (no flush needed)", "parallelism": f"replicas x{world}",
                       "launch": {k: v for k, v in tune.items() if k != "us_per_step"}},
            "sim_time_per_wall_s": round(value * 1e9 / cells * DT, 1),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "traffic": traffic,
                         "kernel": "step_tma_kernel<float> (fused step, TMA-fed)", "algorithmic_bytes_per_launch": ALG_BYTES_F32 * cells,
                         "avg_launch_us": round(step_ms * 1e3, 2), "peak_source": src},
            "e2e": {"value": round(e2e_value, 3), "unit": "GLUPS", "h2d_bytes_per_step": 3 * cells * 8,
                    "d2h_bytes_per_step": 3 * cells * 8 + 8 * 8, "host_link_gbs": link,
                    "how": "ppf_upload (pinned float64 host arrays) + 100 ppf_step + ppf_reduce + ppf_download "
                           f"per bench step; {E2E_CONTEXTS} contexts on their own streams, one host thread each, take "
                           "turns at the bench steps so that copies overlap stepping; wall clock over all steps"},
            "gpu_launches": args.steps * (INNER + 1 + 2),
            "clocks": clk,
            "final_stats": {k: stats[k] for k in ("mass", "solid", "free_energy", "nonfinite")},
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample((eS, eL, c), cells)
        if not args.no_fp64:
            # the reference's precision on the GPU (the CPU arm computes in FP64)
            line["fp64"] = fp64_section((eS, eL, c), shape)
        if not args.no_surrogate:
            line["surrogate"] = surrogate_section((eS, eL, c), shape)
        if not args.no_ensemble:
            line["ensemble"] = ensemble_section(args.seed, steps=max(3, args.steps // 4), warmup=2)
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        dist.destroy_process_group()


def ensemble_measure(doms, steps, warmup, world=1, launch=None):
    """The ensemble of domains `doms` advanced by one persistent launch per
    time step under CUDA-graph replay, against the same domains stepped one
    context at a time (64 launches per time step).  Host wall-clock around
    step(n) + sync, so launch overheads count.  `launch` = (z chunk, unroll)
    fixes the launch choice (work items from the counter, programmatic
    dependent launch, one launch over every tile, 64 x 16 tiles) instead of
    the autotuner's.  Returns (ensemble, section dict, tune); the caller
    closes the ensemble."""
    import numpy as np

    import phasefield_coarsening_gb300 as ppf

    shapes = [d[0].shape for d in doms]
    cells = int(sum(np.prod(s) for s in shapes))
    prm = ppf.params_default(dt=DT)
    ens = ppf.Ensemble(shapes, prm, bc="periodic", precision="f32")
    for i, (eS, eL, c, _) in enumerate(doms):
        ens.upload(i, eS, eL, c)
    if launch:
        ens.set_tune(launch[0], launch[1], 1, 1, 0, 0)
        tune = ens.get_tune()
    else:
        tune = ens.autotune(trial_steps=5)

    def timed(step_fn, sync_fn):
        for _ in range(warmup):
            step_fn()
        sync_fn()
        t = []
        for _ in range(steps):
            w0 = time.perf_counter()
            step_fn()
            sync_fn()
            t.append(time.perf_counter() - w0)
        return sum(t), t

    ens_s, per = timed(lambda: ens.step(INNER), ens.sync)
    ens_s = max_over_ranks(ens_s)
    value = job_glups(world, cells, INNER * steps, ens_s)

    sims = []
    for eS, eL, c, _ in doms:
        s = ppf.Simulation(eS.shape, prm, bc="periodic", precision="f32")
        s.upload(eS, eL, c)
        sims.append(s)                     # each context's own default launch choice

    def seq_step():
        for s in sims:
            s.step(INNER)

    seq_s, _ = timed(seq_step, lambda: [s.sync() for s in sims])
    seq_s = max_over_ranks(seq_s)
    seq_value = job_glups(world, cells, INNER * steps, seq_s)
    # bit-exact agreement of the two paths on one domain after equal step counts
    same = all(np.array_equal(a, b) for a, b in zip(ens.download(0), sims[0].download()))
    for s in sims:
        s.close()
    hbm, src = peaks()
    achieved = ALG_BYTES_F32 * cells * INNER * steps / ens_s / 1e9
    sec = {
        "workload": "ensemble64_edges48to128_vf10to40", "value": round(value, 3), "unit": "GLUPS",
        "steps": steps, "warmup": warmup, "ms_per_step": round(1e3 * ens_s / steps, 4),
        "spread": round((max(per) - min(per)) / min(per), 4) if per else None,
        "domains": len(doms), "edges": sorted({s[0] for s in shapes}), "cells": cells,
        "time_steps_per_bench_step": INNER, "launch": tune,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_source": src,
                     "what": "24 B per cell-step over all domains / host wall-clock of step(100) + sync"},
        "sequential_contexts": {"value": round(seq_value, 3), "unit": "GLUPS",
                                "how": "one ppf_step per domain per bench step, each context's default launch choice"},
        "sequential_equals_ensemble": bool(same),
    }
    return ens, sec, tune


def ensemble_section(seed, steps, warmup):
    """Config 2 as a section of the default line: 64 domains, K bench steps."""
    from phasefield_coarsening_gb300 import ic
    doms = ic.ensemble_workload(seed=seed)
    ens, sec, _ = ensemble_measure(doms, steps, warmup)
    ens.close()
    return sec


def run_ensemble(args):
    """--workload ensemble64: 64 periodic cubes (edges 48/64/96/128, solid
    fraction U[0.1, 0.4]) advanced by one persistent launch per time step
    under CUDA-graph replay (see ensemble_measure), plus the end-to-end line
    through the C-ABI with host buffers."""
    import numpy as np
    import torch

    import phasefield_coarsening_gb300 as ppf
    from phasefield_coarsening_gb300 import ic

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    doms = ic.ensemble_workload(seed=args.seed + rank)
    shapes = [d[0].shape for d in doms]
    cells = int(sum(np.prod(s) for s in shapes))
    prm = ppf.params_default(dt=DT)
    clocks = ClockSampler(local)
    clocks.start()
    ens, sec, tune = ensemble_measure(doms, args.steps, args.warmup, world,
                                      launch=args.launch[:2] if args.launch else None)
    clk = clocks.stop()

    # e2e through the C-ABI: every bench step uploads all domains from pinned
    # host memory, steps, and downloads all domains.  ENS_E2E_ENSEMBLES ensembles,
    # one host thread each, take turns at the bench steps so that the
    # host-link copies of some overlap the others' stepping (as in the
    # single-domain line).
    # (plain launches: with programmatic dependent launch, an ensemble's next
    # step grid holds SM slots while it waits, which the other ensemble's
    # kernels then wait for)
    extra = []
    ens.set_tune(tune["zc"], tune["roll"], tune["sched"], 0, tune["split"], tune["tile"])
    for _ in range(ENS_E2E_ENSEMBLES - 1):
        ex = ppf.Ensemble(shapes, prm, bc="periodic", precision="f32")
        ex.set_tune(tune["zc"], tune["roll"], tune["sched"], 0, tune["split"], tune["tile"])
        extra.append(ex)
    pin_in = [[torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in d[:3]] for d in doms]
    pin_out = [[[torch.empty(s, dtype=torch.float64).pin_memory() for _ in range(3)] for s in shapes]
               for _ in range(ENS_E2E_ENSEMBLES)]

    ptr_in = [[t.data_ptr() for t in arrs] for arrs in pin_in]

    def e2e_worker(e, outs, n):
        ptr_out = [[t.data_ptr() for t in arrs] for arrs in outs]
        for _ in range(n):
            e.upload_from_all(ptr_in)          # ppf_ensemble_upload_all
            e.step(INNER)
            e.download_into_all(ptr_out)       # ppf_ensemble_download_all
            e.sync()

    def e2e_run(n):
        k = ENS_E2E_ENSEMBLES
        ths = [threading.Thread(target=e2e_worker, args=(e, o, (n + k - 1 - i) // k))
               for i, (e, o) in enumerate(zip([ens] + extra, pin_out))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    e2e_run(max(ENS_E2E_ENSEMBLES, args.warmup))
    w0 = time.perf_counter()
    e2e_run(args.steps)
    e2e_s = max_over_ranks(time.perf_counter() - w0)
    for ex in extra:
        ex.close()
    e2e_value = job_glups(world, cells, INNER * args.steps, e2e_s)
    if rank == 0:
        line = {
            "metric": "GLUPS (ensemble of 64 domains, one persistent launch per time step)", "value": sec["value"],
            "unit": "GLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic: {len(doms)} seeded sphere microstructures, {cells} cells in total",
            "config": {"workload": sec["workload"], "domains": len(doms), "edges": sec["edges"], "cells": cells,
                       "bc": "periodic", "dt": DT, "time_steps_per_bench_step": INNER, "launch": tune,
                       "l2": f"state {cells * 24 / 1e9:.2f} GB > 129 MB L2 (no flush needed)"},
            "roofline": sec["roofline"],
            "sequential_contexts": sec["sequential_contexts"],
            "sequential_equals_ensemble": sec["sequential_equals_ensemble"],
            "e2e": {"value": round(e2e_value, 3), "unit": "GLUPS", "h2d_bytes_per_step": 3 * cells * 8,
                    "d2h_bytes_per_step": 3 * cells * 8,
                    "how": "ppf_ensemble_upload_all (pinned float64 host arrays of every domain) + 100 steps + "
                           "ppf_ensemble_download_all per bench step; ENS_E2E_ENSEMBLES ensembles, one host "
                           "thread each, take turns at the bench steps so that copies overlap stepping; wall clock"
                           .replace("ENS_E2E_ENSEMBLES", str(ENS_E2E_ENSEMBLES))},
            "gpu_launches": args.steps * INNER,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ens.close()
    if world > 1:
        dist.destroy_process_group()


# FP64 arithmetic of one cell-step of the fused kernel with AS == AL (the
# reference's constants): pass A 18 (incl. one reciprocal), pass B 61;
# an FMA counts 2.  Algorithmic: the ring and halo-plane recomputation are
# not counted.
FP64_FLOP_PER_CELL = 79


def fp64_section(state, shape, steps=30):
    """The reference's precision on the GPU: the FP64 fused step on the same
    256^3 state, device-timed (CUDA events on its stream), with its roofline
    against this GPU's measured FP64 FMA rate (the FP64 pipe bounds it) and
    its HBM fraction (48 B per cell-step)."""
    import torch

    import phasefield_coarsening_gb300 as ppf
    cells = int(shape[0] * shape[1] * shape[2])
    peak = ppf.measure_fp64_peak()
    sim = ppf.Simulation(shape, ppf.params_default(dt=DT), bc="periodic", precision="f64")
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.upload(*state)
    tune = sim.autotune(trial_steps=3)
    sim.step(3)
    sim.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    sim.sync()
    us = e0.elapsed_time(e1) * 1e3 / steps
    sim.close()
    tf = FP64_FLOP_PER_CELL * cells / (us * 1e-6) / 1e12
    hbm, src = peaks()
    gbs = 48 * cells / (us * 1e-6) / 1e9
    return {
        "kernel": "step_tma_kernel<double> (fused step, TMA-fed)", "value": round(cells / (us * 1e-6) / 1e9, 3),
        "unit": "GLUPS", "us_per_step": round(us, 1), "steps": steps, "launch": tune,
        "roofline": {"bound": "fp64", "achieved": round(tf, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
                     "frac": round(tf / peak, 4), "flop_per_cell": FP64_FLOP_PER_CELL,
                     "peak_source": "measured: ppf_measure_fp64_peak (DFMA chains on every SM, CUDA events)",
                     "hbm_frac": round(gbs / hbm, 4), "hbm_achieved_gbs": round(gbs, 1)},
    }


def run_coarsen(args):
    """--workload coarsen512: the long FP32 coarsening run (512^3 periodic,
    solid fraction 0.2, lognormal radii of median 4, dt = 0.8 of the limit),
    R-bar and the particle count every 1000 steps, the R-bar^3 ~ t fit.
    --steps is the number of 1000-step observation intervals (default 100:
    the configuration's 100k steps)."""
    import torch

    from phasefield_coarsening_gb300 import coarsen
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if rank != 0:
        return
    clocks = ClockSampler(local)
    clocks.start()
    r = coarsen.run("spheres512_lognormal4_vf20", steps=1000 * args.steps, every=1000, seed=args.seed)
    clk = clocks.stop()
    cells = 512 ** 3
    line = {
        "metric": "GLUPS (512^3 coarsening run, R-bar and count every 1000 steps)",
        "value": round(r["glups_stepping"], 3), "unit": "GLUPS", "n_gpus": 1, "steps": args.steps, "warmup": 0,
        "ms_per_step": round(1e3 * r["stepping_s"] / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic: {r['particles_initial']} seeded lognormal spheres (median R 4) at solid fraction 0.2",
        "config": {"workload": "spheres512_lognormal4_vf20", "grid": r["grid"], "bc": "periodic", "dt": r["dt"],
                   "time_steps_per_bench_step": 1000, "launch": r["launch"],
                   "l2": f"state {cells * 24 / 1e9:.2f} GB > 129 MB L2 (no flush needed)"},
        "wall_s": round(r["wall_s"], 2), "mass_drift_max": r["mass_drift_max"],
        "free_energy_rel_change": r["free_energy_rel_change"], "fit": r["fit"],
        "series": [{k: p[k] for k in ("step", "rbar", "count", "solid_fraction", "free_energy")} for p in r["series"]],
        "gpu_launches": None, "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def _product_library_loaded() -> bool:
    try:
        with open("/proc/self/maps") as f:
            return any("libppf_gb300" in ln for ln in f)
    except OSError:
        return False


def run_reference(args):
    """The reference's own CPU implementation of the step on the host cores:
    the reference program (phasefield.c, patched serial build with OpenMP on
    its three passes, oracle/build_ref.py) when it can be built here, else
    the oracle restatement (C, OpenMP).  Rank 0 only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    import oracle
    import oracle.build_ref as br
    import __graft_entry__ as ge
    from phasefield_coarsening_gb300 import ic      # numpy only: the product library is not loaded
    ncores = os.cpu_count() or 1
    eS, eL, c, info = ic.workload(WORKLOAD, seed=args.seed)
    cells = int(np.prod(eS.shape))
    steps_per_run = ge.REF_BENCH["n_iter"]
    try:
        exe = br.build(**ge.REF_BENCH)
        kind = "reference"
    except Exception as e:               # no reference sources nor patched unit: the oracle port
        print(f"reference program unavailable ({str(e)[:120]}); timing the oracle restatement", file=sys.stderr)
        exe, kind = None, "port"
    loop = []
    if exe is not None:
        with tempfile.TemporaryDirectory() as td:
            inp = os.path.join(td, "in.h5")
            oracle.write_fields(inp, eS, eL, c)
            for _ in range(args.warmup):
                br.run(exe, inp, threads=ncores, timeout=1800)
            for _ in range(args.steps):
                r = br.run(exe, inp, threads=ncores, timeout=1800)
                if r["rc"] != 0 or not r["loop_s"]:
                    print(json.dumps({"impl": "reference", "unavailable": "reference run failed: " + r["stderr"][-200:]}))
                    return
                loop.append(r["loop_s"])
        sample = (f"{steps_per_run} time steps per run of the reference phasefield.c (serial build + OpenMP on "
                  f"sweep_fields, gcc -O2), {ncores} threads")
    else:
        prm = oracle.reference_params(dt=DT)
        for _ in range(args.warmup):
            oracle.run(eS, eL, c, steps_per_run, bc=0, params=prm)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            oracle.run(eS, eL, c, steps_per_run, bc=0, params=prm)
            loop.append(time.perf_counter() - t0)
        sample = (f"{steps_per_run} time steps per run of the oracle restatement of phasefield.c's step (C, "
                  f"OpenMP), {ncores} threads")
    total = sum(loop)
    value = cells * steps_per_run * args.steps / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "GLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic: seeded spheres ({info['particles']} particles)",
        "config": {"workload": WORKLOAD, "grid": list(eS.shape), "bc": "periodic", "dt": DT,
                   "time_steps_per_bench_step": steps_per_run, "parallelism": f"OpenMP x{ncores} (host)"},
        "sim_time_per_wall_s": round(value * 1e9 / cells * DT, 1),
        "cpu_baseline": {"value": round(value, 4), "unit": "GLUPS", "cores": ncores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
        # this process's mapped libraries: the product library must not be among them
        "product_library_loaded": _product_library_loaded(),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--launch", type=int, nargs="+", metavar="N",
                    help="fixed launch choice of the stencil instead of autotuning: z chunk, unroll (1 or 3) "
                         "[, tail chunk, tail planes]")
    ap.add_argument("--workload", choices=[WORKLOAD, "ensemble64", "coarsen512"], default=WORKLOAD)
    ap.add_argument("--no-ensemble", action="store_true", help="leave the ensemble section out of the default line")
    ap.add_argument("--no-fp64", action="store_true", help="leave the FP64 section out of the default line")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("note: warm-up below 3 steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble64":
        run_ensemble(args)
    elif args.workload == "coarsen512":
        run_coarsen(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
