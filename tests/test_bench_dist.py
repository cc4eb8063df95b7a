"""bench.py's multi-rank host logic on CPU with two gloo ranks: the job time
is the slowest rank's, the whole-job value counts every replica, and the
reference arm's non-zero ranks exit without work."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 + rank)          # rank 1 is the slow one
        v = bench.job_glups(world, 1000, 10, t)
        q.put((rank, t, v))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_value_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, v in got:
        assert t == 2.5                               # both ranks see the slowest time
        assert v == pytest.approx(2 * 1000 * 10 / 2.5 / 1e9)


def test_single_process_needs_no_process_group():
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.job_glups(1, 16777216, 100, 0.0125) == pytest.approx(134.217728)


def test_reference_arm_nonzero_rank_exits_without_work(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, seed = 1, 0, 0
    assert bench.run_reference(A()) is None
    assert capsys.readouterr().out == ""


def test_reference_arm_falls_back_to_the_oracle_port(monkeypatch, capsys):
    """Without the reference's sources or a patched unit, --impl reference
    times the oracle restatement and says so (kind "port")."""
    import json

    import oracle.build_ref as br
    from phasefield_coarsening_gb300 import ic
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")

    def no_build(**kw):
        raise FileNotFoundError("reference sources absent")
    monkeypatch.setattr(br, "build", no_build)
    small = ic.workload("spheres64_uniform4to8", seed=0)
    monkeypatch.setattr(ic, "workload", lambda name, seed=0, shape=None: small)

    class A:
        steps, warmup, seed = 2, 1, 0
    bench.run_reference(A())
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "port"
    assert line["value"] > 0 and line["unit"] == "GLUPS" and line["e2e"]["h2d_bytes_per_step"] == 0
