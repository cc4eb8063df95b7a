"""The slab decomposition's plan and exchange schedule on CPU, with two gloo
ranks standing in for two devices: each rank owns the slabs the plan deals
it, steps them with the oracle (a slab plus one ghost plane per side), and
trades boundary planes with isend/irecv after every step the way the
reference's MPI halo exchange does (phasefield.c:683-708).  The gathered
result must equal the oracle on the undivided domain bit for bit."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from helpers import smooth_state  # noqa: E402

SHAPE = (11, 6, 7)
STEPS = 6


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, nslabs, bc, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        import phasefield_coarsening_gb300 as ppf
        plan = ppf.slabs_plan(SHAPE[0], nslabs, bc)      # the C-ABI's partitioner (no device needed)
        full = smooth_state(SHAPE, seed=31)
        mine = [k for k in range(nslabs) if k % world == rank]
        owner = {k: k % world for k in range(nslabs)}
        slab = {k: [f[plan["z0"][k]:plan["z0"][k] + plan["nz"][k]].copy() for f in full] for k in mine}
        bcn = 0 if bc == "periodic" else 1
        for _ in range(STEPS):
            # ghost planes: the neighbour's boundary plane, or the slab's own (no-flux end)
            ghosts = {}
            reqs, inbox = [], {}
            for k in mine:
                for side, nb in (("lo", plan["lower"][k]), ("hi", plan["upper"][k])):
                    if nb < 0:
                        ghosts[(k, side)] = [f[0] if side == "lo" else f[-1] for f in slab[k]]
                    elif owner[nb] == rank:
                        ghosts[(k, side)] = [f[-1] if side == "lo" else f[0] for f in slab[nb]]
                    else:
                        buf = torch.empty((3,) + SHAPE[1:], dtype=torch.float64)
                        inbox[(k, side)] = buf
                        reqs.append(dist.irecv(buf, src=owner[nb], tag=2 * k + (side == "hi")))
            for k in mine:
                # the planes this slab gives: its top to its upper neighbour's lower ghost, its bottom to the lower's upper
                for nb, plane, tag in ((plan["upper"][k], -1, lambda j: 2 * j), (plan["lower"][k], 0, lambda j: 2 * j + 1)):
                    if nb >= 0 and owner[nb] != rank:
                        t = torch.from_numpy(np.stack([f[plane] for f in slab[k]]).copy())
                        reqs.append(dist.isend(t, dst=owner[nb], tag=tag(nb)))
            for r in reqs:
                r.wait()
            for key, buf in inbox.items():
                ghosts[key] = list(buf.numpy())
            for k in mine:
                ext = [np.concatenate([g_lo[None], f, g_hi[None]])
                       for f, g_lo, g_hi in zip(slab[k], ghosts[(k, "lo")], ghosts[(k, "hi")])]
                out = oracle.run(*ext, 1, bc=bcn)
                slab[k] = [o[1:-1].copy() for o in out[:3]]
        q.put((rank, {k: [f.tobytes() for f in v] for k, v in slab.items()}))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("nslabs", [2, 3, 4])
@pytest.mark.parametrize("bc", ["periodic", "noflux"])
def test_two_ranks_exchanging_ghost_planes_equal_the_undivided_domain(nslabs, bc):
    import oracle
    import phasefield_coarsening_gb300 as ppf
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, nslabs, bc, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(2):
        _, part = q.get(timeout=180)
        got.update(part)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    plan = ppf.slabs_plan(SHAPE[0], nslabs, bc)
    full = smooth_state(SHAPE, seed=31)
    ref = oracle.run(*full, STEPS, bc=0 if bc == "periodic" else 1)
    for k in range(nslabs):
        z0, n = plan["z0"][k], plan["nz"][k]
        for f, r in zip(got[k], ref[:3]):
            assert np.frombuffer(f, dtype=np.float64).reshape((n,) + SHAPE[1:]).tobytes() == r[z0:z0 + n].tobytes()


def test_plan_is_balanced_and_wraps_only_when_periodic():
    import phasefield_coarsening_gb300 as ppf
    for nz in (1, 7, 64, 257):
        for n in range(1, min(nz, 9) + 1):
            for bc in ("periodic", "noflux"):
                p = ppf.slabs_plan(nz, n, bc)
                assert sum(p["nz"]) == nz and max(p["nz"]) - min(p["nz"]) <= 1
                assert p["z0"] == [sum(p["nz"][:k]) for k in range(n)]
                per = bc == "periodic" and n > 1
                assert p["lower"][0] == (n - 1 if per else -1) and p["upper"][-1] == (0 if per else -1)
                assert all(p["lower"][k] == k - 1 for k in range(1, n))
                assert all(p["upper"][k] == k + 1 for k in range(n - 1))
    with pytest.raises(ppf.PPFError):
        ppf.slabs_plan(4, 5, "periodic")
