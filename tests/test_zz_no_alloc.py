"""ppf_observe_noalloc: the observables for callers that may not allocate
device memory (a hook inside an application whose device memory belongs to
the application's own pool).  Checked through the C-ABI against
ppf_reduce's observables of the same state, on two calls in a row (the
second on a different grid and BC, so stale partial sums would show)."""
import ctypes

import numpy as np
import pytest

import phasefield_coarsening_gb300 as ppf
from helpers import smooth_state

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    L = ppf.lib()
    f = L.ppf_observe_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ppf.Params), ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _reference_and_device_state(shape, bc, seed):
    """ppf_reduce's observables after 4 steps, and the same state in
    caller-owned device buffers (allocated here, by the test)."""
    import torch
    st = smooth_state(shape, seed=seed)
    dev = [torch.empty(shape, dtype=torch.float64, device="cuda") for _ in range(3)]
    with ppf.Simulation(shape, bc=bc, precision="f64") as s:
        s.upload(*st)
        s.step(4)
        torch.cuda.synchronize()
        ppf.lib().ppf_download_device(s.handle, *[ctypes.c_void_p(t.data_ptr()) for t in dev])
        ref = s.reduce()
    return ref, dev


def _check(ref, out):
    mass, solid, cells, energy, bad = out
    assert abs(mass - ref["mass"]) <= 1e-13 * abs(ref["mass"])
    assert abs(solid - ref["solid"]) <= 1e-12 * abs(ref["solid"])
    assert cells == ref["solid_cells"] and bad == ref["nonfinite"] == 0
    assert abs(energy - ref["free_energy"]) <= 1e-12 * abs(ref["free_energy"])


def test_observe_noalloc_matches_ppf_reduce_twice():
    import torch
    f = _noalloc_fn()
    prm = ppf.params_default()
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for shape, bc, seed in [((24, 30, 70), ppf.BC_PERIODIC, 3), ((9, 41, 33), ppf.BC_NOFLUX, 4)]:
        ref, dev = _reference_and_device_state(shape, bc, seed)
        out.fill_(-1.0)
        rc = f(shape[0], shape[1], shape[2], ctypes.byref(prm), bc, *[t.data_ptr() for t in dev],
               out.data_ptr(), stream)
        assert rc == 0, ppf.lib().ppf_last_error()
        torch.cuda.synchronize()
        _check(ref, out.cpu().numpy().tolist())


def test_observe_noalloc_rejects_grids_beyond_its_scratch():
    f = _noalloc_fn()
    prm = ppf.params_default()
    fake = ctypes.c_void_p(0x1000)     # never dereferenced: the size check comes first
    rc = f(1024, 1024, 129, ctypes.byref(prm), 0, fake, fake, fake, fake, None)
    assert rc == -1
    assert b"allocation-free limit" in ppf.lib().ppf_last_error()
