"""The C-ABI library: it loads, exports every function include/*.h
declares, and fails cleanly (no CPU fallback) without a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

import phasefield_coarsening_gb300 as ppf
from conftest import REPO, has_gpu

DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\**\s*\b(ppf_[a-z0-9_]+)\s*\(", re.M)


def declared_functions():
    names = set()
    for h in ("ppf.h", "ppf_h5.h"):
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(DECL.findall(src))
    return sorted(names)


def test_every_declared_function_is_exported():
    names = declared_functions()
    assert "ppf_step" in names and "ppf_h5_read3d" in names
    L = ppf.lib()
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(ppf.EXPORTS) | set(names)


def test_nm_exports_match_header():
    out = subprocess.run(["nm", "-D", "--defined-only", ppf.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln and ln.split()[-1].startswith("ppf_")}
    assert set(declared_functions()) == exported


def test_params_default_are_reference_constants():
    p = ppf.params_default()
    assert (p.AS, p.AL, p.CS, p.CL) == (1e9, 1e9, -1e6, 1e7)
    assert (p.cS0, p.cL0, p.cSeq, p.cLeq) == (0.455, 0.978, 0.999, 0.476)
    assert (p.DL, p.DS, p.sigma, p.gamma, p.dx) == (1e-14, 0.0, 2.0, 1.5, 1.0)


def test_derive_matches_oracle():
    import oracle
    d = ppf.derive().as_dict()
    o = oracle.derive()
    for k, v in o.items():
        assert d[k] == v, k
    d2 = ppf.derive(ppf.params_default(dt=1.5e13)).as_dict()
    assert d2["dt"] == 1.5e13
    assert abs(d["dt_limit"] - 1.0 / 6e-14) < 1e-3


def test_invalid_arguments_are_rejected():
    L = ppf.lib()
    h = ctypes.c_void_p()
    assert L.ppf_create(0, 4, 4, None, 0, 0, ctypes.byref(h)) == -1
    assert b"out of range" in L.ppf_last_error()
    assert L.ppf_create(4, 4, 4, None, 7, 0, ctypes.byref(h)) == -1
    assert L.ppf_create(4, 4, 4, None, 0, 9, ctypes.byref(h)) == -1
    bad = ppf.params_default(dx=0.0)
    assert L.ppf_create(4, 4, 4, ctypes.byref(bad), 0, 0, ctypes.byref(h)) == -1
    assert L.ppf_step(None, 1) == -1
    assert L.ppf_reduce(None, None) == -1


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU failure path")
def test_create_without_gpu_fails_loudly():
    with pytest.raises(ppf.PPFError) as e:
        ppf.Simulation((4, 4, 4))
    assert e.value.code == -2 and "CUDA" in str(e.value) or "device" in str(e.value)


def test_cli_usage_and_exit_code():
    r = subprocess.run([ppf.EXE_PATH], capture_output=True, text=True)
    assert r.returncode == 255 and r.stderr == "Usage:\nppf filename\n"
    r = subprocess.run([ppf.EXE_PATH, "x.h5", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 255 and "Usage" in r.stderr


def test_cli_missing_input_reports_error(tmp_path):
    r = subprocess.run([ppf.EXE_PATH, str(tmp_path / "nothere.h5")], capture_output=True, text=True)
    assert r.returncode == 1
    assert r.stderr.startswith("The job name is " + str(tmp_path / "nothere_"))
    assert "cannot open" in r.stderr
