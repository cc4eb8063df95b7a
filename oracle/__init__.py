"""ORACLE -- test infrastructure, not product code.

ctypes access to the CPU restatement of the reference step
(oracle/ppf_oracle.c, built into oracle/_build/libppf_oracle.so), to the
oracle's own HDF5 subset (oracle/hdf5_shim/h5ref.c, independent of the
product's HDF5 code) and to the patched reference build recipe
(oracle/build_ref.py).  Only tests/, the smoke check and bench.py's CPU
baseline and reference arm import this package.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libppf_oracle.so")

_PARAM_FIELDS = ("AS", "AL", "CS", "CL", "cS0", "cL0", "cSeq", "cLeq", "DL", "DS", "sigma", "gamma", "dx", "dt", "l")


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in _PARAM_FIELDS]


class Derived(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("ML", "MS", "h2", "dt", "l", "m", "kappa", "L", "dt_limit")]


def reference_params(**over) -> Params:
    """phasefield.c:76-97 (dt=0 / l=0 select the reference's formulas)."""
    v = dict(AS=1e9, AL=1e9, CS=-1e6, CL=1e7, cS0=0.455, cL0=0.978, cSeq=0.999, cLeq=0.476, DL=1e-14, DS=0.0,
             sigma=2.0, gamma=1.5, dx=1.0, dt=0.0, l=0.0)
    v.update(over)
    return Params(*[float(v[n]) for n in _PARAM_FIELDS])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} missing: run phasefield_coarsening_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.ppf_oracle_run.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                                          ctypes.c_int64] + [ctypes.c_void_p] * 4
        L.ppf_oracle_observe.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4
        L.ppf_oracle_particles.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                                               ctypes.c_void_p, ctypes.c_int64]
        L.ppf_oracle_derive.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ppf_oracle_derive.restype = None
        L.h5ref_write.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                  ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_int64)]
        L.h5ref_dims.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]
        L.h5ref_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64]
        L.h5ref_list.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int64)]
        L.h5ref_read_any.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64,
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int64)]
        L.h5ref_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _as_params(p):
    if p is None:
        return reference_params()
    if isinstance(p, Params):
        return p
    return Params(*[float(getattr(p, n)) for n in _PARAM_FIELDS])


def derive(p=None) -> dict:
    d = Derived()
    lib().ppf_oracle_derive(ctypes.byref(_as_params(p)), ctypes.byref(d))
    return {n: getattr(d, n) for n, _ in d._fields_}


def run(etaS, etaL, c, nsteps, bc=0, params=None, n_iter_init=1 << 62):
    """nsteps iterations of the reference loop body; returns (etaS, etaL, c, sums)."""
    a = [np.array(x, dtype=np.float64, order="C", copy=True) for x in (etaS, etaL, c)]
    nz, ny, nx = a[0].shape
    sums = np.zeros(3)
    p = _as_params(params)
    rc = lib().ppf_oracle_run(nz, ny, nx, ctypes.byref(p), int(bc), int(nsteps), int(n_iter_init),
                              *[x.ctypes.data for x in a], sums.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle run failed ({rc})")
    return a[0], a[1], a[2], sums


def observe(etaS, etaL, c, bc=0, params=None) -> dict:
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (etaS, etaL, c)]
    nz, ny, nx = a[0].shape
    out = np.zeros(5)
    p = _as_params(params)
    rc = lib().ppf_oracle_observe(nz, ny, nx, ctypes.byref(p), int(bc), *[x.ctypes.data for x in a],
                                  out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle observe failed ({rc})")
    return {"mass": out[0], "solid": out[1], "solid_cells": out[2], "free_energy": out[3], "nonfinite": out[4]}


def particles(etaS, bc=0, threshold=0.5) -> dict:
    """Particles of etaS > threshold (6-connected, periodic wrap for bc=0)."""
    a = np.ascontiguousarray(etaS, dtype=np.float64)
    nz, ny, nx = a.shape
    out = np.zeros(5)
    cap = a.size
    vols = np.zeros(cap, dtype=np.int64)
    rc = lib().ppf_oracle_particles(nz, ny, nx, int(bc), a.ctypes.data, float(threshold), out.ctypes.data,
                                    vols.ctypes.data, cap)
    if rc != 0:
        raise RuntimeError(f"oracle particles failed ({rc})")
    n = int(out[0])
    return {"count": n, "mean_radius": out[1] / n if n else 0.0, "solid_volume": out[2],
            "largest_volume": out[3], "interface_area": out[4], "volumes": np.sort(vols[:n])}


# ------------------------------------------------ the oracle's HDF5 subset --

class H5Error(RuntimeError):
    pass


def _h5check(rc):
    if rc != 0:
        raise H5Error(f"h5ref error {rc}: {lib().h5ref_error().decode(errors='replace')}")


def h5_write(path, fields: dict, float32=False, chunk=None):
    """Rank-3 datasets of one shape, float64 (or float32) little endian,
    contiguous or chunked (full-size edge chunks)."""
    names = list(fields)
    arrs = [np.ascontiguousarray(fields[n], dtype=np.float64) for n in names]
    shape = arrs[0].shape
    if any(a.ndim != 3 or a.shape != shape for a in arrs):
        raise ValueError("all datasets must be rank-3 and of one shape")
    cn = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
    cp = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    dims = (ctypes.c_int64 * 3)(*shape)
    ch = (ctypes.c_int64 * 3)(*chunk) if chunk is not None else None
    _h5check(lib().h5ref_write(str(path).encode(), len(names), cn, cp, dims, int(bool(float32)), ch))


def h5_read(path, name) -> np.ndarray:
    d = (ctypes.c_int64 * 3)()
    _h5check(lib().h5ref_dims(str(path).encode(), name.encode(), d))
    out = np.empty(tuple(d), np.float64)
    _h5check(lib().h5ref_read(str(path).encode(), name.encode(), out.ctypes.data, out.size))
    return out


def h5_list(path):
    """[(name, rank, dims)] of the objects in the root group."""
    out = []
    for i in range(1 << 16):
        name = ctypes.create_string_buffer(256)
        rank = ctypes.c_int(0)
        dims = (ctypes.c_int64 * 3)()
        rc = lib().h5ref_list(str(path).encode(), i, name, 256, ctypes.byref(rank), dims)
        if rc == -3:
            break
        _h5check(rc)
        out.append((name.value.decode(), rank.value, tuple(dims)))
    return out


def h5_read_any(path, name, capacity=1 << 20) -> np.ndarray:
    """A rank 1-3 contiguous float dataset of any HDF5 file, as stored."""
    out = np.empty(capacity, np.float64)
    rank = ctypes.c_int(0)
    dims = (ctypes.c_int64 * 3)()
    _h5check(lib().h5ref_read_any(str(path).encode(), name.encode(), out.ctypes.data, capacity, ctypes.byref(rank),
                                  dims))
    shape = tuple(dims)[:rank.value]
    return out[:int(np.prod(shape))].reshape(shape).copy()


def write_fields(path, etaS, etaL, c, chunk=None):
    h5_write(path, {"etaS": etaS, "etaL": etaL, "c": c}, chunk=chunk)


def read_fields(path):
    return tuple(h5_read(path, n) for n in ("/etaS", "/etaL", "/c"))
