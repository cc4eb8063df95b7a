"""ppf-gb300: the explicit Moelans multi-phase-field / KKS solute step of
jijn/phasefield_coarsening (phasefield.c:301-476) on NVIDIA GB300.

The product is the C-ABI library built from ``csrc/`` (``include/ppf.h``,
``include/ppf_h5.h``) and the ``ppf`` program.  This module is a thin
ctypes mirror of that boundary for Python callers and tests: it loads the
in-tree ``_build/libppf_gb300.so`` and fails loudly when it is missing.
There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libppf_gb300.so")
EXE_PATH = os.path.join(_PKG, "_build", "ppf")

BC_PERIODIC, BC_NOFLUX = 0, 1
INJECT_NONE, INJECT_STALL_WAIT = 0, 1
F64, F32 = 0, 1
_BC = {"periodic": BC_PERIODIC, "noflux": BC_NOFLUX, BC_PERIODIC: BC_PERIODIC, BC_NOFLUX: BC_NOFLUX}
_PREC = {"f64": F64, "f32": F32, F64: F64, F32: F32}

EXPORTS = (
    "ppf_params_default", "ppf_params_derive", "ppf_create", "ppf_destroy", "ppf_get_dims", "ppf_set_stream",
    "ppf_upload", "ppf_download", "ppf_upload_device", "ppf_download_device", "ppf_step", "ppf_step_c_only",
    "ppf_reduce", "ppf_sync", "ppf_set_wait_limit", "ppf_debug_inject", "ppf_get_tune", "ppf_set_tune",
    "ppf_autotune", "ppf_observe_noalloc", "ppf_particles", "ppf_ensemble_create", "ppf_ensemble_destroy",
    "ppf_ensemble_domain", "ppf_ensemble_upload", "ppf_ensemble_download", "ppf_ensemble_upload_all",
    "ppf_ensemble_download_all", "ppf_ensemble_step",
    "ppf_ensemble_reduce", "ppf_ensemble_sync", "ppf_ensemble_get_tune", "ppf_ensemble_set_tune",
    "ppf_ensemble_autotune", "ppf_slabs_plan", "ppf_slabs_create", "ppf_slabs_destroy", "ppf_slabs_upload",
    "ppf_slabs_download", "ppf_slabs_step", "ppf_slabs_reduce", "ppf_slabs_sync", "ppf_mass_project", "ppf_copy_state", "ppf_surrogate_config_default",
    "ppf_surrogate_create", "ppf_surrogate_destroy", "ppf_surrogate_get_config", "ppf_surrogate_num_params",
    "ppf_surrogate_set_params", "ppf_surrogate_get_params", "ppf_surrogate_loss_grad", "ppf_surrogate_train_step",
    "ppf_surrogate_predict", "ppf_surrogate_advance", "ppf_surrogate_debug_inject", "ppf_measure_fp64_peak",
    "ppf_last_error", "ppf_version",
    "ppf_h5_dims", "ppf_h5_read3d", "ppf_h5_write3d", "ppf_h5_write3d_meta", "ppf_h5_last_error",
)

_PARAM_FIELDS = ("AS", "AL", "CS", "CL", "cS0", "cL0", "cSeq", "cLeq", "DL", "DS", "sigma", "gamma", "dx", "dt", "l")


class Params(ctypes.Structure):
    """ppf_params: the constants of phasefield.c:76-97."""
    _fields_ = [(n, ctypes.c_double) for n in _PARAM_FIELDS]

    def as_dict(self):
        return {n: getattr(self, n) for n in _PARAM_FIELDS}


class Derived(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("ML", "MS", "h2", "dt", "l", "m", "kappa", "L", "dt_limit")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Stats(ctypes.Structure):
    _fields_ = [("sum_dc2", ctypes.c_double), ("sum_detaS2", ctypes.c_double), ("sum_detaL2", ctypes.c_double),
                ("mass", ctypes.c_double), ("solid", ctypes.c_double), ("solid_cells", ctypes.c_double),
                ("free_energy", ctypes.c_double), ("cells", ctypes.c_int64), ("nonfinite", ctypes.c_int64),
                ("steps", ctypes.c_int64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Tune(ctypes.Structure):
    """ppf_tune: launch choices of the fused step."""
    _fields_ = [("zc", ctypes.c_int), ("roll", ctypes.c_int), ("grid", ctypes.c_int), ("pdl", ctypes.c_int),
                ("sched", ctypes.c_int), ("zc2", ctypes.c_int), ("tail", ctypes.c_int), ("split", ctypes.c_int),
                ("tile", ctypes.c_int), ("us_per_step", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class ParticleStats(ctypes.Structure):
    """ppf_particle_stats."""
    _fields_ = [("count", ctypes.c_int64), ("mean_radius", ctypes.c_double), ("solid_volume", ctypes.c_double),
                ("largest_volume", ctypes.c_double), ("interface_area", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class SurrogateConfig(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("k_steps", ctypes.c_int), ("c_solid", ctypes.c_double),
                ("c_liquid", ctypes.c_double), ("in_scale_c", ctypes.c_double),
                ("out_scale", ctypes.c_double * 3), ("loss_weight", ctypes.c_double * 3)]

    def as_dict(self) -> dict:
        return {"width": self.width, "k_steps": self.k_steps, "c_solid": self.c_solid, "c_liquid": self.c_liquid,
                "in_scale_c": self.in_scale_c, "out_scale": list(self.out_scale),
                "loss_weight": list(self.loss_weight)}


class PPFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ppf error {code}: {msg}")
        self.code = code


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library (built by ``build.build()``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with phasefield_coarsening_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.ppf_last_error.restype = ctypes.c_char_p
        L.ppf_version.restype = ctypes.c_char_p
        L.ppf_h5_last_error.restype = ctypes.c_char_p
        L.ppf_params_default.restype = None
        L.ppf_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params), ctypes.c_int,
                                 ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        for n in ("ppf_destroy", "ppf_sync"):
            getattr(L, n).argtypes = [ctypes.c_void_p]
        L.ppf_set_stream.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        for n in ("ppf_upload", "ppf_download", "ppf_upload_device", "ppf_download_device"):
            getattr(L, n).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        for n in ("ppf_step", "ppf_step_c_only"):
            getattr(L, n).argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.ppf_reduce.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats)]
        L.ppf_set_wait_limit.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.ppf_debug_inject.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ppf_get_tune.argtypes = [ctypes.c_void_p, ctypes.POINTER(Tune)]
        L.ppf_set_tune.argtypes = [ctypes.c_void_p, ctypes.POINTER(Tune)]
        L.ppf_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Tune)]
        L.ppf_particles.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ParticleStats),
                                    ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
        L.ppf_get_dims.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 3
        L.ppf_ensemble_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(Params),
                                          ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        for n in ("ppf_ensemble_destroy", "ppf_ensemble_sync"):
            getattr(L, n).argtypes = [ctypes.c_void_p]
        L.ppf_ensemble_domain.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        for n in ("ppf_ensemble_upload", "ppf_ensemble_download"):
            getattr(L, n).argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
        for n in ("ppf_ensemble_upload_all", "ppf_ensemble_download_all"):
            getattr(L, n).argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_void_p)] * 3
        L.ppf_ensemble_step.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.ppf_ensemble_reduce.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Stats)]
        L.ppf_ensemble_get_tune.argtypes = [ctypes.c_void_p, ctypes.POINTER(Tune)]
        L.ppf_ensemble_set_tune.argtypes = [ctypes.c_void_p, ctypes.POINTER(Tune)]
        L.ppf_ensemble_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Tune)]
        L.ppf_slabs_plan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 4
        L.ppf_slabs_create.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(Params), ctypes.c_int, ctypes.c_int,
                                                           ctypes.POINTER(ctypes.c_void_p)]
        for n in ("ppf_slabs_destroy", "ppf_slabs_sync"):
            getattr(L, n).argtypes = [ctypes.c_void_p]
        for n in ("ppf_slabs_upload", "ppf_slabs_download"):
            getattr(L, n).argtypes = [ctypes.c_void_p] * 4
        L.ppf_slabs_step.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.ppf_slabs_reduce.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats)]
        L.ppf_mass_project.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.ppf_copy_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ppf_surrogate_config_default.argtypes = [ctypes.POINTER(SurrogateConfig)]
        L.ppf_surrogate_config_default.restype = None
        L.ppf_surrogate_create.argtypes = [ctypes.POINTER(SurrogateConfig), ctypes.POINTER(ctypes.c_void_p)]
        L.ppf_surrogate_destroy.argtypes = [ctypes.c_void_p]
        L.ppf_surrogate_get_config.argtypes = [ctypes.c_void_p, ctypes.POINTER(SurrogateConfig)]
        L.ppf_surrogate_num_params.argtypes = [ctypes.c_void_p]
        L.ppf_surrogate_num_params.restype = ctypes.c_int64
        for n in ("ppf_surrogate_set_params", "ppf_surrogate_get_params"):
            getattr(L, n).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
        L.ppf_surrogate_loss_grad.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_int64]
        L.ppf_surrogate_train_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                               ctypes.POINTER(ctypes.c_double)]
        L.ppf_surrogate_predict.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.ppf_surrogate_advance.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.ppf_surrogate_debug_inject.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ppf_measure_fp64_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]
        L.ppf_h5_dims.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]
        L.ppf_h5_read3d.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64), _dp,
                                    ctypes.c_int64]
        L.ppf_h5_write3d.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                     ctypes.POINTER(_dp), ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int64)]
        L.ppf_h5_write3d_meta.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                          ctypes.POINTER(_dp), ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_int64), ctypes.c_char_p, _dp, ctypes.c_int]
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        raise PPFError(rc, lib().ppf_last_error().decode(errors="replace"))


def params_default(**overrides) -> Params:
    p = Params()
    lib().ppf_params_default(ctypes.byref(p))
    for k, v in overrides.items():
        setattr(p, k, float(v))
    return p


def derive(p: Params | None = None) -> Derived:
    p = p if p is not None else params_default()
    d = Derived()
    _check(lib().ppf_params_derive(ctypes.byref(p), ctypes.byref(d)))
    return d


def _c64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Simulation:
    """Host-side mirror of a ppf_ctx (include/ppf.h): one grid, three
    fields, stepped on the current CUDA device."""

    def __init__(self, shape, params: Params | None = None, bc="periodic", precision="f64"):
        nz, ny, nx = (int(s) for s in shape)
        self.shape = (nz, ny, nx)
        self.params = params if params is not None else params_default()
        self.bc = _BC[bc]
        self.precision = _PREC[precision]
        h = ctypes.c_void_p()
        _check(lib().ppf_create(nz, ny, nx, ctypes.byref(self.params), self.bc, self.precision, ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().ppf_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_ptr: int | None):
        _check(lib().ppf_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def upload(self, etaS, etaL, c):
        a = [_c64(x) for x in (etaS, etaL, c)]
        for x in a:
            if x.shape != self.shape:
                raise ValueError(f"field shape {x.shape} != grid {self.shape}")
        _check(lib().ppf_upload(self._h, *[x.ctypes.data for x in a]))

    def upload_device(self, ptrs):
        _check(lib().ppf_upload_device(self._h, *[ctypes.c_void_p(int(p)) for p in ptrs]))

    def download(self):
        out = [np.empty(self.shape, np.float64) for _ in range(3)]
        _check(lib().ppf_download(self._h, *[x.ctypes.data for x in out]))
        return tuple(out)

    def download_into(self, etaS, etaL, c):
        _check(lib().ppf_download(self._h, *[ctypes.c_void_p(int(p)) for p in (etaS, etaL, c)]))

    def upload_from(self, etaS, etaL, c):
        """Upload from raw host pointers (e.g. pinned buffers)."""
        _check(lib().ppf_upload(self._h, *[ctypes.c_void_p(int(p)) for p in (etaS, etaL, c)]))

    def step(self, n: int = 1):
        _check(lib().ppf_step(self._h, int(n)))

    def step_c_only(self, n: int = 1):
        _check(lib().ppf_step_c_only(self._h, int(n)))

    def sync(self):
        _check(lib().ppf_sync(self._h))

    def set_wait_limit(self, seconds: float):
        _check(lib().ppf_set_wait_limit(self._h, float(seconds)))

    def debug_inject(self, fault: int):
        _check(lib().ppf_debug_inject(self._h, int(fault)))

    def get_tune(self) -> dict:
        t = Tune()
        _check(lib().ppf_get_tune(self._h, ctypes.byref(t)))
        return t.as_dict()

    def set_tune(self, zc: int, roll: int = 1, pdl: int = 1, sched: int = 1, zc2: int = 0, tail: int = 0,
                 split: int = 1, tile: int = 0):
        t = Tune(int(zc), int(roll), 0, int(pdl), int(sched), int(zc2), int(tail), int(split), int(tile), 0.0)
        _check(lib().ppf_set_tune(self._h, ctypes.byref(t)))

    def particles(self, threshold: float = 0.5, volumes: bool = False) -> dict:
        """Particles of etaS > threshold: count, mean radius R-bar, ...;
        with volumes=True also the sorted particle volumes (cells)."""
        st = ParticleStats()
        n = ctypes.c_int64(0)
        if volumes:
            cap = int(np.prod(self.shape)) // 2 + 1
            buf = np.zeros(cap, dtype=np.int64)
            _check(lib().ppf_particles(self._h, float(threshold), ctypes.byref(st), buf.ctypes.data, cap,
                                       ctypes.byref(n)))
            d = st.as_dict()
            d["volumes"] = np.sort(buf[:min(n.value, cap)])
            return d
        _check(lib().ppf_particles(self._h, float(threshold), ctypes.byref(st), None, 0, ctypes.byref(n)))
        return st.as_dict()

    def autotune(self, trial_steps: int = 10) -> dict:
        t = Tune()
        _check(lib().ppf_autotune(self._h, int(trial_steps), ctypes.byref(t)))
        return t.as_dict()

    def reduce(self) -> dict:
        s = Stats()
        _check(lib().ppf_reduce(self._h, ctypes.byref(s)))
        return s.as_dict()

    def mass_project(self, target_mass: float):
        """Set sum(c) to target_mass (FP32 states; FP64 arithmetic)."""
        _check(lib().ppf_mass_project(self._h, float(target_mass)))

    def copy_from(self, other: "Simulation"):
        """This state := other's current state (same shape, precision, BC)."""
        _check(lib().ppf_copy_state(self._h, other._h))


class Surrogate:
    """Host-side mirror of a ppf_surrogate: the learned k-step network
    (six 3x3x3 convolutions, BF16 tensor-core kernels), its training on the
    device, and its use as a time stepper with FP64 mass projection."""

    def __init__(self, width: int = 32, k_steps: int = 50, **overrides):
        cfg = SurrogateConfig()
        lib().ppf_surrogate_config_default(ctypes.byref(cfg))
        cfg.width = int(width)
        cfg.k_steps = int(k_steps)
        for k, v in overrides.items():
            if k in ("out_scale", "loss_weight"):
                setattr(cfg, k, (ctypes.c_double * 3)(*[float(x) for x in v]))
            else:
                setattr(cfg, k, v)
        h = ctypes.c_void_p()
        _check(lib().ppf_surrogate_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().ppf_surrogate_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def config(self) -> dict:
        c = SurrogateConfig()
        _check(lib().ppf_surrogate_get_config(self._h, ctypes.byref(c)))
        return c.as_dict()

    @property
    def num_params(self) -> int:
        return int(lib().ppf_surrogate_num_params(self._h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        _check(lib().ppf_surrogate_get_params(self._h, out.ctypes.data, out.size))
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(lib().ppf_surrogate_set_params(self._h, p.ctypes.data, p.size))

    def loss_grad(self, inp: Simulation, tgt: Simulation):
        g = np.empty(self.num_params, np.float32)
        loss = ctypes.c_double()
        _check(lib().ppf_surrogate_loss_grad(self._h, inp._h, tgt._h, ctypes.byref(loss), g.ctypes.data, g.size))
        return loss.value, g

    def train_step(self, inp: Simulation, tgt: Simulation, lr: float = 1e-3, want_loss: bool = True):
        loss = ctypes.c_double()
        _check(lib().ppf_surrogate_train_step(self._h, inp._h, tgt._h, float(lr),
                                              ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def predict(self, sim: Simulation):
        """Predicted change of (etaS, etaL, c) over k_steps (float64, [z][y][x] each)."""
        out = np.empty((3,) + tuple(sim.shape), np.float64)
        _check(lib().ppf_surrogate_predict(self._h, sim._h, out.ctypes.data))
        return out

    def advance(self, sim: Simulation, ncalls: int = 1):
        _check(lib().ppf_surrogate_advance(self._h, sim._h, int(ncalls)))

    def debug_inject(self, fault: int = INJECT_STALL_WAIT):
        _check(lib().ppf_surrogate_debug_inject(self._h, int(fault)))


class Ensemble:
    """Host-side mirror of a ppf_ensemble: independent domains of different
    sizes stepped together by one persistent launch per time step."""

    def __init__(self, shapes, params: Params | None = None, bc="periodic", precision="f32"):
        self.shapes = [tuple(int(v) for v in sh) for sh in shapes]
        self.params = params if params is not None else params_default()
        dims = (ctypes.c_int * (3 * len(self.shapes)))(*[v for sh in self.shapes for v in sh])
        h = ctypes.c_void_p()
        _check(lib().ppf_ensemble_create(len(self.shapes), dims, ctypes.byref(self.params), _BC[bc], _PREC[precision],
                                         ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().ppf_ensemble_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        """The ppf_ensemble* handle for direct C-ABI calls."""
        return self._h

    def __len__(self):
        return len(self.shapes)

    def upload(self, d, etaS, etaL, c):
        a = [_c64(x) for x in (etaS, etaL, c)]
        if any(x.shape != self.shapes[d] for x in a):
            raise ValueError("field shape does not match the domain")
        _check(lib().ppf_ensemble_upload(self._h, int(d), *[x.ctypes.data for x in a]))

    def download(self, d):
        out = [np.empty(self.shapes[d], np.float64) for _ in range(3)]
        _check(lib().ppf_ensemble_download(self._h, int(d), *[x.ctypes.data for x in out]))
        return tuple(out)

    @staticmethod
    def _ptr_arrays(ptrs):
        # ptrs: per domain (etaS, etaL, c) addresses -> three C arrays of pointers
        n = len(ptrs)
        return [(ctypes.c_void_p * n)(*[int(p[f]) for p in ptrs]) for f in range(3)]

    def upload_from_all(self, ptrs):
        """Every domain from raw host pointers (e.g. pinned buffers) in one
        call: ptrs[d] = (etaS, etaL, c) addresses of domain d."""
        if len(ptrs) != len(self.shapes):
            raise ValueError("one (etaS, etaL, c) triple per domain")
        _check(lib().ppf_ensemble_upload_all(self._h, *self._ptr_arrays(ptrs)))

    def download_into_all(self, ptrs):
        if len(ptrs) != len(self.shapes):
            raise ValueError("one (etaS, etaL, c) triple per domain")
        _check(lib().ppf_ensemble_download_all(self._h, *self._ptr_arrays(ptrs)))

    def upload_all(self, states):
        """Every domain in one call: states[d] = (etaS, etaL, c)."""
        arrs = [[_c64(x) for x in st] for st in states]
        for d, a in enumerate(arrs):
            if any(x.shape != self.shapes[d] for x in a):
                raise ValueError(f"field shape of domain {d} does not match")
        self.upload_from_all([[x.ctypes.data for x in a] for a in arrs])

    def download_all(self):
        out = [tuple(np.empty(s, np.float64) for _ in range(3)) for s in self.shapes]
        self.download_into_all([[x.ctypes.data for x in o] for o in out])
        return out

    def step(self, n=1):
        _check(lib().ppf_ensemble_step(self._h, int(n)))

    def sync(self):
        _check(lib().ppf_ensemble_sync(self._h))

    def reduce(self, d) -> dict:
        s = Stats()
        _check(lib().ppf_ensemble_reduce(self._h, int(d), ctypes.byref(s)))
        return s.as_dict()

    def particles(self, d, threshold=0.5) -> dict:
        ctx = ctypes.c_void_p()
        _check(lib().ppf_ensemble_domain(self._h, int(d), ctypes.byref(ctx)))
        st = ParticleStats()
        _check(lib().ppf_particles(ctx, float(threshold), ctypes.byref(st), None, 0, None))
        return st.as_dict()

    def get_tune(self) -> dict:
        t = Tune()
        _check(lib().ppf_ensemble_get_tune(self._h, ctypes.byref(t)))
        return t.as_dict()

    def set_tune(self, zc: int, roll: int = 1, sched: int = 1, pdl: int = 1, split: int = 0, tile: int = 0):
        t = Tune(int(zc), int(roll), 0, int(pdl), int(sched), 0, 0, int(split), int(tile), 0.0)
        _check(lib().ppf_ensemble_set_tune(self._h, ctypes.byref(t)))

    def autotune(self, trial_steps: int = 5) -> dict:
        t = Tune()
        _check(lib().ppf_ensemble_autotune(self._h, int(trial_steps), ctypes.byref(t)))
        return t.as_dict()


def slabs_plan(nz: int, nslabs: int, bc="periodic") -> dict:
    """ppf_slabs_plan: {z0, nz, lower, upper} lists (no device needed)."""
    arrs = [(ctypes.c_int * nslabs)() for _ in range(4)]
    _check(lib().ppf_slabs_plan(int(nz), int(nslabs), _BC[bc], *arrs))
    return {k: list(a) for k, a in zip(("z0", "nz", "lower", "upper"), arrs)}


class Slabs:
    """Host-side mirror of a ppf_slabs: one domain as z slabs (one context
    each) with a ghost-plane exchange per step."""

    def __init__(self, shape, nslabs, params: Params | None = None, bc="periodic", precision="f64"):
        nz, ny, nx = (int(v) for v in shape)
        self.shape = (nz, ny, nx)
        self.params = params if params is not None else params_default()
        h = ctypes.c_void_p()
        _check(lib().ppf_slabs_create(nz, ny, nx, int(nslabs), ctypes.byref(self.params), _BC[bc], _PREC[precision],
                                      ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().ppf_slabs_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload(self, etaS, etaL, c):
        a = [_c64(x) for x in (etaS, etaL, c)]
        if any(x.shape != self.shape for x in a):
            raise ValueError("field shape does not match the domain")
        _check(lib().ppf_slabs_upload(self._h, *[x.ctypes.data for x in a]))

    def download(self):
        out = [np.empty(self.shape, np.float64) for _ in range(3)]
        _check(lib().ppf_slabs_download(self._h, *[x.ctypes.data for x in out]))
        return tuple(out)

    def step(self, n=1):
        _check(lib().ppf_slabs_step(self._h, int(n)))

    def sync(self):
        _check(lib().ppf_slabs_sync(self._h))

    def reduce(self) -> dict:
        s = Stats()
        _check(lib().ppf_slabs_reduce(self._h, ctypes.byref(s)))
        return s.as_dict()


def measure_fp64_peak() -> float:
    """The current device's FP64 FMA rate, TFLOP/s (roofline of the FP64 step)."""
    v = ctypes.c_double()
    _check(lib().ppf_measure_fp64_peak(ctypes.byref(v)))
    return v.value


# ---------------------------------------------------------------- HDF5 ----

def h5_dims(path: str, name: str):
    d = (ctypes.c_int64 * 3)()
    rc = lib().ppf_h5_dims(path.encode(), name.encode(), d)
    if rc != 0:
        raise PPFError(rc, lib().ppf_h5_last_error().decode())
    return tuple(d)


def h5_read(path: str, name: str) -> np.ndarray:
    dims = h5_dims(path, name)
    out = np.empty(dims, np.float64)
    d = (ctypes.c_int64 * 3)()
    rc = lib().ppf_h5_read3d(path.encode(), name.encode(), d, out.ctypes.data_as(_dp), out.size)
    if rc != 0:
        raise PPFError(rc, lib().ppf_h5_last_error().decode())
    return out


def h5_write(path: str, fields: dict, dtype="f64", chunk=None, meta=None):
    """Rank-3 datasets of one shape; `meta` = (name, values) adds one float64
    dataset of shape (1, 1, len(values)) (the program's restart record)."""
    names = list(fields)
    arrs = [_c64(fields[n]) for n in names]
    shape = arrs[0].shape
    if any(a.shape != shape or a.ndim != 3 for a in arrs):
        raise ValueError("all datasets must be rank-3 and of one shape")
    cn = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
    cp = (_dp * len(arrs))(*[a.ctypes.data_as(_dp) for a in arrs])
    dims = (ctypes.c_int64 * 3)(*shape)
    ch = (ctypes.c_int64 * 3)(*chunk) if chunk is not None else None
    if meta is None:
        rc = lib().ppf_h5_write3d(path.encode(), len(names), cn, cp, dims, 0 if dtype == "f64" else 1, ch)
    else:
        mv = _c64(np.asarray(meta[1], dtype=np.float64).ravel())
        rc = lib().ppf_h5_write3d_meta(path.encode(), len(names), cn, cp, dims, 0 if dtype == "f64" else 1, ch,
                                       meta[0].encode(), mv.ctypes.data_as(_dp), mv.size)
    if rc != 0:
        raise PPFError(rc, lib().ppf_h5_last_error().decode())


def read_fields(path: str):
    return tuple(h5_read(path, n) for n in ("/etaS", "/etaL", "/c"))


def write_fields(path: str, etaS, etaL, c, dtype="f64", chunk=None):
    h5_write(path, {"etaS": etaS, "etaL": etaL, "c": c}, dtype=dtype, chunk=chunk)


__all__ = ["Simulation", "Ensemble", "Slabs", "slabs_plan", "Params", "Stats", "Derived", "PPFError", "params_default", "derive", "lib",
           "h5_read", "h5_write", "h5_dims", "read_fields", "write_fields", "BC_PERIODIC", "BC_NOFLUX",
           "F64", "F32", "LIB_PATH", "EXE_PATH", "EXPORTS"]
