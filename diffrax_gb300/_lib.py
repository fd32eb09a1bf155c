"""ctypes binding of libgbdx.so (include/gbdx.h).

The library is the only execution path: if it cannot be built or loaded, or no
CUDA device is present, every solve raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import math
import os
import threading

from . import _build

_c = ctypes
i32, i64, f64, u64 = _c.c_int32, _c.c_int64, _c.c_double, _c.c_uint64
vp = _c.c_void_p
dp = _c.POINTER(_c.c_double)
ip = _c.POINTER(_c.c_int32)


class ProblemDesc(_c.Structure):
    """Mirror of gbdx_problem_desc."""
    _fields_ = [
        ("solver", i32), ("controller", i32), ("field", i32), ("dim", i32),
        ("rtol", f64), ("atol", f64), ("pcoeff", f64), ("icoeff", f64),
        ("dcoeff", f64), ("safety", f64), ("factormin", f64), ("factormax", f64),
        ("dtmin", f64), ("dtmax", f64), ("force_dtmin", i32), ("error_order", f64),
        ("n_ts", i32), ("save_t0", i32), ("save_t1", i32), ("max_steps", i32),
        ("n_args", i32), ("mlp_depth", i32), ("mlp_widths", i32 * 9), ("diffusion", i32),
        ("vbt_t0", f64), ("vbt_t1", f64), ("vbt_tol", f64), ("seed", u64),
        ("norm", i32), ("schedule", i32),
        ("dtype", i32), ("kernel", i32), ("adjoint", i32), ("checkpoints", i32),
        ("block_threads", i32), ("ctas_per_sm", i32), ("mlp_precision", i32),
        ("save_steps", i32), ("save_dense", i32), ("n_step_ts", i32), ("n_jump_ts", i32),
        ("n_event", i32), ("event_root", i32), ("ev_kind", i32 * 4), ("ev_dir", i32 * 4),
        ("levy_area", i32), ("newton_rtol", f64), ("newton_atol", f64), ("ev_coef", f64 * 24),
    ]


class FwdExtras(_c.Structure):
    """Mirror of gbdx_fwd_extras."""
    _fields_ = [("dense_ts", vp), ("dense_info", vp), ("dense_n", vp), ("event_index", vp),
                ("state_in", vp), ("state_out", vp)]


_lock = threading.Lock()
_LIB = None


def bounds_requested() -> bool:
    """GBDX_BOUNDS=1 selects the bounds-checked library (libgbdx_bounds.so)."""
    return os.environ.get("GBDX_BOUNDS", "0") not in ("", "0")


def load():
    """Build (when stale) and load libgbdx.so -- libgbdx_bounds.so under
    GBDX_BOUNDS=1; raise loudly on failure."""
    global _LIB
    with _lock:
        if _LIB is not None:
            return _LIB
        bounds = bounds_requested()
        path = _build.BOUNDS_LIB_PATH if bounds else _build.LIB_PATH
        if _build.is_stale(bounds):
            path = _build.build(bounds=bounds)
        if not os.path.exists(path):
            raise RuntimeError(f"{os.path.basename(path)} is missing at {path}")
        lib = _c.CDLL(path)
        lib.gbdx_problem_create.argtypes = [_c.POINTER(ProblemDesc), _c.POINTER(vp)]
        lib.gbdx_problem_create.restype = i32
        lib.gbdx_problem_destroy.argtypes = [vp]
        lib.gbdx_problem_destroy.restype = i32
        lib.gbdx_num_saves.argtypes = [vp]
        lib.gbdx_num_saves.restype = i32
        lib.gbdx_workspace_size.argtypes = [vp, i64]
        lib.gbdx_workspace_size.restype = _c.c_size_t
        lib.gbdx_param_count.argtypes = [vp]
        lib.gbdx_param_count.restype = i64
        lib.gbdx_solve_fwd.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, i64, vp, vp, vp,
                                       vp, vp, vp, vp, _c.c_size_t, vp]
        lib.gbdx_solve_fwd.restype = i32
        lib.gbdx_solve_fwd_ex.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, i64, vp, vp,
                                          vp, vp, vp, vp, _c.POINTER(FwdExtras), vp,
                                          _c.c_size_t, vp]
        lib.gbdx_solve_fwd_ex.restype = i32
        lib.gbdx_dense_evaluate.argtypes = [vp, i64, vp, vp, i64, vp, vp, vp, vp, i64, vp, i64,
                                            i32, i32, vp, vp]
        lib.gbdx_dense_evaluate.restype = i32
        lib.gbdx_selftest_tcgen05.argtypes = [vp, vp, vp, vp, vp]
        lib.gbdx_selftest_tcgen05.restype = i32
        lib.gbdx_solve_bwd.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, i64, vp, vp, vp, vp,
                                       vp, vp, _c.c_size_t, vp]
        lib.gbdx_solve_bwd.restype = i32
        lib.gbdx_backsolve_bwd.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, vp, vp, vp, vp,
                                           vp, vp, vp, _c.c_size_t, vp]
        lib.gbdx_backsolve_bwd.restype = i32
        lib.gbdx_backsolve_bwd_ex.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, vp, vp, i64,
                                              vp, vp, vp, vp, vp, vp, _c.c_size_t, vp]
        lib.gbdx_backsolve_bwd_ex.restype = i32
        lib.gbdx_last_error.argtypes = []
        lib.gbdx_last_error.restype = _c.c_char_p
        lib.gbdx_version.restype = i32
        lib.gbdx_bounds_checked.argtypes = []
        lib.gbdx_bounds_checked.restype = i32
        lib.gbdx_host_device_pointer.argtypes = [vp, _c.POINTER(vp)]
        lib.gbdx_host_device_pointer.restype = i32
        if bool(lib.gbdx_bounds_checked()) != bounds:
            raise RuntimeError(f"{os.path.basename(path)} is not the requested build")
        lib.gbdx_problem_desc_size.restype = _c.c_size_t
        if lib.gbdx_problem_desc_size() != _c.sizeof(ProblemDesc):
            raise RuntimeError("gbdx_problem_desc layout mismatch between Python and C")
        _LIB = lib
        return lib


def last_error() -> str:
    return load().gbdx_last_error().decode()


class GbdxError(RuntimeError):
    pass


class GbdxBoundsError(GbdxError, IndexError):
    """A kernel index left its buffer (bounds-checked build, GBDX_ERR_BOUNDS)."""


def check(rc: int, what: str):
    if rc != 0:
        msg = last_error()
        if rc == -1:
            raise ValueError(f"{what}: {msg}")
        if rc == -5:
            raise GbdxBoundsError(f"{what}: {msg}")
        raise GbdxError(f"{what} failed ({rc}): {msg}")


def host_device_pointer(ptr: int):
    """The device address of page-locked host memory at `ptr` (kernels read
    and write it in place), or None when it is not mapped for the current
    device."""
    out = _c.c_void_p()
    if load().gbdx_host_device_pointer(_c.c_void_p(ptr), _c.byref(out)) != 0:
        return None
    return out.value


def make_desc(fields: dict) -> ProblemDesc:
    d = ProblemDesc()
    for k, v in fields.items():
        if k == "mlp_widths":
            d.mlp_widths = (i32 * 9)(*([int(x) for x in v] + [0] * (9 - len(v))))
        elif k in ("ev_kind", "ev_dir"):
            setattr(d, k, (i32 * 4)(*([int(x) for x in v] + [0] * (4 - len(v)))))
        elif k == "ev_coef":
            v = [float(x) for x in v]
            setattr(d, k, (f64 * 24)(*(v + [0.0] * (24 - len(v)))))
        elif k in ("dtmin", "dtmax") and v is None:
            setattr(d, k, math.nan)
        else:
            setattr(d, k, v)
    return d


class Problem:
    """Owns a gbdx_problem handle."""

    def __init__(self, fields: dict):
        self.lib = load()
        self.fields = dict(fields)
        self.desc = make_desc(fields)
        h = vp()
        check(self.lib.gbdx_problem_create(_c.byref(self.desc), _c.byref(h)),
              "gbdx_problem_create")
        self.handle = h

    @property
    def n_save(self) -> int:
        return self.lib.gbdx_num_saves(self.handle)

    def workspace_size(self, batch: int) -> int:
        return self.lib.gbdx_workspace_size(self.handle, batch)

    def param_count(self) -> int:
        return self.lib.gbdx_param_count(self.handle)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.gbdx_problem_destroy(h)
            except Exception:
                pass


_problem_cache: dict = {}


def get_problem(fields: dict) -> Problem:
    key = tuple(sorted((k, tuple(v) if isinstance(v, (list, tuple)) else v)
                       for k, v in fields.items()))
    p = _problem_cache.get(key)
    if p is None:
        p = Problem(fields)
        _problem_cache[key] = p
    return p
