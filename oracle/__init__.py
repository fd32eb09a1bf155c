"""FP64 CPU oracle for the batched diffeqsolve hot path -- TEST INFRASTRUCTURE.

This package wraps ``gbdx_oracle.c`` (an FP64 C restatement of Diffrax's
``diffeqsolve`` loop, solvers, controllers, interpolants, virtual Brownian
tree and gradients) through ctypes.  It is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` load it.
The product library (``diffrax_gb300``) never imports it and has no CPU path.

The descriptor fields mirror ``gbdx_problem_desc`` in ``include/gbdx.h`` so
that one lowered problem can be given to both the kernels and the oracle.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from .build import build_oracle, oracle_lib_path

__all__ = [
    "OracleDesc", "load", "solve", "grad_recursive", "vbt_increments", "vbt_levy_increments",
    "vbt_levy_points", "normal4", "SHARK", "SRA1", "SEA",
    "dense_evaluate", "n_saves", "STAGES", "clip_times", "clip_find", "clip_adapt",
    "EULER", "HEUN", "DOPRI5", "TSIT5", "DOPRI8", "CONSTANT", "PID",
    "LOTKA_VOLTERRA", "VAN_DER_POL", "ORNSTEIN_UHLENBECK", "MLP", "LINEAR", "CALLBACK",
    "DIFF_NONE", "DIFF_OU", "DIFF_TANH_DIAG", "RESULT_NAMES", "EV_LINEAR", "EV_LINEAR_BOOL",
    "EV_STEADY", "EV_EITHER", "EV_UP", "EV_DOWN",
]

EULER, HEUN, DOPRI5, TSIT5, DOPRI8, SHARK, SRA1, SEA = 0, 1, 2, 3, 4, 5, 6, 7
CONSTANT, PID = 0, 1
LOTKA_VOLTERRA, VAN_DER_POL, ORNSTEIN_UHLENBECK, MLP, LINEAR, CALLBACK = 0, 1, 2, 3, 4, 5
DIFF_NONE, DIFF_OU, DIFF_TANH_DIAG = 0, 1, 2
NORM_RMS, NORM_ADJOINT_SEMI = 0, 1
EV_LINEAR, EV_LINEAR_BOOL, EV_STEADY = 0, 1, 2
EV_EITHER, EV_UP, EV_DOWN = 0, 1, 2
RESULT_NAMES = {0: "successful", 1: "max_steps_reached", 2: "dt_min_reached",
                3: "event_occurred", 4: "max_steps_rejected", 5: "internal_error",
                6: "nonlinear_max_steps_reached"}


class OracleDesc(ctypes.Structure):
    _fields_ = [
        ("solver", ctypes.c_int32), ("controller", ctypes.c_int32),
        ("field", ctypes.c_int32), ("dim", ctypes.c_int32),
        ("rtol", ctypes.c_double), ("atol", ctypes.c_double),
        ("pcoeff", ctypes.c_double), ("icoeff", ctypes.c_double),
        ("dcoeff", ctypes.c_double), ("safety", ctypes.c_double),
        ("factormin", ctypes.c_double), ("factormax", ctypes.c_double),
        ("dtmin", ctypes.c_double), ("dtmax", ctypes.c_double),
        ("force_dtmin", ctypes.c_int32), ("error_order", ctypes.c_double),
        ("n_ts", ctypes.c_int32), ("save_t0", ctypes.c_int32),
        ("save_t1", ctypes.c_int32), ("max_steps", ctypes.c_int32),
        ("n_args", ctypes.c_int32), ("mlp_depth", ctypes.c_int32),
        ("mlp_widths", ctypes.c_int32 * 9), ("diffusion", ctypes.c_int32),
        ("vbt_t0", ctypes.c_double), ("vbt_t1", ctypes.c_double),
        ("vbt_tol", ctypes.c_double), ("seed", ctypes.c_uint64),
        ("norm", ctypes.c_int32), ("save_steps", ctypes.c_int32),
        ("save_dense", ctypes.c_int32), ("n_step_ts", ctypes.c_int32),
        ("n_jump_ts", ctypes.c_int32), ("n_event", ctypes.c_int32),
        ("event_root", ctypes.c_int32), ("ev_kind", ctypes.c_int32 * 4),
        ("ev_dir", ctypes.c_int32 * 4), ("levy_area", ctypes.c_int32),
        ("newton_rtol", ctypes.c_double),
        ("newton_atol", ctypes.c_double), ("ev_coef", ctypes.c_double * 24),
    ]


_DEFAULTS = dict(solver=TSIT5, controller=PID, field=LOTKA_VOLTERRA, dim=2,
                 rtol=1e-3, atol=1e-6, pcoeff=0.0, icoeff=1.0, dcoeff=0.0,
                 safety=0.9, factormin=0.2, factormax=10.0, dtmin=math.nan,
                 dtmax=math.nan, force_dtmin=1, error_order=0.0, n_ts=0,
                 save_t0=0, save_t1=1, max_steps=4096, n_args=0, mlp_depth=0,
                 mlp_widths=(), diffusion=DIFF_NONE, vbt_t0=0.0, vbt_t1=1.0,
                 vbt_tol=1e-3, seed=0, norm=0, save_steps=0, save_dense=0,
                 n_step_ts=0, n_jump_ts=0, n_event=0, event_root=0, ev_kind=(), ev_dir=(),
                 levy_area=0, newton_rtol=1e-5, newton_atol=1e-5, ev_coef=())

STAGES = {EULER: 1, HEUN: 2, DOPRI5: 7, TSIT5: 7, DOPRI8: 14, SHARK: 2, SRA1: 2, SEA: 1}


def n_saves(desc) -> int:
    """Output length of the descriptor's SaveAt (_integrate.py:1273-1293)."""
    n = desc.save_t0 + desc.n_ts
    if desc.save_steps:
        n += desc.max_steps // desc.save_steps
    if desc.save_t1 and (desc.save_steps == 0 or desc.max_steps % desc.save_steps):
        n += 1
    return n


def oracle_fields(fields: dict) -> dict:
    """The subset of a lowered GPU descriptor (diffrax_gb300.lower) that the
    oracle's descriptor holds: the problem definition without the GPU launch
    policy (kernel family, launch shape, schedule, precision mode)."""
    return {k: v for k, v in fields.items() if k in _DEFAULTS}


def make_desc(**kw) -> OracleDesc:
    vals = dict(_DEFAULTS)
    unknown = set(kw) - set(vals)
    if unknown:
        raise KeyError(f"unknown descriptor fields {sorted(unknown)}")
    vals.update(kw)
    d = OracleDesc()
    for k, v in vals.items():
        if k == "mlp_widths":
            arr = (ctypes.c_int32 * 9)(*([int(x) for x in v] + [0] * (9 - len(v))))
            d.mlp_widths = arr
        elif k in ("ev_kind", "ev_dir"):
            setattr(d, k, (ctypes.c_int32 * 4)(*([int(x) for x in v] + [0] * (4 - len(v)))))
        elif k == "ev_coef":
            v = [float(x) for x in v]
            setattr(d, k, (ctypes.c_double * 24)(*(v + [0.0] * (24 - len(v)))))
        elif k in ("dtmin", "dtmax") and v is None:
            setattr(d, k, math.nan)
        else:
            setattr(d, k, v)
    return d


_LIB = None
VF_CB = ctypes.CFUNCTYPE(None, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                         ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p)


def load():
    """Load (building on first use) the oracle shared library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = oracle_lib_path()
    src = os.path.join(os.path.dirname(__file__), "gbdx_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        build_oracle()
    lib = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int32)
    i64 = ctypes.c_int64
    lib.orc_solve.argtypes = [ctypes.POINTER(OracleDesc), i64, dp, dp, dp, i64, dp, dp,
                              i64, dp, dp, VF_CB, ctypes.c_void_p, dp, dp, ip, ip,
                              ctypes.c_int]
    lib.orc_solve.restype = ctypes.c_int
    lib.orc_solve_dense.argtypes = lib.orc_solve.argtypes[:-1] + [dp, dp, ip, ip, ctypes.c_int]
    lib.orc_solve_dense.restype = ctypes.c_int
    lib.orc_solve_state.argtypes = lib.orc_solve.argtypes[:-1] + [dp, dp, ip, ip, dp, dp,
                                                                  ctypes.c_int]
    lib.orc_solve_state.restype = ctypes.c_int
    lib.orc_dense_evaluate.argtypes = [ctypes.POINTER(OracleDesc), i64, dp, dp, i64, dp, dp,
                                       dp, ip, i64, dp, i64, ctypes.c_int, ctypes.c_int, dp]
    lib.orc_dense_evaluate.restype = ctypes.c_int
    lib.orc_clip_find.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    lib.orc_clip_find.restype = ctypes.c_int
    lib.orc_clip_adapt.argtypes = [dp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_double)]
    lib.orc_clip_adapt.restype = ctypes.c_int
    lib.orc_grad_recursive.argtypes = [ctypes.POINTER(OracleDesc), i64, dp, dp, dp, i64,
                                       dp, dp, i64, dp, i64, dp, dp, dp, dp, ip, ip, dp,
                                       dp, dp, ctypes.c_int]
    lib.orc_grad_recursive.restype = ctypes.c_int
    lib.orc_backsolve.argtypes = [ctypes.POINTER(OracleDesc), i64, dp, dp, dp, i64, dp, dp,
                                  dp, dp, i64, dp, i64, dp, dp, dp, ip, ip, ctypes.c_int]
    lib.orc_backsolve.restype = ctypes.c_int
    lib.orc_vbt_increments.argtypes = [ctypes.POINTER(OracleDesc), i64,
                                       ctypes.POINTER(ctypes.c_uint32), dp, dp, dp]
    lib.orc_vbt_levy_increments.argtypes = [ctypes.POINTER(OracleDesc), i64,
                                            ctypes.POINTER(ctypes.c_uint32), dp, dp, dp, dp]
    lib.orc_vbt_levy_points.argtypes = [ctypes.POINTER(OracleDesc), i64,
                                        ctypes.POINTER(ctypes.c_uint32), dp, dp, dp]
    lib.orc_normal4.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_uint32, ctypes.c_uint32, dp]
    lib.orc_desc_size.restype = ctypes.c_int
    if lib.orc_desc_size() != ctypes.sizeof(OracleDesc):
        raise RuntimeError("oracle descriptor layout mismatch")
    _LIB = lib
    return lib


def _dptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


def _prep(desc, B, t0, t1, dt0, y0, args, params, ts):
    t0 = np.asarray(t0, dtype=np.float64)
    t1 = np.asarray(t1, dtype=np.float64)
    time_stride = 0 if (t0.ndim == 0 and t1.ndim == 0 and
                        (dt0 is None or np.ndim(dt0) == 0)) else 1
    if time_stride:
        t0 = np.ascontiguousarray(np.broadcast_to(t0, (B,)), dtype=np.float64)
        t1 = np.ascontiguousarray(np.broadcast_to(t1, (B,)), dtype=np.float64)
        if dt0 is not None:
            dt0 = np.ascontiguousarray(np.broadcast_to(np.asarray(dt0, np.float64), (B,)))
    else:
        t0 = t0.reshape(1).copy()
        t1 = t1.reshape(1).copy()
        if dt0 is not None:
            dt0 = np.asarray(dt0, dtype=np.float64).reshape(1).copy()
    y0 = _f64(y0, (B, desc.dim))
    if args is None or desc.n_args == 0:
        args_arr = np.zeros((1, max(desc.n_args, 1)))
        args_stride = 0
    else:
        args_arr = _f64(args)
        if args_arr.ndim == 1:
            args_arr = args_arr.reshape(1, desc.n_args)
            args_stride = 0
        else:
            args_arr = args_arr.reshape(B, desc.n_args)
            args_stride = desc.n_args
    params = _f64(params) if params is not None else np.zeros(1)
    ts = _f64(ts) if ts is not None and len(ts) else np.zeros(1)
    return t0, t1, dt0, time_stride, y0, args_arr, args_stride, params.reshape(-1), ts


def clip_times(desc: OracleDesc, ts=None, step_ts=None, jump_ts=None):
    """The solve's times array: SaveAt ts, then ClipStepSizeController step_ts
    and jump_ts (each sorted increasing), with the descriptor's counts set."""
    parts = [np.zeros(0) if ts is None else np.asarray(ts, np.float64).reshape(-1)]
    for name, v in (("n_step_ts", step_ts), ("n_jump_ts", jump_ts)):
        v = np.zeros(0) if v is None else np.sort(np.asarray(v, np.float64).reshape(-1))
        setattr(desc, name, int(v.size))
        parts.append(v)
    return np.concatenate(parts)


STATE_HEAD = 7  # the resume record: 7 + dim doubles per trajectory (gbdx_oracle.c)


def solve(desc: OracleDesc, t0, t1, dt0, y0, args=None, params=None, ts=None,
          nthreads: int = 1, callback=None, step_ts=None, jump_ts=None, state_in=None,
          want_state=False):
    """Run the oracle.  Returns dict(ys [B,n_save,D], ts [B,n_save], result [B],
    stats [B,3] = (num_steps, num_accepted, num_rejected)).  step_ts / jump_ts
    wrap the PID controller in ClipStepSizeController (clip.py).  state_in
    [B, STATE_HEAD + D] resumes from a previous solve's record; want_state
    returns this solve's final record as "state"."""
    lib = load()
    if step_ts is not None or jump_ts is not None:
        ts = clip_times(desc, ts, step_ts, jump_ts)
    y0 = np.asarray(y0, dtype=np.float64)
    B = y0.shape[0] if y0.ndim == 2 else 1
    t0, t1, dt0, tstride, y0, args_arr, astride, params, ts = _prep(
        desc, B, t0, t1, dt0, y0, args, params, ts)
    n_save = n_saves(desc)
    ys = np.empty((B, n_save, desc.dim))
    ts_out = np.empty((B, n_save))
    res = np.empty(B, dtype=np.int32)
    stats = np.empty((B, 3), dtype=np.int32)
    dense = None
    if desc.save_dense:
        L = desc.max_steps + 1
        rec = (2 + STAGES[desc.solver]) * desc.dim
        dense = dict(ts=np.empty((B, L)), info=np.empty((B, L - 1, rec)),
                     n=np.empty(B, dtype=np.int32))
    cb = VF_CB(0)
    keep = None
    if callback is not None:
        dim = desc.dim

        def _cb(t, yp, outp, n, ctx):
            yv = np.ctypeslib.as_array(yp, shape=(dim,))
            ov = np.ctypeslib.as_array(outp, shape=(dim,))
            ov[:] = callback(t, yv.copy())
        keep = cb = VF_CB(_cb)
    ip = ctypes.POINTER(ctypes.c_int32)
    ev = np.full(B, -1, dtype=np.int32) if desc.n_event else None
    st_in = None if state_in is None else np.ascontiguousarray(
        np.asarray(state_in, dtype=np.float64).reshape(B, STATE_HEAD + desc.dim))
    st_out = np.empty((B, STATE_HEAD + desc.dim)) if want_state else None
    rc = lib.orc_solve_state(ctypes.byref(desc), B, _dptr(t0), _dptr(t1), _dptr(dt0), tstride,
                             _dptr(y0), _dptr(args_arr), astride, _dptr(params), _dptr(ts), cb,
                             None, _dptr(ys), _dptr(ts_out), res.ctypes.data_as(ip),
                             stats.ctypes.data_as(ip),
                             _dptr(dense["ts"]) if dense else None,
                             _dptr(dense["info"]) if dense else None,
                             dense["n"].ctypes.data_as(ip) if dense else None,
                             ev.ctypes.data_as(ip) if ev is not None else None,
                             _dptr(st_in), _dptr(st_out), int(nthreads))
    del keep
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    out = dict(ys=ys, ts=ts_out, result=res, stats=stats)
    if ev is not None:
        out["event_index"] = ev
    if st_out is not None:
        out["state"] = st_out
    if dense:
        out.update(dense_ts=dense["ts"], dense_info=dense["info"], dense_n=dense["n"])
    return out


def clip_find(ts, t, hint, direction=1) -> int:
    """_find_idx_with_hint (clip.py:102-118) in the direction-flipped time."""
    lib = load()
    a = _f64(np.sort(np.asarray(ts, np.float64)))
    return int(lib.orc_clip_find(_dptr(a), int(a.size), int(direction), float(t), int(hint)))


def clip_adapt(step_ts, jump_ts, next_t0, next_t1, idx=(0, 0), direction=1):
    """ClipStepSizeController.adapt_step_size after the inner controller
    proposed (next_t0, next_t1) (clip.py:330-389).  Returns (next_t0, next_t1,
    made_jump, (step_index, jump_index))."""
    lib = load()
    st = _f64(np.sort(np.asarray([] if step_ts is None else step_ts, np.float64)))
    jt = _f64(np.sort(np.asarray([] if jump_ts is None else jump_ts, np.float64)))
    ix = np.asarray(idx, dtype=np.int32).copy()
    a, b = ctypes.c_double(next_t0), ctypes.c_double(next_t1)
    mj = lib.orc_clip_adapt(_dptr(st) if st.size else None, int(st.size),
                            _dptr(jt) if jt.size else None, int(jt.size), int(direction),
                            ix.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                            ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value, bool(mj), (int(ix[0]), int(ix[1]))


def dense_evaluate(desc: OracleDesc, t0, t1, y0, sol, query, left=True, order=0):
    """DenseInterpolation.evaluate (order 0) or .derivative (order 1) of a
    solve(..., save_dense=1) result at `query` ([Q] shared or [B, Q]).
    Returns [B, Q, dim]."""
    lib = load()
    y0 = _f64(y0)
    B = y0.shape[0]
    t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, np.float64), (B,)))
    t1 = np.ascontiguousarray(np.broadcast_to(np.asarray(t1, np.float64), (B,)))
    q = _f64(query)
    if q.ndim == 1:
        Q, qstride = q.shape[0], 0
    else:
        Q, qstride = q.shape[1], q.shape[1]
    out = np.empty((B, Q, desc.dim))
    ip = ctypes.POINTER(ctypes.c_int32)
    dn = np.ascontiguousarray(sol["dense_n"], dtype=np.int32)
    rc = lib.orc_dense_evaluate(ctypes.byref(desc), B, _dptr(t0), _dptr(t1), 1, _dptr(y0),
                                _dptr(_f64(sol["dense_ts"])), _dptr(_f64(sol["dense_info"])),
                                dn.ctypes.data_as(ip), Q, _dptr(q), qstride, int(bool(left)),
                                int(order), _dptr(out))
    if rc != 0:
        raise ValueError(f"oracle rejected the evaluation (code {rc})")
    return out


def grad_recursive(desc: OracleDesc, t0, t1, dt0, y0, grad_ys, args=None, params=None,
                   ts=None, nthreads: int = 1):
    """Discretise-then-optimise gradient of sum(grad_ys * ys).  Returns dict with
    ys, ts, result, stats, grad_y0 [B,D], grad_args [B,n_args], grad_params [P]."""
    lib = load()
    y0 = np.asarray(y0, dtype=np.float64)
    B = y0.shape[0]
    t0, t1, dt0, tstride, y0, args_arr, astride, params_arr, ts = _prep(
        desc, B, t0, t1, dt0, y0, args, params, ts)
    n_save = n_saves(desc)
    gys = _f64(grad_ys, (B, n_save, desc.dim))
    ys = np.empty((B, n_save, desc.dim))
    ts_out = np.empty((B, n_save))
    res = np.empty(B, dtype=np.int32)
    stats = np.empty((B, 3), dtype=np.int32)
    gy0 = np.zeros((B, desc.dim))
    gargs = np.zeros((B, max(desc.n_args, 1)))
    n_params = params_arr.size if params is not None else 0
    gp = np.zeros(max(n_params, 1))
    rc = lib.orc_grad_recursive(ctypes.byref(desc), B, _dptr(t0), _dptr(t1), _dptr(dt0),
                                tstride, _dptr(y0), _dptr(args_arr), astride,
                                _dptr(params_arr), n_params, _dptr(ts), _dptr(gys),
                                _dptr(ys), _dptr(ts_out),
                                res.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                stats.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                _dptr(gy0), _dptr(gargs) if desc.n_args else None,
                                _dptr(gp), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return dict(ys=ys, ts=ts_out, result=res, stats=stats, grad_y0=gy0,
                grad_args=gargs[:, :desc.n_args], grad_params=gp[:n_params])


def backsolve(desc: OracleDesc, t0, t1, dt0, ts_saved, ys, grad_ys, args=None,
              params=None, nthreads: int = 1):
    """BacksolveAdjoint backward from the forward's saved (ts, ys) and their
    cotangent.  `desc` describes the backward solve (solver, controller, norm)
    and the forward's SaveAt.  Returns dict with grad_y0 [B,D], grad_args
    [B,n_args], grad_params [P] (summed over the batch), result [B] and stats
    [B,3] (steps, accepted, rejected over all segments)."""
    lib = load()
    ys = np.asarray(ys, dtype=np.float64)
    B = ys.shape[0]
    n_save = desc.save_t0 + desc.n_ts + desc.save_t1
    t0, t1, dt0, tstride, _, args_arr, astride, params_arr, _ = _prep(
        desc, B, t0, t1, dt0, np.zeros((B, desc.dim)), args, params, None)
    ts_saved = _f64(ts_saved, (B, n_save))
    ys = _f64(ys, (B, n_save, desc.dim))
    gys = _f64(grad_ys, (B, n_save, desc.dim))
    gy0 = np.zeros((B, desc.dim))
    gargs = np.zeros((B, max(desc.n_args, 1)))
    n_params = params_arr.size if params is not None else 0
    gp = np.zeros(max(n_params, 1))
    res = np.empty(B, dtype=np.int32)
    stats = np.empty((B, 3), dtype=np.int32)
    rc = lib.orc_backsolve(ctypes.byref(desc), B, _dptr(t0), _dptr(t1), _dptr(dt0), tstride,
                           _dptr(ts_saved), _dptr(ys), _dptr(gys), _dptr(args_arr), astride,
                           _dptr(params_arr), n_params, _dptr(gy0),
                           _dptr(gargs) if desc.n_args else None, _dptr(gp),
                           res.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                           stats.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle rejected the problem (code {rc})")
    return dict(result=res, stats=stats, grad_y0=gy0, grad_args=gargs[:, :desc.n_args],
                grad_params=gp[:n_params])


def vbt_increments(desc: OracleDesc, traj, ta, tb):
    """Brownian increments W(tb) - W(ta) of the oracle's virtual Brownian tree."""
    lib = load()
    traj = np.ascontiguousarray(traj, dtype=np.uint32)
    ta = _f64(ta)
    tb = _f64(tb)
    out = np.empty((traj.size, desc.dim))
    lib.orc_vbt_increments(ctypes.byref(desc), traj.size,
                           traj.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                           _dptr(ta), _dptr(tb), _dptr(out))
    return out


def vbt_levy_increments(desc: OracleDesc, traj, ta, tb):
    """(W, H) of [ta, tb] from the oracle's tree with space-time Levy area
    (VirtualBrownianTree.evaluate(ta, tb, use_levy=True))."""
    lib = load()
    traj = np.ascontiguousarray(traj, dtype=np.uint32)
    ta = _f64(ta)
    tb = _f64(tb)
    w = np.empty((traj.size, desc.dim))
    h = np.empty((traj.size, desc.dim))
    lib.orc_vbt_levy_increments(ctypes.byref(desc), traj.size,
                                traj.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                _dptr(ta), _dptr(tb), _dptr(w), _dptr(h))
    return w, h


def vbt_levy_points(desc: OracleDesc, traj, r):
    """W(r) and bar H(r) = r H_{0,r} of the Levy area tree on the unit interval."""
    lib = load()
    traj = np.ascontiguousarray(traj, dtype=np.uint32)
    r = _f64(r)
    w = np.empty((traj.size, desc.dim))
    h = np.empty((traj.size, desc.dim))
    lib.orc_vbt_levy_points(ctypes.byref(desc), traj.size,
                            traj.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                            _dptr(r), _dptr(w), _dptr(h))
    return w, h


def normal4(seed, traj, node, kind, q):
    lib = load()
    z = np.empty(4)
    lib.orc_normal4(seed, traj, node, kind, q, _dptr(z))
    return z
