"""The allocation-free forward solve (gbdx_solve_fwd_noalloc).

Callers that cannot allocate device memory -- hosts that reserve all of it at
start-up, plugin hosts that only pass input and output buffers -- use this
entry point, which takes its scratch from a fixed array inside the library.
It must give the same results as gbdx_solve_fwd with a caller workspace, on
repeated calls (the array keeps the previous call's contents), and reject
batches larger than the array.  This file is collected last so that a run that
stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
from diffrax_gb300 import _lib
from diffrax_gb300._integrate import Lowered

pytestmark = pytest.mark.gpu

vp, i64 = ctypes.c_void_p, ctypes.c_int64


def _bind(lib):
    f = lib.gbdx_solve_fwd_noalloc
    f.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, i64, vp, vp, vp, vp, vp, vp, vp]
    f.restype = ctypes.c_int32
    return f


def _problem(B, seed):
    dev = torch.device("cuda")
    rng = np.random.default_rng(seed)
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), B))
    y0 = rng.uniform(-2, 2, (B, 2))
    t1 = rng.uniform(5, 50, B)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    return Lowered(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(), 0.0,
                   torch.tensor(t1, device=dev), None,
                   torch.tensor(y0, dtype=torch.float32, device=dev),
                   torch.tensor(mu[:, None], dtype=torch.float32, device=dev),
                   dfx.SaveAt(t1=True), pid, None, 4096, "fused", 0, 0)


def _noalloc_solve(fn, low):
    dev = low.device
    B, D, n = low.B, low.dim, low.n_save
    ys = torch.full((B, n, D), -7.0, dtype=low.dtype, device=dev)
    ts = torch.full((B, n), -7.0, dtype=torch.float64, device=dev)
    res = torch.full((B,), -7, dtype=torch.int32, device=dev)
    st = torch.full((B, 3), -7, dtype=torch.int32, device=dev)
    p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    rc = fn(low.problem.handle, B, p(low.t0), p(low.t1), p(low.dt0), low.tstride, p(low.y0),
            p(low.args), low.args_stride, p(low.params), p(low.save_ts), p(ys), p(ts), p(res),
            p(st), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    return ys, ts, res, st


def test_noalloc_matches_workspace_solve_on_repeated_calls():
    fn = _bind(_lib.load())
    low = _problem(5000, 41)
    ref = [t.clone() for t in low.run_forward()]
    torch.cuda.synchronize()
    for _ in range(2):  # the second call reuses the array the first one left behind
        out = _noalloc_solve(fn, low)
        # the fused kernel is deterministic: the same solve gives the same bits
        assert torch.equal(out[0], ref[0])
        assert torch.equal(out[1], ref[1])
        assert torch.equal(out[2], ref[2])
        assert torch.equal(out[3], ref[3])
        assert (out[2] == 0).all()


def test_noalloc_second_problem_after_first():
    # A different batch size and input set on the same array.
    fn = _bind(_lib.load())
    for B, seed in ((777, 42), (3000, 43)):
        low = _problem(B, seed)
        ref = [t.clone() for t in low.run_forward()]
        out = _noalloc_solve(fn, low)
        assert torch.equal(out[0], ref[0])
        assert torch.equal(out[3], ref[3])


def test_noalloc_rejects_batches_beyond_the_array():
    fn = _bind(_lib.load())
    low = _problem(16, 44)
    # All pointers null: the size check must reject the call before any launch.
    rc = fn(low.problem.handle, 2_000_000, None, None, None, 1, None, None, 1, None, None,
            None, None, None, None, torch.cuda.current_stream().cuda_stream)
    assert rc == -4
    msg = _lib.last_error()
    assert "4 MiB" in msg and "2000000 trajectories" in msg


def test_noalloc_rejects_problems_with_an_adjoint():
    # A gradient's tape must outlive the call in a workspace the backward
    # reads, which the shared array cannot be.
    fn = _bind(_lib.load())
    dev = torch.device("cuda")
    w = [64, 128, 128, 64]
    field = dfx.MLPField([torch.zeros(w[i + 1], w[i], device=dev) for i in range(3)],
                         [torch.zeros(w[i + 1], device=dev) for i in range(3)])
    low = Lowered(dfx.ODETerm(field), dfx.Tsit5(), 0.0, 1.0, 0.1,
                  torch.zeros(4, 64, device=dev), None, dfx.SaveAt(t1=True),
                  dfx.ConstantStepSize(), dfx.RecursiveCheckpointAdjoint(), 16, "fused", 0, 0,
                  want_grad=True)
    rc = fn(low.problem.handle, 4, None, None, None, 0, None, None, 0, None, None,
            None, None, None, None, torch.cuda.current_stream().cuda_stream)
    assert rc != 0
    assert "forward-only" in _lib.last_error()
