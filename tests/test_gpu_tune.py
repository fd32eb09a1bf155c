"""The launch-shape autotuner and CUDA-graph replay of repeated solves
(diffrax_gb300/_tune.py) on the GPU: a tuned launch shape and a replayed graph
give bit-identical results to the default solve on the same inputs (analytic
fields), or results equal to the solve's accuracy (MLP fields)."""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
from diffrax_gb300 import _tune

pytestmark = pytest.mark.gpu


def vdp_inputs(B, seed):
    rng = np.random.default_rng(seed)
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), (B, 1)))
    y0 = rng.uniform(-2, 2, (B, 2))
    t1 = rng.uniform(5, 50, B)
    dev = torch.device("cuda")
    return (torch.tensor(y0, dtype=torch.float32, device=dev),
            torch.tensor(mu, dtype=torch.float32, device=dev),
            torch.tensor(t1, dtype=torch.float64, device=dev))


PID = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)


def test_autotune_picks_a_candidate_and_keeps_results():
    y0, mu, t1 = vdp_inputs(8192, 0)
    term = dfx.ODETerm(dfx.VanDerPol())
    ref = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID)
    sol = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID,
                          autotune=True)
    assert torch.equal(sol.ys, ref.ys) and torch.equal(sol.stats["num_steps"],
                                                      ref.stats["num_steps"])
    shapes = list(_tune.tuned_shapes().values())
    assert len(shapes) == 1
    fields = dfx.lower(term, dfx.Dopri5(), PID, dfx.SaveAt(t1=True), dim=2,
                       dtype=torch.float32, max_steps=4096, n_ts=0)
    assert shapes[0] in _tune.candidates(fields, 8192)
    # a second solve of the same problem class reuses the choice
    dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID,
                    autotune=True)
    assert len(_tune.tuned_shapes()) == 1


def test_autotune_mlp_row_tiles():
    # the neural-ODE field 64-128-128-64 (W ~ N(0, 1/fan_in), zero biases)
    rng = np.random.default_rng(1)
    dev = torch.device("cuda")
    widths = (64, 128, 128, 64)
    Ws = [torch.tensor(rng.standard_normal((o, i)) / np.sqrt(i), dtype=torch.float32,
                       device=dev) for i, o in zip(widths[:-1], widths[1:])]
    bs = [torch.zeros(o, dtype=torch.float32, device=dev) for o in widths[1:]]
    term = dfx.ODETerm(dfx.MLPField(Ws, bs))
    y0 = torch.tensor(rng.standard_normal((1024, 64)), dtype=torch.float32, device=dev)
    pid = dfx.PIDController(rtol=1e-5, atol=1e-7)
    ref = dfx.diffeqsolve(term, dfx.Tsit5(), 0.0, 1.0, None, y0, stepsize_controller=pid)
    sol = dfx.diffeqsolve(term, dfx.Tsit5(), 0.0, 1.0, None, y0, stepsize_controller=pid,
                          autotune=True)
    # the MLP kernels sum each row's error norm with shared-memory atomics,
    # whose order (and last bit) may change with the launch shape, and the
    # tuner may pick the tcgen05 tiles: equal to the solve's accuracy, not bit
    # for bit
    chosen = [v for v in _tune.tuned_shapes().values() if v[0] in ("fused", "tc")]
    assert chosen
    err = (sol.ys - ref.ys).abs().max() / ref.ys.abs().max()
    assert float(err) < 1e-4


def test_graphed_solve_replays_new_inputs():
    term = dfx.ODETerm(dfx.VanDerPol())
    y0, mu, t1 = vdp_inputs(4096, 2)
    g = dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID,
                         autotune=True)
    for seed in (3, 4):
        y0n, mun, t1n = vdp_inputs(4096, seed)
        sol = g(y0=y0n, args=mun, t1=t1n)
        ref = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1n, None, y0n, mun,
                              stepsize_controller=PID, kernel=g.shape[0],
                              block_threads=g.shape[1], ctas_per_sm=g.shape[2])
        assert torch.equal(sol.ys, ref.ys) and torch.equal(sol.ts, ref.ts)
        assert torch.equal(sol.stats["num_accepted_steps"], ref.stats["num_accepted_steps"])
    # the inputs given to the constructor were copied, not aliased
    assert torch.equal(y0, vdp_inputs(4096, 2)[0])


def test_graphed_solve_with_event():
    term = dfx.ODETerm(dfx.VanDerPol())
    y0, mu, t1 = vdp_inputs(2048, 5)
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-5, 1e-5), direction=False)
    g = dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID,
                         event=ev, throw=False)
    y0n, mun, t1n = vdp_inputs(2048, 6)
    sol = g(y0=y0n, args=mun, t1=t1n)
    ref = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1n, None, y0n, mun, stepsize_controller=PID,
                          event=ev, throw=False)
    assert torch.equal(sol.ys, ref.ys) and torch.equal(sol.event_mask, ref.event_mask)


def test_graphed_solve_host_io():
    # host_io: the page-locked inputs are the graph's staging buffers and the
    # outputs land in page-locked host tensors, one graph launch per solve
    term = dfx.ODETerm(dfx.VanDerPol())
    y0, mu, t1 = vdp_inputs(4096, 7)
    y0_h, mu_h, t1_h = (x.cpu().pin_memory() for x in (y0, mu, t1))
    g = dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1_h, None, y0_h, mu_h,
                         stepsize_controller=PID, throw=False, host_io=True)
    # page-locked buffers are mapped on this GPU: the kernels read and write
    # them in place
    assert g.zero_copy
    sol = g()
    ref = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID)
    assert sol.ys.device.type == "cpu" and sol.ys.is_pinned()
    assert torch.equal(sol.ys, ref.ys.cpu()) and torch.equal(sol.result, ref.result.cpu())
    # new inputs written into the staging buffers by the caller, or passed
    y0n, mun, t1n = vdp_inputs(4096, 8)
    y0_h.copy_(y0n.cpu())
    sol2 = g(args=mun.cpu(), t1=t1n.cpu())
    assert sol2 is sol  # the same host tensors, overwritten
    ref = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1n, None, y0n, mun, stepsize_controller=PID)
    assert torch.equal(sol.ys, ref.ys.cpu())
    assert torch.equal(sol.ts, ref.ts.cpu())
    assert torch.equal(sol.stats["num_steps"], ref.stats["num_steps"].cpu())
    # the copy path: the graph copies the staging buffers in and the
    # results out
    gc = dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1_h, None, y0_h, mu_h,
                          stepsize_controller=PID, throw=False, host_io="copy")
    assert not gc.zero_copy
    y0_h.copy_(y0.cpu())
    t1_h.copy_(t1.cpu())
    mu_h.copy_(mu.cpu())
    ref = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID)
    solc = gc()
    assert torch.equal(solc.ys, ref.ys.cpu()) and torch.equal(solc.result, ref.result.cpu())
    # a strided staging buffer would be gathered once, at capture
    y0_t = torch.empty((2, 4096), dtype=torch.float32).pin_memory()
    with pytest.raises(ValueError, match="contiguous"):
        dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1_h, None, y0_t.t(), mu_h,
                         stepsize_controller=PID, host_io=True)
    with pytest.raises(ValueError, match="page-locked"):
        dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1.cpu(), None, y0.cpu(), mu.cpu(),
                         stepsize_controller=PID, host_io=True)


def test_graphed_solve_host_io_with_events():
    # zero-copy host I/O with the event index among the outputs
    term = dfx.ODETerm(dfx.VanDerPol())
    y0, mu, t1 = vdp_inputs(2048, 9)
    y0_h, mu_h, t1_h = (x.cpu().pin_memory() for x in (y0, mu, t1))
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-5, 1e-5), direction=False)
    g = dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1_h, None, y0_h, mu_h,
                         stepsize_controller=PID, throw=False, event=ev, host_io=True)
    assert g.zero_copy
    sol = g()
    ref = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1, None, y0, mu, stepsize_controller=PID,
                          event=ev, throw=False)
    assert sol.event_mask.device.type == "cpu"
    assert torch.equal(sol.ys, ref.ys.cpu()) and torch.equal(sol.event_mask, ref.event_mask.cpu())


def test_host_device_pointer():
    from diffrax_gb300 import _lib
    assert _lib.host_device_pointer(torch.zeros(16).pin_memory().data_ptr()) is not None
    assert _lib.host_device_pointer(torch.zeros(16).data_ptr()) is None  # pageable
    assert _lib.host_device_pointer(torch.zeros(16, device="cuda").data_ptr()) is None
