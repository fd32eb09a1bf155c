"""GPU parity of events (diffrax/_event.py, diffrax/_integrate.py:542-877) on
the analytic-field kernels against the FP64 oracle, whose event restatement
is pinned to the reference's test/test_event.py in tests/test_oracle_pins.py.

FP64-state solves must take the oracle's step sequence and reproduce its
saves, event times (the Newton root of the last step's interpolant), fired
conditions and RESULTS codes on at least 95 % of each batch (1e-9 relative;
all within 1e-4).  FP32-state solves agree within the solve's tolerance.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu

SOLVERS = {"heun": dfx.Heun(), "dopri5": dfx.Dopri5(), "tsit5": dfx.Tsit5()}
LV_ARGS = np.array([0.1, 0.02, 0.4, 0.02])


def solve_pair(field, solver, ctrl, saveat, event, t0, t1, dt0, y0, args, dtype, kernel,
               max_steps=4096):
    dev = torch.device("cuda")
    tt = lambda x: torch.tensor(x, dtype=torch.float64, device=dev) if isinstance(  # noqa
        x, np.ndarray) else x
    sol = dfx.diffeqsolve(dfx.ODETerm(field), solver, tt(t0), tt(t1), tt(dt0),
                          torch.tensor(y0, dtype=dtype, device=dev),
                          torch.tensor(args, dtype=dtype, device=dev), saveat=saveat,
                          stepsize_controller=ctrl, max_steps=max_steps, throw=False,
                          kernel=kernel, event=event)
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(dfx.ODETerm(field), solver, ctrl, saveat, dim=y0.shape[1], dtype=dtype,
                       max_steps=max_steps, n_ts=0 if ts is None else ts.size, event=event)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, t0, t1, dt0, y0, args=args, ts=ts, nthreads=8)
    return sol, r


def event_index(sol, event):
    masks = [sol.event_mask] if not isinstance(sol.event_mask, list) else sol.event_mask
    idx = np.full(masks[0].shape[0], -1)
    for i, m in enumerate(masks):
        idx[m.cpu().numpy()] = i
    return idx


def rows_close(a, b, rows, tol, min_frac=0.95, loose=1e-4):
    """As in tests/test_gpu_dense.py: rows that took the oracle's step counts
    share the inf pattern, min_frac of the batch agrees to tol, all to loose."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    n = a.shape[0]
    a, b = a[rows], b[rows]
    assert np.array_equal(np.isposinf(a), np.isposinf(b))
    assert np.array_equal(np.isneginf(a), np.isneginf(b))
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin)
    ax = tuple(range(1, b.ndim))
    scale = np.abs(np.where(fin, b, 0)).max(axis=ax) + 1e-300
    diff = np.abs(np.where(fin, a, 0) - np.where(fin, b, 0)).max(axis=ax) / scale
    exact = (diff < tol).sum() / n
    assert exact >= min_frac, f"{exact:.3f} of the batch within {tol}"
    assert diff.max() < loose, f"max rel err {diff.max():.2e} >= {loose}"


def check_parity(sol, r, event):
    same = sol.stats["num_steps"].cpu().numpy() == r["stats"][:, 0]
    same &= sol.stats["num_accepted_steps"].cpu().numpy() == r["stats"][:, 1]
    assert same.mean() >= 0.95, f"only {same.mean():.3f} took the oracle's steps"
    assert np.array_equal(event_index(sol, event)[same], r["event_index"][same])
    assert np.array_equal(sol.result.cpu().numpy()[same], r["result"][same])
    rows_close(sol.ts.cpu().numpy(), r["ts"], same, 1e-9)
    rows_close(sol.ys.cpu().numpy(), r["ys"], same, 1e-9)


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("solver", ["heun", "dopri5", "tsit5"])
@pytest.mark.parametrize("direction", [None, True, False])
def test_event_root_fp64_matches_oracle(kernel, solver, direction):
    # Lotka-Volterra prey crossing a level per trajectory-independent set-up:
    # x = 12 (either / up / down), Newton(1e-8, 1e-8), ts and t1 saves.
    rng = np.random.default_rng(31)
    B = 96
    y0 = rng.uniform(5, 15, (B, 2))
    t1 = rng.uniform(40.0, 80.0, B)
    tol = 1e-5 if solver == "heun" else 1e-7
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0], offset=-12.0), dfx.Newton(1e-8, 1e-8),
                   direction=direction)
    saveat = dfx.SaveAt(ts=np.linspace(0.0, 40.0, 9), t1=True)
    sol, r = solve_pair(dfx.LotkaVolterra(), SOLVERS[solver],
                        dfx.PIDController(rtol=tol, atol=tol * 1e-2), saveat, ev, 0.0, t1, 0.1,
                        y0, LV_ARGS, torch.float64, kernel)
    check_parity(sol, r, ev)
    # most trajectories meet the level; where Newton converged (RESULTS 3) the
    # final save is the event's, with the prey at the level.  (Newton from the
    # end of the step, clipped to it, can stall when the interpolant turns
    # inside the step: RESULTS 6, as the reference's root find reports.)
    fired = (r["event_index"] == 0) & (r["result"] == 3)
    assert fired.mean() > 0.5
    ys, ts = sol.ys.cpu().numpy(), sol.ts.cpu().numpy()
    last = np.array([ys[b][np.isfinite(ts[b])][-1, 0] for b in range(ys.shape[0])])
    assert np.allclose(last[fired], 12.0, atol=1e-6)


@pytest.mark.parametrize("kernel", ["plain", "fused"])
def test_event_booleans_and_steps_saves(kernel):
    # Two conditions without a root finder, the first a boolean on time and
    # the second a real one on the predator, with every step saved backwards
    # in time from t0 = 60.
    rng = np.random.default_rng(32)
    B = 64
    y0 = rng.uniform(5, 15, (B, 2))
    ev = dfx.Event([dfx.LinearCondition([], t_coeff=1.0, offset=35.0, boolean=True),
                    dfx.LinearCondition([0.0, 1.0], offset=-20.0)])
    saveat = dfx.SaveAt(steps=True, t1=True)
    sol, r = solve_pair(dfx.LotkaVolterra(), dfx.Tsit5(),
                        dfx.PIDController(rtol=1e-7, atol=1e-9), saveat, ev, 60.0, 0.0, -0.1,
                        y0, LV_ARGS, torch.float64, kernel)
    check_parity(sol, r, ev)
    assert set(np.unique(r["event_index"])) == {0, 1}  # both conditions fire somewhere


@pytest.mark.parametrize("kernel", ["plain", "fused"])
def test_event_root_with_steps_and_dense(kernel):
    # The root finder with SaveAt(steps=2, t0, ts) and dense output: the save
    # after the event is dropped and the event's (t, y) saved in its place.
    rng = np.random.default_rng(33)
    B = 64
    y0 = rng.uniform(-2, 2, (B, 2))
    mu = np.exp(rng.uniform(np.log(0.1), np.log(3.0), (B, 1)))
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-8, 1e-8), direction=False)
    saveat = dfx.SaveAt(t0=True, ts=np.linspace(0.0, 12.0, 7), steps=2, dense=True)
    sol, r = solve_pair(dfx.VanDerPol(), dfx.Dopri5(),
                        dfx.PIDController(rtol=1e-7, atol=1e-9, pcoeff=0.3, icoeff=0.4),
                        saveat, ev, 0.0, 12.0, None, y0, mu, torch.float64, kernel)
    check_parity(sol, r, ev)


def test_event_steady_state_infinite_t1():
    # Ornstein-Uhlenbeck drift theta (mu - y) settles; steady_state_event with
    # the PID tolerances ends the solve (t1 = inf).
    rng = np.random.default_rng(34)
    B = 64
    y0 = rng.uniform(-3, 3, (B, 2))
    args = np.array([1.5, 0.5, 0.0])
    ev = dfx.Event(dfx.steady_state_event())
    sol, r = solve_pair(dfx.OrnsteinUhlenbeck(), dfx.Tsit5(),
                        dfx.PIDController(rtol=1e-4, atol=1e-6), dfx.SaveAt(t1=True), ev, 0.0,
                        np.inf, 0.1, y0, args, torch.float64, "fused")
    check_parity(sol, r, ev)
    assert (r["event_index"] == 0).all()
    assert np.allclose(sol.ys.cpu().numpy()[:, 0], 0.5, atol=1e-3)


def test_event_at_t0_and_constant_infinite_t1():
    # A boolean condition true at t0 ends the solve with no step; a constant
    # step grid to t1 = inf stops on t >= 3.
    y0 = np.array([[1.0, -0.5], [1.0, 0.5]])
    args = np.array([0.0, 0.0, 0.0])  # y' = 0
    ev = dfx.Event(dfx.LinearCondition([0.0, -1.0], boolean=True))
    sol, r = solve_pair(dfx.OrnsteinUhlenbeck(), dfx.Tsit5(), dfx.ConstantStepSize(),
                        dfx.SaveAt(t1=True), ev, 0.0, 10.0, 0.5, y0, args, torch.float64,
                        "plain")
    assert list(sol.stats["num_steps"].cpu().numpy()) == [0, 20]
    assert list(event_index(sol, ev)) == [0, -1] and list(r["event_index"]) == [0, -1]
    assert list(sol.ts.cpu().numpy()[:, 0]) == [0.0, 10.0]
    ev = dfx.Event(dfx.LinearCondition([], t_coeff=1.0, offset=-3.0))
    sol, r = solve_pair(dfx.OrnsteinUhlenbeck(), dfx.Heun(), dfx.ConstantStepSize(),
                        dfx.SaveAt(steps=True), ev, 0.0, np.inf, 0.5, y0, args,
                        torch.float64, "fused")
    ts = sol.ts.cpu().numpy()
    assert list(ts[0][np.isfinite(ts[0])]) == [0.5, 1.0, 1.5, 2.0, 2.5, 3.0]
    assert np.array_equal(ts, r["ts"])


def test_event_fp32_fused_van_der_pol():
    # FP32 state (FP64 time) on the headline shape: x crossing 0 downwards,
    # located by Newton(1e-5, 1e-5); event times within the solve's accuracy.
    rng = np.random.default_rng(35)
    B = 1024
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), (B, 1)))
    y0 = rng.uniform(-2, 2, (B, 2))
    t1 = rng.uniform(5, 50, B)
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-5, 1e-5), direction=False)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    sol, r = solve_pair(dfx.VanDerPol(), dfx.Dopri5(), pid, dfx.SaveAt(t1=True), ev, 0.0, t1,
                        None, y0, mu, torch.float32, "fused")
    idx = event_index(sol, ev)
    assert (idx == r["event_index"]).mean() > 0.99
    both = (idx == 0) & (r["event_index"] == 0)
    tg, to = sol.ts.cpu().numpy()[both, 0], r["ts"][both, 0]
    assert np.median(np.abs(tg - to)) < 1e-4 and np.abs(tg - to).max() < 1e-2
    assert np.abs(sol.ys.cpu().numpy()[both, 0, 0]).max() < 1e-4
