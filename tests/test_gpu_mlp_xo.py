"""SaveAt(steps=n), SaveAt(dense=True) and ClipStepSizeController on the MLP
fields (the fused MLP integrator) against the FP64 oracle on the same inputs
(diffrax/_integrate.py:492-540, 847-877, 1273-1323;
diffrax/_global_interpolation.py:315-393; _step_size_controller/clip.py).

With constant steps both precisions (FP32 parity mode, three-piece BF16)
take the oracle's steps and must reproduce its step saves, step times and
interpolated values to FP32 accuracy.  Adaptive solves run at a tolerance
well above FP32 rounding, where the FP32 controller takes the oracle's step
counts (its step sizes differ by the FP32 rounding of the factors).
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O
from test_gpu_mlp import mlp_params, flat, sde_setup

pytestmark = pytest.mark.gpu


def mlp_pair(widths, solver, controller, saveat, t1, dt0, y0, precision, seed=0,
             diffusion=None, bm=None, max_steps=256, step_ts=None, jump_ts=None):
    dev = torch.device("cuda")
    Ws, bs = mlp_params(widths, seed, bias_scale=0.1)
    Ws = [W.astype(np.float32).astype(np.float64) for W in Ws]
    bs = [b.astype(np.float32).astype(np.float64) for b in bs]
    field = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                         [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs],
                         precision=precision)
    params = flat(Ws, bs)
    if diffusion is not None:
        Wsig, bsig = diffusion
        terms = dfx.MultiTerm(dfx.ODETerm(field), dfx.ControlTerm(
            dfx.TanhDiagonalDiffusion(torch.tensor(Wsig, dtype=torch.float32, device=dev),
                                      torch.tensor(bsig, dtype=torch.float32, device=dev)),
            bm))
        params = np.concatenate([params, Wsig.reshape(-1), bsig])
    else:
        terms = dfx.ODETerm(field)
    sol = dfx.diffeqsolve(terms, solver, 0.0, t1, dt0,
                          torch.tensor(y0, dtype=torch.float32, device=dev), saveat=saveat,
                          stepsize_controller=controller, max_steps=max_steps, throw=False)
    torch.cuda.synchronize()
    fields = dfx.lower(terms, solver, controller, saveat, dim=y0.shape[1],
                       dtype=torch.float32, max_steps=max_steps, n_ts=0)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, 0.0, t1, dt0, y0, params=params, nthreads=8, step_ts=step_ts,
                jump_ts=jump_ts)
    return sol, r, d


def compare_rows(sol, r, tol, ts_tol=1e-12):
    """Trajectories with the oracle's step counts (at least 95 %): saved ys
    within tol and ts within ts_tol of the row's largest value, the same
    +inf padding."""
    same = sol.stats["num_accepted_steps"].cpu().numpy() == r["stats"][:, 1]
    assert same.mean() >= 0.95, f"only {same.mean():.3f} took the oracle's steps"
    ys = sol.ys.cpu().double().numpy()[same]
    ts = sol.ts.cpu().numpy()[same]
    ry, rt = r["ys"][same], r["ts"][same]
    assert np.array_equal(np.isfinite(ys), np.isfinite(ry))
    assert np.array_equal(np.isfinite(ts), np.isfinite(rt))
    fin = np.isfinite(rt)
    assert np.abs(ts[fin] - rt[fin]).max() <= ts_tol * np.abs(rt[fin]).max()
    fy = np.isfinite(ry)
    err = np.abs(ys[fy] - ry[fy]).max() / np.abs(ry[fy]).max()
    print(f"steps equal {same.mean():.3f}, max rel err {err:.2e}")
    assert err < tol
    return same


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("solver", ["tsit5", "dopri5"])
@pytest.mark.parametrize("steps", [1, 3])
def test_mlp_saveat_steps_matches_oracle(steps, solver, precision):
    # 64 -> 128 -> 128 -> 64, ConstantStepSize dt 0.05 on [0, 1] (20 steps):
    # every (steps=1) or every 3rd step saved, then t1 unless a step save
    # already holds it; max_steps 64 leaves +inf slots
    rng = np.random.default_rng(21)
    y0 = rng.standard_normal((192, 64))
    solver = {"tsit5": dfx.Tsit5(), "dopri5": dfx.Dopri5()}[solver]
    sol, r, _ = mlp_pair([64, 128, 128, 64], solver, dfx.ConstantStepSize(),
                         dfx.SaveAt(steps=steps, t1=True), 1.0, 0.05, y0, precision, seed=3,
                         max_steps=64)
    assert sol.ys.shape == r["ys"].shape
    compare_rows(sol, r, 5e-6, ts_tol=0.0)  # the grid times bit for bit


def test_mlp_wide_saveat_steps_and_dense_match_oracle():
    # 64 -> 256 -> 256 -> 64, Dopri5, dt 0.1 on [0, 1]: step saves and the
    # dense interpolation (value and derivative) at 33 times
    rng = np.random.default_rng(22)
    y0 = rng.standard_normal((128, 64))
    sol, r, d = mlp_pair([64, 256, 256, 64], dfx.Dopri5(), dfx.ConstantStepSize(),
                         dfx.SaveAt(steps=2, t1=True, dense=True), 1.0, 0.1, y0, "fp32",
                         seed=4, max_steps=32)
    compare_rows(sol, r, 5e-6)
    q = np.linspace(0.0, 1.0, 33)
    ev = sol.evaluate(torch.tensor(q, dtype=torch.float64, device="cuda")).cpu().double()
    rq = O.dense_evaluate(d, 0.0, 1.0, y0, r, q)
    err = np.abs(ev.numpy() - rq).max() / np.abs(rq).max()
    print(f"dense evaluation max rel err {err:.2e}")
    assert err < 5e-6
    dv = sol.derivative(torch.tensor(q, dtype=torch.float64, device="cuda")).cpu().double()
    rd = O.dense_evaluate(d, 0.0, 1.0, y0, r, q, order=1)
    errd = np.abs(dv.numpy() - rd).max() / np.abs(rd).max()
    print(f"dense derivative max rel err {errd:.2e}")
    # the interpolant's derivative differences the FP32 stage increments
    assert errd < 5e-4


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_mlp_adaptive_step_saves(precision):
    # Tsit5 + PID(1e-3, 1e-4) on [0, 3], every accepted step saved.  The FP32
    # controller grows steps less than the FP64 one (its error estimate
    # carries FP32 rounding), so the step times are checked against the
    # solve's own: one save per accepted step, increasing, the last at t1 with
    # the value a SaveAt(t1=True) solve of the same problem gives
    dev = torch.device("cuda")
    rng = np.random.default_rng(27)
    y0 = rng.standard_normal((128, 64))
    ctrl = dfx.PIDController(rtol=1e-3, atol=1e-4)
    sol, r, _ = mlp_pair([64, 128, 128, 64], dfx.Tsit5(), ctrl, dfx.SaveAt(steps=1, t1=True),
                         3.0, None, y0, precision, seed=1)
    n = sol.stats["num_accepted_steps"].cpu().numpy()
    ts = sol.ts.cpu().numpy()
    fin = np.isfinite(ts)
    assert np.array_equal(fin.sum(axis=1), n)  # steps=1 saves every step; t1 is the last
    for row in range(ts.shape[0]):
        t = ts[row, :n[row]]
        assert (np.diff(t) > 0).all() and t[-1] == 3.0
    last = sol.ys[torch.arange(128, device=dev), torch.tensor(n - 1, device=dev)]
    t1_sol, _, _ = mlp_pair([64, 128, 128, 64], dfx.Tsit5(), ctrl, dfx.SaveAt(t1=True), 3.0,
                            None, y0, precision, seed=1)
    assert torch.allclose(last, t1_sol.ys[:, 0], rtol=1e-6, atol=1e-6)
    ry = r["ys"][np.arange(128), r["stats"][:, 1] - 1]
    assert np.abs(last.cpu().double().numpy() - ry).max() < 1e-2 * np.abs(ry).max()


def test_mlp_dense_is_consistent_with_step_saves_bf16():
    # the dense record at an accepted step's end time reproduces that step's
    # saved value (both written by the same kernel from the same registers)
    rng = np.random.default_rng(23)
    y0 = rng.standard_normal((256, 64))
    ctrl = dfx.PIDController(rtol=1e-5, atol=1e-7)
    sol, _, _ = mlp_pair([64, 128, 128, 64], dfx.Tsit5(), ctrl,
                         dfx.SaveAt(steps=1, dense=True), 1.0, None, y0, "bf16", seed=5)
    ts = sol.ts.clone()
    ok = torch.isfinite(ts)
    ts[~ok] = 0.0
    ev = sol.evaluate(ts)  # [B, Q, D] at each trajectory's own step times
    diff = (ev - sol.ys)[ok]
    assert float(diff.abs().max()) <= 1e-6 * float(sol.ys[ok].abs().max())


def test_neural_sde_saveat_steps_matches_oracle():
    # drift 32 -> 64 -> 64 -> 32, diffusion 0.1 tanh(W y + b), Heun dt 0.05,
    # the same Brownian path: every 2nd step saved
    rng = np.random.default_rng(24)
    y0 = rng.standard_normal((128, 32))
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (32,), key=77)
    sol, r, _ = mlp_pair([32, 64, 64, 32], dfx.Heun(), dfx.ConstantStepSize(),
                         dfx.SaveAt(steps=2, t1=True), 1.0, 0.05, y0, "fp32", seed=6,
                         diffusion=sde_setup(25), bm=bm)
    assert sol.ys.shape[1] == 128  # max_steps / 2 slots, t1 already a step save
    compare_rows(sol, r, 1e-4)


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_mlp_clip_controller_matches_oracle(precision):
    # Tsit5 + ClipStepSizeController(PID(1e-3, 1e-4), step_ts, jump_ts) on
    # the 64 -> 128 -> 128 -> 64 field over [0, 3], every step saved: the step
    # times hit every step_ts exactly, end just before each jump and restart
    # past it; the step counts are the oracle's
    rng = np.random.default_rng(26)
    y0 = rng.standard_normal((160, 64))
    step_ts = np.array([0.3, 0.75, 1.5, 2.25])
    jump_ts = np.array([1.0, 2.0])
    ctrl = dfx.ClipStepSizeController(dfx.PIDController(rtol=1e-3, atol=1e-4),
                                      step_ts=step_ts, jump_ts=jump_ts)
    sol, r, _ = mlp_pair([64, 128, 128, 64], dfx.Tsit5(), ctrl, dfx.SaveAt(steps=1), 3.0,
                         None, y0, precision, seed=8, step_ts=step_ts, jump_ts=jump_ts)
    same = compare_rows(sol, r, 1e-2, ts_tol=1e-4)
    ts = sol.ts.cpu().numpy()
    for row in range(ts.shape[0]):
        t = ts[row][np.isfinite(ts[row])]
        for st in step_ts:
            assert st in t
        for jt in jump_ts:
            assert np.nextafter(jt, -np.inf) in t
    assert np.array_equal(sol.stats["num_steps"].cpu().numpy()[same], r["stats"][same, 0])


def contracting_mlp(dev, D=64, H=128, scale=1.0):
    """f(y) = -s W2 tanh(W1 tanh(W0 y)) with W0 = [I; I]/2, W1 = I,
    W2 = [I, I]/2 (BF16-exact): a field with f(y) ~ -s y/2 near 0, so every
    trajectory decays to the steady state y = 0."""
    W0 = np.concatenate([np.eye(D), np.eye(D)], axis=0)[:H] * 0.5
    W1 = np.eye(H)
    W2 = -scale * np.concatenate([np.eye(D), np.eye(D)], axis=1)[:, :H] * 0.5
    Ws = [W0, W1, W2]
    bs = [np.zeros(H), np.zeros(H), np.zeros(D)]
    return Ws, bs


def mlp_event_pair(Ws, bs, solver, controller, saveat, event, t1, dt0, y0, precision,
                   max_steps=1024):
    dev = torch.device("cuda")
    field = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                         [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs],
                         precision=precision)
    sol = dfx.diffeqsolve(dfx.ODETerm(field), solver, 0.0, t1, dt0,
                          torch.tensor(y0, dtype=torch.float32, device=dev), saveat=saveat,
                          stepsize_controller=controller, event=event, max_steps=max_steps,
                          throw=False)
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(dfx.ODETerm(field), solver, controller, saveat, dim=y0.shape[1],
                       dtype=torch.float32, max_steps=max_steps,
                       n_ts=0 if ts is None else ts.size, event=event)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, 0.0, t1, dt0, y0, params=flat(Ws, bs), ts=ts, nthreads=8)
    return sol, r


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("solver", ["tsit5", "heun"])
def test_mlp_steady_state_event_matches_oracle(solver, precision):
    # a contracting 64 -> 128 -> 128 -> 64 field, dt 0.1 on [0, 60]: the
    # steady-state event (rtol 1e-3, atol 1e-3) ends each trajectory at the
    # first step end where rms f < atol + rtol rms y; Heun evaluates f(y1)
    # for it, Tsit5 reuses its FSAL value.  Some trajectories start at the
    # steady state already and end at t0.
    rng = np.random.default_rng(28)
    B = 128
    y0 = rng.standard_normal((B, 64)) * rng.uniform(0.0, 3.0, (B, 1))
    y0[:4] = 1e-5
    Ws, bs = contracting_mlp(None)
    solver = {"tsit5": dfx.Tsit5(), "heun": dfx.Heun()}[solver]
    ev = dfx.Event(dfx.steady_state_event(rtol=1e-3, atol=1e-3))
    sol, r = mlp_event_pair(Ws, bs, solver, dfx.ConstantStepSize(),
                            dfx.SaveAt(t1=True, steps=5), ev, 60.0, 0.1, y0, precision)
    res = sol.result.cpu().numpy()
    assert (res == int(dfx.RESULTS.event_occurred)).all() and (r["result"] == 3).all()
    assert bool(sol.event_mask.all())
    n = sol.stats["num_steps"].cpu().numpy()
    same = n == r["stats"][:, 0]
    print(f"steady state: steps equal {same.mean():.3f}, steps {n.min()}..{n.max()}")
    assert same.mean() >= 0.95
    assert (n[:4] == 0).all()  # already steady at t0
    compare_rows(sol, r, 5e-5 if precision == "bf16" else 1e-5)


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("direction", [None, True])
def test_mlp_linear_event_root_matches_oracle(direction, precision):
    # 64 -> 128 -> 128 -> 64 (random BF16 weights), Tsit5 dt 0.02 on [0, 4]:
    # y0 + 0.5 y1 crossing 0.25 ends the solve at the root of the step's
    # interpolant (Newton(1e-6, 1e-6)); ts saves after the root are not made
    rng = np.random.default_rng(29)
    B = 160
    y0 = rng.standard_normal((B, 64))
    Ws, bs = mlp_params([64, 128, 128, 64], 11, bias_scale=0.1)
    Ws = [W.astype(np.float32).astype(np.float64) for W in Ws]
    bs = [b.astype(np.float32).astype(np.float64) for b in bs]
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.5], offset=-0.25), dfx.Newton(1e-6, 1e-6),
                   direction=direction)
    saveat = dfx.SaveAt(ts=np.linspace(0.0, 4.0, 9), t1=True)
    sol, r = mlp_event_pair(Ws, bs, dfx.Tsit5(), dfx.ConstantStepSize(), saveat, ev, 4.0, 0.02,
                            y0, precision)
    res = sol.result.cpu().numpy()
    mask = sol.event_mask.cpu().numpy()
    # the FP32 solve and the FP64 oracle agree on which trajectories fire (a
    # crossing within FP32 rounding of the step's end may go either way)
    agree = (res == r["result"]) & (mask == (r["event_index"] == 0))
    fired = r["event_index"] == 0
    print(f"linear event: {fired.mean():.3f} fired, {agree.mean():.3f} agree")
    assert agree.mean() >= 0.97 and fired.mean() > 0.1
    ts, rt = sol.ts.cpu().numpy()[agree], r["ts"][agree]
    assert np.array_equal(np.isfinite(ts), np.isfinite(rt))
    fin = np.isfinite(rt)
    assert np.abs(ts[fin] - rt[fin]).max() < 1e-5
    ys, ry = sol.ys.cpu().double().numpy()[agree], r["ys"][agree]
    fy = np.isfinite(ry)
    assert np.abs(ys[fy] - ry[fy]).max() < 1e-4 * np.abs(ry[fy]).max()
    # the final save of a trajectory whose root find converged sits on the
    # condition's zero
    ok = (fired & (res == 3))[agree]
    last = np.array([ys[b][np.isfinite(ts[b])][-1] for b in range(ys.shape[0])])
    g = last[:, 0] + 0.5 * last[:, 1] - 0.25
    assert np.abs(g[ok]).max() < 1e-4


def test_mlp_reverse_time_steps_dense_and_event():
    # t0 = 1 > t1 = 0, Tsit5 dt 0.05 (the loop runs in flipped time): step
    # saves, the dense output and a downward crossing with Newton, against
    # the oracle
    rng = np.random.default_rng(30)
    B = 128
    y0 = rng.standard_normal((B, 64))
    Ws, bs = mlp_params([64, 128, 128, 64], 12, bias_scale=0.1)
    Ws = [W.astype(np.float32).astype(np.float64) for W in Ws]
    bs = [b.astype(np.float32).astype(np.float64) for b in bs]
    dev = torch.device("cuda")
    field = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                         [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs],
                         precision="fp32")
    ev = dfx.Event(dfx.LinearCondition([1.0], offset=-0.5), dfx.Newton(1e-6, 1e-6),
                   direction=False)
    saveat = dfx.SaveAt(steps=2, t1=True, dense=True)
    sol = dfx.diffeqsolve(dfx.ODETerm(field), dfx.Tsit5(), 1.0, 0.0, -0.05,
                          torch.tensor(y0, dtype=torch.float32, device=dev), saveat=saveat,
                          stepsize_controller=dfx.ConstantStepSize(), event=ev, max_steps=64,
                          throw=False)
    torch.cuda.synchronize()
    fields = dfx.lower(dfx.ODETerm(field), dfx.Tsit5(), dfx.ConstantStepSize(), saveat, dim=64,
                       dtype=torch.float32, max_steps=64, n_ts=0, event=ev)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, 1.0, 0.0, -0.05, y0, params=flat(Ws, bs), nthreads=8)
    res = sol.result.cpu().numpy()
    agree = (res == r["result"]) & (sol.event_mask.cpu().numpy() == (r["event_index"] == 0))
    assert agree.mean() >= 0.97
    ts, rt = sol.ts.cpu().numpy()[agree], r["ts"][agree]
    assert np.array_equal(np.isneginf(ts), np.isneginf(rt))  # direction * inf padding
    fin = np.isfinite(rt)
    assert np.abs(ts[fin] - rt[fin]).max() < 1e-5
    ys, ry = sol.ys.cpu().double().numpy()[agree], r["ys"][agree]
    fy = np.isfinite(ry)
    assert np.abs(ys[fy] - ry[fy]).max() < 1e-4 * np.abs(ry[fy]).max()
    q = np.linspace(1.0, 0.3, 15)
    ev_q = sol.evaluate(torch.tensor(q, dtype=torch.float64, device=dev)).cpu().double().numpy()
    rq = O.dense_evaluate(d, 1.0, 0.0, y0, r, q)
    ok = np.isfinite(rq).all(axis=(1, 2)) & agree
    assert np.abs(ev_q[ok] - rq[ok]).max() < 1e-4 * np.abs(rq[ok]).max()


def test_mlp_two_conditions_with_steps_and_dense():
    # a boolean condition on time and a real one on y1, no root finder, with
    # every 3rd step saved and the dense output (the first condition that
    # fires, in order, ends the solve at the step's end)
    rng = np.random.default_rng(31)
    B = 128
    y0 = rng.standard_normal((B, 64))
    Ws, bs = mlp_params([64, 128, 128, 64], 14, bias_scale=0.1)
    Ws = [W.astype(np.float32).astype(np.float64) for W in Ws]
    bs = [b.astype(np.float32).astype(np.float64) for b in bs]
    ev = dfx.Event([dfx.LinearCondition([], t_coeff=1.0, offset=-0.6, boolean=True),
                    dfx.LinearCondition([0.0, 1.0], offset=-0.3)])
    saveat = dfx.SaveAt(steps=3, t1=True, dense=True)
    sol, r = mlp_event_pair(Ws, bs, dfx.Tsit5(), dfx.ConstantStepSize(), saveat, ev, 1.0, 0.05,
                            y0, "fp32", max_steps=64)
    masks = [m.cpu().numpy() for m in sol.event_mask]
    evi = np.where(masks[0], 0, np.where(masks[1], 1, -1))
    agree = (evi == r["event_index"]) & (sol.result.cpu().numpy() == r["result"])
    print(f"two conditions: fired {np.bincount(r['event_index'] + 1)}, agree {agree.mean():.3f}")
    assert agree.mean() >= 0.97 and (r["event_index"] == 0).any() and (r["event_index"] == 1).any()
    ts, rt = sol.ts.cpu().numpy()[agree], r["ts"][agree]
    assert np.array_equal(np.isfinite(ts), np.isfinite(rt))
    fin = np.isfinite(rt)
    assert np.abs(ts[fin] - rt[fin]).max() < 1e-9
    ys, ry = sol.ys.cpu().double().numpy()[agree], r["ys"][agree]
    fy = np.isfinite(ry)
    assert np.abs(ys[fy] - ry[fy]).max() < 1e-5 * np.abs(ry[fy]).max()
