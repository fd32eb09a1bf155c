"""GPU parity of ClipStepSizeController(PIDController(...), step_ts, jump_ts)
(diffrax/_step_size_controller/clip.py:120-427) on the analytic-field kernels
against the FP64 oracle, which restates clip.py and is pinned to the
reference's test/test_adaptive_stepsize_controller.py in
tests/test_oracle_pins.py.

FP64-state solves must take the oracle's step sequence and reproduce its saved
steps to 1e-9 relative on at least 95 % of each batch; every step time and
jump edge must be stepped to exactly.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu

SOLVERS = {"heun": dfx.Heun(), "dopri5": dfx.Dopri5(), "tsit5": dfx.Tsit5()}
LV_ARGS = np.array([0.1, 0.02, 0.4, 0.02])


def solve_pair(field, solver, pid, step_ts, jump_ts, saveat, t0, t1, y0, args, dtype, kernel,
               max_steps=4096, dt0=None):
    dev = torch.device("cuda")
    tt = lambda x: torch.tensor(x, dtype=torch.float64, device=dev) if isinstance(  # noqa
        x, np.ndarray) else x
    ctrl = dfx.ClipStepSizeController(pid, step_ts=step_ts, jump_ts=jump_ts)
    sol = dfx.diffeqsolve(dfx.ODETerm(field), solver, tt(t0), tt(t1), tt(dt0),
                          torch.tensor(y0, dtype=dtype, device=dev),
                          torch.tensor(args, dtype=dtype, device=dev), saveat=saveat,
                          stepsize_controller=ctrl, max_steps=max_steps, throw=False,
                          kernel=kernel)
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(dfx.ODETerm(field), solver, ctrl, saveat, dim=y0.shape[1], dtype=dtype,
                       max_steps=max_steps, n_ts=0 if ts is None else ts.size)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, t0, t1, dt0, y0, args=args, ts=ts, nthreads=8, step_ts=step_ts,
                jump_ts=jump_ts)
    return sol, r


def same_steps(sol, r):
    same = sol.stats["num_steps"].cpu().numpy() == r["stats"][:, 0]
    same &= sol.stats["num_accepted_steps"].cpu().numpy() == r["stats"][:, 1]
    assert same.mean() >= 0.95, f"only {same.mean():.3f} of the batch took the oracle's steps"
    return same


def rows_close(a, b, rows, tol, min_frac=0.95, loose=1e-4):
    """Rows `rows` (the trajectories that took the oracle's step counts) of a
    and b: the same +-inf/NaN pattern, at least `min_frac` of the batch within
    tol relative to the row's largest magnitude, and all of them within `loose`
    (GPU and host FP64 pow differ by an ulp now and then, which can move a step
    and the solution by the solve's tolerance)."""
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
    return diff.max()


def hits(ts_row, times):
    return all(t in ts_row for t in times)


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("solver", ["heun", "dopri5", "tsit5"])
def test_clip_fp64_matches_oracle(kernel, solver):
    # Lotka-Volterra on [0, 60], PID(1e-6, 1e-8), step_ts and jump_ts, every
    # accepted step saved.
    rng = np.random.default_rng(21)
    B = 96
    y0 = rng.uniform(5, 15, (B, 2))
    step_ts, jump_ts = [12.5, 30.0, 41.25], [20.0, 47.5]
    tol = 1e-5 if solver == "heun" else 1e-6
    sol, r = solve_pair(dfx.LotkaVolterra(), SOLVERS[solver], dfx.PIDController(rtol=tol,
                        atol=tol * 1e-2), step_ts, jump_ts, dfx.SaveAt(steps=True, t1=True), 0.0,
                        60.0, y0, LV_ARGS, torch.float64, kernel, dt0=0.1)
    same = same_steps(sol, r)
    rows_close(sol.ys.cpu().numpy(), r["ys"], same, 1e-9)
    rows_close(sol.ts.cpu().numpy(), r["ts"], same, 1e-9)
    ts = sol.ts.cpu().numpy()
    ok = sol.result.cpu().numpy() == 0
    assert ok.all()
    pb, na = np.nextafter(20.0, -np.inf), np.nextafter(20.0, np.inf)
    for b in range(B):
        assert hits(ts[b], step_ts + [pb, np.nextafter(47.5, -np.inf)]) and 20.0 not in ts[b]
        # the step after the jump starts one ulp past it (clip.py:79-99)
        k = int(np.searchsorted(ts[b], pb))
        assert ts[b][k] == pb and ts[b][k + 1] > na


@pytest.mark.parametrize("kernel", ["plain", "fused"])
def test_clip_backwards_per_trajectory_t1(kernel):
    # Lotka-Volterra backwards from t0 = 60 to per-trajectory t1 in [0, 20],
    # Dopri5 PID(1e-7, 1e-9, p=0.3, i=0.4), step_ts and a jump inside.
    rng = np.random.default_rng(22)
    B = 64
    y0 = rng.uniform(5, 15, (B, 2))
    t1 = rng.uniform(0.0, 20.0, B)
    step_ts, jump_ts = [25.5, 40.0], [33.0]
    pid = dfx.PIDController(rtol=1e-7, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    sol, r = solve_pair(dfx.LotkaVolterra(), dfx.Dopri5(), pid, step_ts, jump_ts,
                        dfx.SaveAt(steps=True, t1=True), 60.0, t1, y0, LV_ARGS, torch.float64,
                        kernel)
    same = same_steps(sol, r)
    rows_close(sol.ys.cpu().numpy(), r["ys"], same, 1e-9)
    rows_close(sol.ts.cpu().numpy(), r["ts"], same, 1e-9)
    ts = sol.ts.cpu().numpy()
    assert (sol.result.cpu().numpy() == 0).all()
    for b in range(B):
        # backwards, the step before the jump ends one ulp above it
        assert hits(ts[b], step_ts + [np.nextafter(33.0, np.inf)]) and 33.0 not in ts[b]


def test_clip_fp32_fused_steps_exactly_to_step_ts():
    # FP32 state, FP64 time: the Van der Pol headline shape with step_ts; the
    # solve lands on every step time exactly and keeps the solve's accuracy.
    rng = np.random.default_rng(23)
    B = 512
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), (B, 1)))
    y0 = rng.uniform(-2, 2, (B, 2))
    step_ts = [2.5, 4.0]
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    sol, r = solve_pair(dfx.VanDerPol(), dfx.Dopri5(), pid, step_ts, [3.0],
                        dfx.SaveAt(steps=True, t1=True), 0.0, 5.0, y0, mu, torch.float32,
                        "fused")
    ts = sol.ts.cpu().numpy()
    assert (sol.result.cpu().numpy() == 0).all()
    for b in range(B):
        assert hits(ts[b], step_ts + [np.nextafter(3.0, -np.inf)])
    last = lambda a: np.stack([row[np.isfinite(row).all(axis=-1)][-1] for row in a])  # noqa
    got, want = last(sol.ys.cpu().double().numpy()), last(r["ys"])
    per = np.abs(got - want).max(axis=1) / np.abs(want).max(axis=1)
    assert np.median(per) < 1e-4 and per.max() < 5e-2, (np.median(per), per.max())


def test_clip_t0_just_before_jump():
    # A solve that starts at prevbefore(jump) takes a zero-length first step and
    # restarts past the jump (clip.py:354-372).
    y0 = np.array([[1.0, 0.5], [2.0, -1.0]])
    t0 = np.nextafter(0.98, -np.inf)
    # y' = 0 (Ornstein-Uhlenbeck drift with theta = 0)
    sol, r = solve_pair(dfx.OrnsteinUhlenbeck(), dfx.Heun(),
                        dfx.PIDController(rtol=1e-6, atol=1e-6), None, [0.98],
                        dfx.SaveAt(t1=True), t0, 1.2, y0, np.array([0.0, 0.0, 0.0]),
                        torch.float64, "plain", max_steps=100)
    assert (sol.result.cpu().numpy() == 0).all() and (r["result"] == 0).all()
    assert np.array_equal(sol.stats["num_steps"].cpu().numpy(), r["stats"][:, 0])
    assert (sol.ts.cpu().numpy() == 1.2).all()
    np.testing.assert_array_equal(sol.ys.cpu().numpy(), y0[:, None])
