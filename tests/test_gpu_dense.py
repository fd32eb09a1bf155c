"""GPU parity of SaveAt(steps=n) and SaveAt(dense=True) (the extended-output
analytic-field kernels and gbdx_dense_evaluate) against the FP64 oracle.

FP64-state solves follow the oracle's arithmetic: trajectories that take the
oracle's step sequence (at least 95 % of each batch) must reproduce its saved
values, step times, dense records and interpolated values to 1e-9 relative.
FP32-state solves must agree within the solve's tolerance.
Reference behaviour: diffrax/_integrate.py:492-540, 847-877, 1273-1323 and
diffrax/_global_interpolation.py:315-393; the reference's tests of it are
test/test_saveat_solution.py:116-368 (restated on the oracle in
tests/test_oracle_pins.py).
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu

SOLVERS = {"euler": dfx.Euler(), "heun": dfx.Heun(), "dopri5": dfx.Dopri5(),
           "tsit5": dfx.Tsit5()}
LV_ARGS = np.array([0.1, 0.02, 0.4, 0.02])


def solve_pair(field, solver, controller, saveat, t0, t1, dt0, y0, args, dtype, kernel,
               max_steps=4096):
    """The GPU solve and the oracle's on the same inputs."""
    dev = torch.device("cuda")
    tt = lambda x: torch.tensor(x, dtype=torch.float64, device=dev) if isinstance(  # noqa
        x, np.ndarray) else x
    args_t = None if args is None else torch.tensor(args, dtype=dtype, device=dev)
    sol = dfx.diffeqsolve(dfx.ODETerm(field), solver, tt(t0), tt(t1), tt(dt0),
                          torch.tensor(y0, dtype=dtype, device=dev), args_t, saveat=saveat,
                          stepsize_controller=controller, max_steps=max_steps, throw=False,
                          kernel=kernel)
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(dfx.ODETerm(field), solver, controller, saveat, dim=y0.shape[1],
                       dtype=dtype, max_steps=max_steps, n_ts=0 if ts is None else ts.size)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, t0, t1, dt0, y0, args=args, ts=ts, nthreads=8)
    return sol, r, d


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


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("solver", ["heun", "dopri5", "tsit5"])
@pytest.mark.parametrize("steps", [1, 3])
def test_saveat_steps_fp64_matches_oracle(kernel, solver, steps):
    # Lotka-Volterra, PID(1e-6, 1e-8), t in [0, 140], dt0 = 0.1, with the
    # t0 and t1 saves around the step saves.
    rng = np.random.default_rng(7)
    y0 = rng.uniform(5, 15, (128, 2))
    saveat = dfx.SaveAt(t0=True, t1=True, steps=steps)
    sol, r, d = solve_pair(dfx.LotkaVolterra(), SOLVERS[solver],
                           dfx.PIDController(rtol=1e-6, atol=1e-8), saveat, 0.0, 140.0, 0.1,
                           y0, LV_ARGS, torch.float64, kernel)
    n = 1 + 4096 // steps + (1 if 4096 % steps else 0)
    assert tuple(sol.ys.shape) == (128, n, 2) and O.n_saves(d) == n
    same = same_steps(sol, r)
    rows_close(sol.ys.cpu().numpy(), r["ys"], same, 1e-9)
    rows_close(sol.ts.cpu().numpy(), r["ts"], same, 1e-9)
    assert np.array_equal(sol.result.cpu().numpy(), r["result"])


@pytest.mark.parametrize("kernel", ["plain", "fused"])
def test_saveat_steps_reverse_time_with_ts(kernel):
    # Van der Pol integrated backwards from t0 = 12 to per-trajectory t1 in
    # [0, 4], Dopri5 PID; ts (decreasing) and every 2nd step, plus t1.
    rng = np.random.default_rng(8)
    B = 96
    y0 = rng.uniform(-2, 2, (B, 2))
    mu = np.exp(rng.uniform(np.log(0.1), np.log(3.0), (B, 1)))
    t1 = rng.uniform(0.0, 4.0, B)
    saveat = dfx.SaveAt(ts=np.linspace(12.0, 4.0, 9), steps=2, t1=True)
    sol, r, d = solve_pair(dfx.VanDerPol(), dfx.Dopri5(),
                           dfx.PIDController(rtol=1e-7, atol=1e-9), saveat, 12.0, t1, None, y0,
                           mu, torch.float64, kernel, max_steps=1001)
    same = same_steps(sol, r)
    rows_close(sol.ys.cpu().numpy(), r["ys"], same, 1e-9)
    rows_close(sol.ts.cpu().numpy(), r["ts"], same, 1e-9)
    # unused slots hold direction * inf, i.e. -inf backwards in time
    ts = sol.ts.cpu().numpy()
    assert np.isneginf(ts[:, -1]).all()


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("reverse", [False, True])
def test_constant_grid_times_equal_oracle_bit_for_bit(kernel, dtype, reverse):
    # ConstantStepSize steps to t0 + (t1 - t0) (n / N) (constant.py:84-86).
    # The kernels form n / N from RN(1 / N) with an FMA correction and round
    # the product and the sum separately: every step time must equal the
    # oracle's (a C division, no contraction) bit for bit, for per-trajectory
    # t1 (N from 73 to 219) and an awkward dt0, forward and backward in time
    rng = np.random.default_rng(31)
    B = 256
    y0 = rng.uniform(5, 15, (B, 2))
    ends = rng.uniform(1.0, 3.0, B)
    t0, t1, dt0 = (ends, 0.0, -0.0137) if reverse else (0.0, ends, 0.0137)
    sol, r, _ = solve_pair(dfx.LotkaVolterra(), dfx.Euler(), dfx.ConstantStepSize(),
                           dfx.SaveAt(steps=1, t1=True), t0, t1, dt0, y0, LV_ARGS, dtype,
                           kernel, max_steps=256)
    assert (sol.result.cpu().numpy() == 0).all()
    assert np.array_equal(sol.stats["num_steps"].cpu().numpy(), r["stats"][:, 0])
    assert np.array_equal(sol.ts.cpu().numpy(), r["ts"])


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("solver", ["euler", "heun", "dopri5", "tsit5"])
def test_dense_fp64_matches_oracle(kernel, solver):
    rng = np.random.default_rng(9)
    B, T1 = 64, 30.0
    y0 = rng.uniform(5, 15, (B, 2))
    ctrl = {"euler": dfx.ConstantStepSize(), "heun": dfx.PIDController(rtol=1e-5, atol=1e-7)
            }.get(solver, dfx.PIDController(rtol=1e-6, atol=1e-8))
    dt0 = 0.05 if solver == "euler" else 0.1
    saveat = dfx.SaveAt(t1=True, dense=True)
    sol, r, d = solve_pair(dfx.LotkaVolterra(), SOLVERS[solver], ctrl, saveat, 0.0, T1, dt0,
                           y0, LV_ARGS, torch.float64, kernel, max_steps=4096)
    same = same_steps(sol, r)
    it = sol.interpolation
    assert np.array_equal(it.ts_size.cpu().numpy()[same], r["dense_n"][same])
    rows_close(it.ts.cpu().numpy(), r["dense_ts"], same, 1e-9)
    rows_close(it.infos.cpu().numpy(), r["dense_info"], same, 1e-9)
    # evaluate / derivative at shared and per-trajectory times, against the
    # oracle's DenseInterpolation over its own records
    q = np.linspace(0.0, T1, 41)
    for order in (0, 1):
        got = (sol.evaluate if order == 0 else sol.derivative)(torch.tensor(q))
        want = O.dense_evaluate(d, 0.0, T1, y0, r, q, order=order)
        rows_close(got.cpu().numpy(), want, same, 1e-9)
    qb = rng.uniform(0.0, T1, (B, 5))
    got = sol.evaluate(torch.tensor(qb, device="cuda"))
    rows_close(got.cpu().numpy(), O.dense_evaluate(d, 0.0, T1, y0, r, qb), same, 1e-9)
    # increments evaluate(t0, t1) and the scalar form
    inc = sol.evaluate(3.0, 7.5).cpu().numpy()
    want = (O.dense_evaluate(d, 0.0, T1, y0, r, [7.5]) -
            O.dense_evaluate(d, 0.0, T1, y0, r, [3.0]))[:, 0]
    rows_close(inc, want, same, 1e-8)
    # out of [t0, t1]: NaN
    assert torch.isnan(sol.evaluate(T1 + 1.0)).all() and torch.isnan(sol.evaluate(-1.0)).all()


@pytest.mark.parametrize("left", [True, False])
def test_dense_step_boundary_side(left):
    # A query exactly on a step boundary takes the step on its left (left=True)
    # or on its right (_interpret_t, searchsorted side).
    rng = np.random.default_rng(10)
    B = 32
    y0 = rng.uniform(5, 15, (B, 2))
    saveat = dfx.SaveAt(t1=True, dense=True)
    sol, r, d = solve_pair(dfx.LotkaVolterra(), dfx.Tsit5(),
                           dfx.PIDController(rtol=1e-6, atol=1e-8), saveat, 0.0, 20.0, 0.1, y0,
                           LV_ARGS, torch.float64, "fused", max_steps=512)
    same = same_steps(sol, r)
    qb = r["dense_ts"][:, 3:4].copy()  # the end of each trajectory's third step
    for order in (0, 1):
        got = sol.interpolation._run(torch.tensor(qb), left, order).cpu().numpy()
        want = O.dense_evaluate(d, 0.0, 20.0, y0, r, qb, left=left, order=order)
        rows_close(got, want, same, 1e-9)


def test_dense_fp32_van_der_pol_uneven_t1():
    # The headline workload's shape (FP32 state, Dopri5 PID(1e-6, 1e-9,
    # p=0.3, i=0.4), uneven t1, dt0=None) with dense output on the fused kernel.
    rng = np.random.default_rng(11)
    B = 512
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), (B, 1)))
    y0 = rng.uniform(-2, 2, (B, 2))
    t1 = rng.uniform(5, 50, B)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    sol, r, d = solve_pair(dfx.VanDerPol(), dfx.Dopri5(), pid,
                           dfx.SaveAt(t1=True, dense=True), 0.0, t1, None, y0, mu,
                           torch.float32, "fused")
    qb = t1[:, None] * np.array([[0.1, 0.5, 0.9, 1.0]])
    got = sol.evaluate(torch.tensor(qb)).cpu().double().numpy()
    want = O.dense_evaluate(d, 0.0, t1, y0, r, qb)
    per = np.abs(got - want).max(axis=(1, 2)) / np.abs(want).max(axis=(1, 2))
    assert np.median(per) < 1e-4 and per.max() < 5e-2, (np.median(per), per.max())
    # the value at t1 is the t1 save
    assert np.allclose(got[:, -1], sol.ys.cpu().double().numpy()[:, 0], rtol=1e-5, atol=1e-6)


def test_dense_only_and_trivial_solve():
    # SaveAt(dense=True) alone saves no ys; a solve with t0 == t1 evaluates to
    # y0 at t0 with zero derivative (_global_interpolation.py:344-345).
    y0 = np.array([[1.0, 2.0], [3.0, 4.0]])
    dev = torch.device("cuda")
    sol = dfx.diffeqsolve(dfx.ODETerm(dfx.OrnsteinUhlenbeck()), dfx.Tsit5(), 0.5, 0.5, 0.1,
                          torch.tensor(y0, device=dev), torch.tensor([1.0, 0.0, 0.0], device=dev),
                          saveat=dfx.SaveAt(dense=True), max_steps=16)
    assert sol.ys is None and sol.ts is None
    assert torch.equal(sol.evaluate(0.5).cpu(), torch.tensor(y0))
    assert torch.equal(sol.derivative(0.5).cpu(), torch.zeros(2, 2, dtype=torch.float64))
    assert torch.isnan(sol.evaluate(0.6)).all()
    # decay y' = -y: evaluate close to exp(-t) y0
    sol = dfx.diffeqsolve(dfx.ODETerm(dfx.OrnsteinUhlenbeck()), dfx.Tsit5(), 0.0, 2.0, 0.1,
                          torch.tensor(y0, device=dev), torch.tensor([1.0, 0.0, 0.0], device=dev),
                          saveat=dfx.SaveAt(dense=True),
                          stepsize_controller=dfx.PIDController(rtol=1e-8, atol=1e-8))
    for t in (0.3, 1.0, 1.7):
        assert np.allclose(sol.evaluate(t).cpu().numpy(), np.exp(-t) * y0, rtol=1e-6)
        assert np.allclose(sol.derivative(t).cpu().numpy(), -np.exp(-t) * y0, rtol=1e-3)
