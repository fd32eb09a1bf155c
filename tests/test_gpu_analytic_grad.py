"""GPU gradients of the analytic-field solves (Lotka-Volterra, Van der Pol,
Ornstein-Uhlenbeck ODE and SDE) with respect to y0 and args, through
diffeqsolve and torch.autograd, against the FP64 oracle's gradients on the
same inputs (diffrax/_adjoint.py:179-312 and 538-734; the reference
differentiates a field's arguments in test/test_adjoint.py:33-215).

FP64-state runs take the oracle's step sequence and must agree to ~1e-8; FP32
runs agree to the FP32 level.  Constant-step solves are also checked against
central finite differences of the GPU's own FP64 forward, and the linear
Ornstein-Uhlenbeck ODE against its closed-form gradient.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu

LV_ARGS = np.array([0.1, 0.02, 0.4, 0.02])
SOLVERS = {"euler": dfx.Euler(), "heun": dfx.Heun(), "dopri5": dfx.Dopri5(),
           "tsit5": dfx.Tsit5()}


def grad_pair(field, solver, ctrl, saveat, t0, t1, dt0, y0, args, dtype, adjoint, G,
              kernel="fused", terms=None):
    """GPU dL/dy0 and dL/dargs of L = sum(G * ys), and the oracle's."""
    dev = torch.device("cuda")
    terms = terms if terms is not None else dfx.ODETerm(field)
    y0_t = torch.tensor(y0, dtype=dtype, device=dev, requires_grad=True)
    a_t = torch.tensor(args, dtype=dtype, device=dev, requires_grad=True)
    sol = dfx.diffeqsolve(terms, solver, t0, t1, dt0, y0_t, a_t, saveat=saveat,
                          stepsize_controller=ctrl, adjoint=adjoint, kernel=kernel)
    (sol.ys * torch.tensor(G, dtype=dtype, device=dev)).sum().backward()
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    low = sol.lowered
    if isinstance(adjoint, dfx.BacksolveAdjoint):
        d = O.make_desc(**O.oracle_fields(low.bwd_fields))
        r = O.backsolve(d, t0, t1, dt0, sol.ts.cpu().numpy(), sol.ys.detach().cpu().double()
                        .numpy(), G, args=args, nthreads=8)
        same = np.all(low.bwd_stats.cpu().numpy() == r["stats"], axis=1)
    else:
        d = O.make_desc(**O.oracle_fields(low.fields))
        r = O.grad_recursive(d, t0, t1, dt0, y0, G, args=args, ts=ts, nthreads=8)
        same = sol.stats["num_steps"].cpu().numpy() == r["stats"][:, 0]
    ga = a_t.grad.double().cpu().numpy()
    if ga.ndim == 2:
        gr = r["grad_args"]
    else:
        # shared args: the batch sum; ra_scale is the sum of the per-trajectory
        # magnitudes, the scale of the sum's rounding
        gr = r["grad_args"].sum(axis=0)
        sol.ra_scale = np.abs(r["grad_args"]).sum(axis=0)
    # same: trajectories whose (backward) step counts equal the oracle's
    return y0_t.grad.double().cpu().numpy(), ga, r["grad_y0"], gr, same, sol


def row_rel(a, b):
    a = np.asarray(a).reshape(a.shape[0], -1)
    b = np.asarray(b).reshape(b.shape[0], -1)
    return np.abs(a - b).max(axis=1) / (np.abs(b).max(axis=1) + 1e-300)


def lv_case(B, seed):
    rng = np.random.default_rng(seed)
    y0 = rng.uniform(5, 15, (B, 2))
    args = np.tile(LV_ARGS, (B, 1)) * rng.uniform(0.8, 1.2, (B, 4))
    return y0, args


@pytest.mark.parametrize("adjoint", [dfx.RecursiveCheckpointAdjoint(), dfx.BacksolveAdjoint()])
@pytest.mark.parametrize("solver", ["tsit5", "dopri5", "heun"])
def test_lotka_volterra_grads_fp64_match_oracle(solver, adjoint):
    # Per-trajectory args, PID(1e-8, 1e-8) (1e-6 for the second-order Heun),
    # saves at 5 times and t1.
    B = 256
    y0, args = lv_case(B, 3)
    ts = np.array([1.0, 4.0, 7.5, 12.0, 19.0])
    saveat = dfx.SaveAt(ts=ts, t1=True)
    G = np.random.default_rng(4).standard_normal((B, 6, 2))
    tol = 1e-6 if solver == "heun" else 1e-8
    gy, ga, ry, ra, same, sol = grad_pair(
        dfx.LotkaVolterra(), SOLVERS[solver], dfx.PIDController(rtol=tol, atol=tol), saveat,
        0.0, 20.0, 0.1, y0, args, torch.float64, adjoint, G)
    e_y, e_a = row_rel(gy, ry), row_rel(ga, ra)
    print(f"LV FP64 {solver} {type(adjoint).__name__}: same steps {same.mean():.3f}, "
          f"dL/dy0 {e_y[same].max():.2e}, dL/dargs {e_a[same].max():.2e} "
          f"(all rows {max(e_y.max(), e_a.max()):.2e})")
    assert same.mean() >= 0.9
    assert e_y[same].max() < 1e-8 and e_a[same].max() < 1e-8
    assert e_y.max() < 1e-4 and e_a.max() < 1e-4


@pytest.mark.parametrize("adjoint", [dfx.RecursiveCheckpointAdjoint(), dfx.BacksolveAdjoint()])
def test_lotka_volterra_grads_fp32(adjoint):
    B = 512
    y0, args = lv_case(B, 5)
    saveat = dfx.SaveAt(ts=np.array([2.0, 9.0]), t1=True)
    G = np.random.default_rng(6).standard_normal((B, 3, 2))
    gy, ga, ry, ra, same, sol = grad_pair(
        dfx.LotkaVolterra(), dfx.Tsit5(), dfx.PIDController(rtol=1e-6, atol=1e-8), saveat,
        0.0, 15.0, 0.1, y0, args, torch.float32, adjoint, G)
    e_y, e_a = row_rel(gy, ry), row_rel(ga, ra)
    print(f"LV FP32 {type(adjoint).__name__}: dL/dy0 median {np.median(e_y):.2e} max "
          f"{e_y.max():.2e}; dL/dargs median {np.median(e_a):.2e} max {e_a.max():.2e}")
    assert np.median(e_y) < 1e-5 and np.median(e_a) < 1e-5
    assert e_y.max() < 1e-3 and e_a.max() < 1e-3


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("solver", ["euler", "heun", "dopri5", "tsit5"])
def test_van_der_pol_shared_args_constant_steps(solver, dtype):
    # Shared mu (summed over the batch), constant steps: both sides
    # differentiate the same step sequence.
    B = 300
    rng = np.random.default_rng(7)
    y0 = rng.uniform(-2, 2, (B, 2))
    args = np.array([1.3])
    G = rng.standard_normal((B, 1, 2))
    gy, ga, ry, ra, same, sol = grad_pair(
        dfx.VanDerPol(), SOLVERS[solver], dfx.ConstantStepSize(), dfx.SaveAt(t1=True), 0.0,
        3.0, 0.01, y0, args, dtype, dfx.RecursiveCheckpointAdjoint(), G)
    assert same.all()
    # FP64: per trajectory; FP32: against the batch's largest gradient (with
    # random cotangents a few trajectories' dL/dy0 nearly cancel, and FP32
    # rounding is then large relative to them)
    e_y = row_rel(gy, ry).max() if dtype == torch.float64 else float(
        np.abs(gy - ry).max() / np.abs(ry).max())
    e_a = float((np.abs(ga - ra) / sol.ra_scale).max())
    print(f"VdP shared mu {solver} {dtype}: dL/dy0 {e_y:.2e}, dL/dmu {e_a:.2e}")
    tol = 1e-10 if dtype == torch.float64 else 2e-5
    assert e_y < tol and e_a < tol


def test_van_der_pol_reverse_time_and_saves():
    # Integration from t0 = 4 back to t1 = 0 with saves on the way (the
    # direction flip of _integrate.py:1157-1176), per-trajectory mu.  In
    # reverse time the limit cycle repels: the states start inside it.
    B = 128
    rng = np.random.default_rng(8)
    y0 = rng.uniform(-1, 1, (B, 2))
    args = np.exp(rng.uniform(np.log(0.3), np.log(3.0), (B, 1)))
    saveat = dfx.SaveAt(ts=np.array([3.5, 2.0, 0.7]), t0=True, t1=True)
    G = rng.standard_normal((B, 5, 2))
    gy, ga, ry, ra, same, sol = grad_pair(
        dfx.VanDerPol(), dfx.Dopri5(), dfx.PIDController(rtol=1e-8, atol=1e-8), saveat, 4.0,
        0.0, None, y0, args, torch.float64, dfx.RecursiveCheckpointAdjoint(), G)
    e_y, e_a = row_rel(gy, ry), row_rel(ga, ra)
    assert same.mean() >= 0.9
    assert e_y[same].max() < 1e-8 and e_a[same].max() < 1e-8


@pytest.mark.parametrize("solver", ["heun", "euler"])
def test_ou_sde_grads_match_oracle_on_the_same_path(solver):
    # dy = theta (mu - y) dt + sigma dW (FP32 state), constant dt 0.01:
    # gradients with respect to y0 and (theta, mu, sigma) on the identical
    # Brownian path.
    B, dim = 512, 2
    rng = np.random.default_rng(9)
    y0 = rng.uniform(-2, 2, (B, dim))
    args = np.array([1.5, 0.5, 0.3])
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (dim,), key=11)
    terms = dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                          dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))
    G = rng.standard_normal((B, 1, dim))
    gy, ga, ry, ra, same, sol = grad_pair(
        None, SOLVERS[solver], dfx.ConstantStepSize(), dfx.SaveAt(t1=True), 0.0, 1.0, 0.01,
        y0, args, torch.float32, dfx.RecursiveCheckpointAdjoint(), G, terms=terms)
    assert same.all()
    e_y = row_rel(gy, ry).max()
    e_a = float((np.abs(ga - ra) / sol.ra_scale).max())
    print(f"OU SDE {solver}: dL/dy0 {e_y:.2e}, dL/d(theta, mu, sigma) {e_a:.2e}")
    assert e_y < 1e-5 and e_a < 1e-4


@pytest.mark.parametrize("adjoint", [dfx.RecursiveCheckpointAdjoint(), dfx.BacksolveAdjoint(),
                                     dfx.BacksolveAdjoint(stepsize_controller=dfx.PIDController(
                                         rtol=1e-9, atol=1e-9, norm=dfx.adjoint_rms_seminorm))])
def test_ou_ode_exact_gradient(adjoint):
    # y' = theta (mu - y): y(t) = mu + (y0 - mu) e^{-theta t}, so for
    # L = sum_i y_i(t1): dL/dy0 = e^{-theta t1}, dL/dmu = dim (1 - e^{-theta t1}),
    # dL/dtheta = -sum_i (y0_i - mu) t1 e^{-theta t1}.  Tight tolerances make
    # both adjoints converge to it.
    B, dim, t1 = 64, 2, 1.7
    rng = np.random.default_rng(10)
    y0 = rng.uniform(-2, 2, (B, dim))
    args = np.column_stack([rng.uniform(0.5, 2.0, B), rng.uniform(-1, 1, B), np.zeros(B)])
    G = np.ones((B, 1, dim))
    gy, ga, _, _, _, sol = grad_pair(
        dfx.OrnsteinUhlenbeck(), dfx.Tsit5(), dfx.PIDController(rtol=1e-9, atol=1e-9),
        dfx.SaveAt(t1=True), 0.0, t1, None, y0, args, torch.float64, adjoint, G)
    th, mu = args[:, 0], args[:, 1]
    e = np.exp(-th * t1)
    gy_ex = np.repeat(e[:, None], dim, axis=1)
    gth_ex = -((y0 - mu[:, None]).sum(axis=1)) * t1 * e
    gmu_ex = dim * (1 - e)
    print(f"OU exact ({adjoint}): dL/dy0 {np.abs(gy - gy_ex).max():.2e}, "
          f"dL/dtheta {np.abs(ga[:, 0] - gth_ex).max():.2e}, "
          f"dL/dmu {np.abs(ga[:, 1] - gmu_ex).max():.2e}")
    assert np.abs(gy - gy_ex).max() < 1e-7
    assert np.abs(ga[:, 0] - gth_ex).max() < 1e-7
    assert np.abs(ga[:, 1] - gmu_ex).max() < 1e-7
    assert np.abs(ga[:, 2]).max() == 0.0  # sigma does not enter an ODE


def test_grads_against_central_differences_of_the_gpu_forward():
    # The recursive adjoint is the exact derivative of the discrete solve:
    # with constant steps it matches central differences (eps 1e-6) of the
    # GPU's own FP64 forward in every argument direction.
    B = 32
    rng = np.random.default_rng(12)
    y0, args = lv_case(B, 13)
    dev = torch.device("cuda")
    term, solver, ctrl = dfx.ODETerm(dfx.LotkaVolterra()), dfx.Tsit5(), dfx.ConstantStepSize()
    saveat = dfx.SaveAt(ts=np.array([3.0, 6.0]), t1=True)
    G = rng.standard_normal((B, 3, 2))
    Gt = torch.tensor(G, device=dev)

    def loss(y0_, a_):
        sol = dfx.diffeqsolve(term, solver, 0.0, 8.0, 0.05, torch.tensor(y0_, device=dev),
                              torch.tensor(a_, device=dev), saveat=saveat,
                              stepsize_controller=ctrl)
        return (sol.ys * Gt).sum(dim=(1, 2)).cpu().numpy()

    y0_t = torch.tensor(y0, device=dev, requires_grad=True)
    a_t = torch.tensor(args, device=dev, requires_grad=True)
    sol = dfx.diffeqsolve(term, solver, 0.0, 8.0, 0.05, y0_t, a_t, saveat=saveat,
                          stepsize_controller=ctrl)
    (sol.ys * Gt).sum().backward()
    ga = a_t.grad.cpu().numpy()
    gy = y0_t.grad.cpu().numpy()
    eps = 1e-6
    worst = 0.0
    for k in range(4):
        dp, dm = args.copy(), args.copy()
        dp[:, k] += eps
        dm[:, k] -= eps
        fd = (loss(y0, dp) - loss(y0, dm)) / (2 * eps)
        worst = max(worst, float(np.abs(fd - ga[:, k]).max() / np.abs(ga[:, k]).max()))
    for k in range(2):
        dp, dm = y0.copy(), y0.copy()
        dp[:, k] += eps
        dm[:, k] -= eps
        fd = (loss(dp, args) - loss(dm, args)) / (2 * eps)
        worst = max(worst, float(np.abs(fd - gy[:, k]).max() / np.abs(gy[:, k]).max()))
    print(f"analytic-field gradients vs central differences: max rel err {worst:.2e}")
    assert worst < 1e-6


def test_backsolve_analytic_failure_raises():
    # BacksolveAdjoint(max_steps=2) cannot cross the saved intervals; the
    # backward raises as the reference's backward diffeqsolve does.
    dev = torch.device("cuda")
    y0 = torch.tensor(np.random.default_rng(14).uniform(5, 15, (8, 2)), device=dev)
    a = torch.tensor(LV_ARGS, device=dev, requires_grad=True)
    sol = dfx.diffeqsolve(dfx.ODETerm(dfx.LotkaVolterra()), dfx.Tsit5(), 0.0, 10.0, 0.1, y0, a,
                          saveat=dfx.SaveAt(ts=np.array([2.0, 5.0, 8.0])),
                          stepsize_controller=dfx.PIDController(rtol=1e-6, atol=1e-8),
                          adjoint=dfx.BacksolveAdjoint(max_steps=2))
    with pytest.raises(RuntimeError, match="maximum number of solver steps"):
        sol.ys.sum().backward()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_uneven_intervals_fused_tape_order(dtype):
    # Per-trajectory t1: the fused forward takes the trajectories longest
    # first and writes their tapes in that order; the backward maps the rows
    # back.  The fused and plain forms take the same steps, so their
    # gradients are identical, and they match the oracle's.
    dev = torch.device("cuda")
    rng = np.random.default_rng(51)
    B = 2048
    y0 = rng.uniform(-2, 2, (B, 2))
    mu = np.exp(rng.uniform(np.log(0.3), np.log(3.0), (B, 1)))
    t1 = rng.uniform(2.0, 12.0, B)
    pid = dfx.PIDController(rtol=1e-7, atol=1e-9)
    grads = []
    for kernel in ("fused", "plain"):
        y0_t = torch.tensor(y0, dtype=dtype, device=dev, requires_grad=True)
        mu_t = torch.tensor(mu, dtype=dtype, device=dev, requires_grad=True)
        sol = dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(), 0.0,
                              torch.tensor(t1, dtype=torch.float64, device=dev), None, y0_t,
                              mu_t, stepsize_controller=pid, kernel=kernel)
        sol.ys.square().sum().backward()
        grads.append((y0_t.grad, mu_t.grad, sol))
    assert torch.equal(grads[0][0], grads[1][0]) and torch.equal(grads[0][1], grads[1][1])
    sol = grads[0][2]
    n = 256
    d = O.make_desc(**O.oracle_fields(sol.lowered.fields))
    G = 2.0 * sol.ys[:n].detach().double().cpu().numpy()
    r = O.grad_recursive(d, 0.0, t1[:n], None, y0[:n], G, args=mu[:n], nthreads=8)
    gy = grads[0][0][:n].double().cpu().numpy()
    e = np.abs(gy - r["grad_y0"]).max(axis=1) / np.abs(r["grad_y0"]).max()
    tol = 1e-8 if dtype == torch.float64 else 2e-3
    # (a trajectory whose accept/reject sequence is ulp-sensitive may take
    # another step sequence than the oracle's)
    assert (e <= tol).mean() >= 0.95 and e.max() < 1e-2
