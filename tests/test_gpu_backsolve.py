"""GPU BacksolveAdjoint gradients against the FP64 oracle's backsolve
(diffrax/_adjoint.py:572-734) run from the same saved forward states.

Both sides solve the augmented adjoint system (y, a, a_theta) backwards
between the saved times with the same solver and controller, so the FP32
parity mode must take the same steps and agree to FP32 accuracy; the BF16
tensor-core mode is checked for its error level.  The neural-ODE shape of the
benchmark (64-256-256-64, 32 saved times, loss = sum of mean squares) is also
checked against central finite differences of the FP64 forward solve.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu


def bf16_round(a):
    t = torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).to(torch.float64)
    return t.numpy()


def mlp_params(widths, seed, bias_scale=0.1, bf16_weights=False):
    rng = np.random.default_rng(seed)
    Ws, bs = [], []
    for i in range(len(widths) - 1):
        W = (rng.standard_normal((widths[i + 1], widths[i])) / np.sqrt(widths[i]))
        W = W.astype(np.float32).astype(np.float64)
        Ws.append(bf16_round(W) if bf16_weights else W)
        bs.append((rng.standard_normal(widths[i + 1]) * bias_scale)
                  .astype(np.float32).astype(np.float64))
    return Ws, bs


def backsolve_case(widths, solver, controller, ts, B, precision, seed=0, seminorm=False,
                   t1=1.0, dt0=None, bf16_weights=True, grad_ys=None, y0=None, kernel="fused"):
    """The model's weights are BF16 values (bf16_weights); the FP32 modes and
    the oracle see the same values."""
    dev = torch.device("cuda")
    rng = np.random.default_rng(seed + 100)
    D = widths[0]
    if y0 is None:
        y0 = rng.standard_normal((B, D))
    y0 = np.asarray(y0).astype(np.float32).astype(np.float64)
    Ws, bs = mlp_params(widths, seed, bf16_weights=bf16_weights)
    tW = [torch.tensor(W, dtype=torch.float32, device=dev, requires_grad=True) for W in Ws]
    tb = [torch.tensor(b, dtype=torch.float32, device=dev, requires_grad=True) for b in bs]
    field = dfx.MLPField(tW, tb, precision=precision)
    if seminorm:
        c = controller
        bwd_ctrl = dfx.PIDController(rtol=c.rtol, atol=c.atol, norm=dfx.adjoint_rms_seminorm)
        adjoint = dfx.BacksolveAdjoint(stepsize_controller=bwd_ctrl)
    else:
        adjoint = dfx.BacksolveAdjoint()
    y0_t = torch.tensor(y0, dtype=torch.float32, device=dev, requires_grad=True)
    sol = dfx.diffeqsolve(dfx.ODETerm(field), solver, 0.0, t1, dt0, y0_t,
                          saveat=dfx.SaveAt(ts=ts), stepsize_controller=controller,
                          adjoint=adjoint, kernel=kernel)
    ys = sol.ys.double()
    G = grad_ys(ys.detach().cpu().numpy()) if grad_ys else rng.standard_normal(ys.shape)
    loss = (ys * torch.tensor(G, device=dev)).sum()
    loss.backward()
    torch.cuda.synchronize()
    low = sol.lowered
    g_params = torch.cat([t.grad.reshape(-1) for pair in zip(tW, tb) for t in pair])
    params = np.concatenate([np.concatenate([W.reshape(-1), b]) for W, b in zip(Ws, bs)])
    d = O.make_desc(**O.oracle_fields(low.bwd_fields))
    r = O.backsolve(d, 0.0, t1, dt0, sol.ts.cpu().numpy(), ys.detach().cpu().numpy(), G,
                    params=params, nthreads=8)
    return dict(g_y0=y0_t.grad.double().cpu().numpy(),
                g_params=g_params.double().cpu().numpy(), oracle=r,
                stats=low.bwd_stats.cpu().numpy(), result=low.bwd_result.cpu().numpy(),
                params=params, y0=y0, G=G, sol=sol)


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def check_steps(c, exact, n_seg, slack=1):
    """Dopri5 and Heun take the FP64 oracle's steps.  Tsit5's error weights
    (sum |e_j| ~ 1.2, against ~0.1 for Dopri5) give its FP32 error estimate a
    noise floor, so after a segment restarts at dt = 0.01 the FP32 controller
    grows dt by less than the 10x cap: at most one extra step per segment."""
    gs, os_ = c["stats"], c["oracle"]["stats"]
    bad = np.nonzero(np.any(gs != os_, axis=1))[0][:4]
    print("steps (gpu, oracle) of differing rows:", [(gs[i].tolist(), os_[i].tolist())
                                                     for i in bad])
    if exact:
        assert np.mean(np.all(gs == os_, axis=1)) >= 0.9
    else:
        assert np.all(gs[:, 0] >= os_[:, 0] - 1)
        assert np.all(gs[:, 0] <= os_[:, 0] + n_seg * slack)


PID = dfx.PIDController(rtol=1e-5, atol=1e-7)
TS6 = np.linspace(0.0, 1.0, 6)


@pytest.mark.parametrize("solver", [dfx.Tsit5(), dfx.Dopri5(), dfx.Heun()])
def test_backsolve_fp32_pid_matches_oracle(solver):
    c = backsolve_case([32, 64, 64, 32], solver, PID, TS6, 40, "fp32", seed=1)
    r = c["oracle"]
    same = np.all(c["stats"] == r["stats"], axis=1)
    e0, ep = rel(c["g_y0"], r["grad_y0"]), rel(c["g_params"], r["grad_params"])
    print(f"backsolve {solver} fp32: same steps {same.mean():.2f}, dL/dy0 {e0:.2e}, "
          f"dL/dtheta {ep:.2e}, steps {c['stats'][:, 0].mean():.1f}")
    assert np.all(c["result"] == 0) and np.all(r["result"] == 0)
    check_steps(c, not isinstance(solver, dfx.Tsit5), 5)
    assert e0 < 1e-4 and ep < 1e-4


@pytest.mark.parametrize("solver", [dfx.Euler(), dfx.Heun(), dfx.Tsit5()])
def test_backsolve_fp32_constant_steps(solver):
    # ConstantStepSize: the backward's carried controller state extends the
    # first segment's grid into later segments, as in the reference.
    c = backsolve_case([32, 64, 64, 32], solver, dfx.ConstantStepSize(),
                       np.array([0.3, 0.55, 1.0]), 36, "fp32", seed=2, dt0=0.04)
    r = c["oracle"]
    assert np.array_equal(c["stats"], r["stats"])
    e0, ep = rel(c["g_y0"], r["grad_y0"]), rel(c["g_params"], r["grad_params"])
    print(f"backsolve constant {solver}: dL/dy0 {e0:.2e}, dL/dtheta {ep:.2e}")
    assert e0 < 1e-4 and ep < 1e-4


@pytest.mark.parametrize("solver", [dfx.Dopri5(), dfx.Tsit5()])
def test_backsolve_fp32_seminorm(solver):
    c = backsolve_case([32, 64, 64, 32], solver, PID, TS6, 40, "fp32", seed=3,
                       seminorm=True)
    r = c["oracle"]
    same = np.all(c["stats"] == r["stats"], axis=1)
    e0, ep = rel(c["g_y0"], r["grad_y0"]), rel(c["g_params"], r["grad_params"])
    print(f"backsolve seminorm {solver} fp32: same steps {same.mean():.2f}, dL/dy0 {e0:.2e}, "
          f"dL/dtheta {ep:.2e}")
    check_steps(c, isinstance(solver, dfx.Dopri5), 5)
    assert e0 < 1e-4 and ep < 1e-4


def test_backsolve_uneven_saves_and_t0_save():
    # Saves that coincide with t0 and with each other give empty segments.
    ts = np.array([0.0, 0.0, 0.4, 0.4, 0.9, 1.0])
    c = backsolve_case([32, 64, 64, 32], dfx.Dopri5(), PID, ts, 24, "fp32", seed=4)
    r = c["oracle"]
    # long segments: the FP32 noise floor of the error estimate limits dt growth
    check_steps(c, False, 3)
    assert rel(c["g_y0"], r["grad_y0"]) < 1e-4
    assert rel(c["g_params"], r["grad_params"]) < 1e-4


@pytest.mark.parametrize("widths", [[32, 64, 64, 32], [64, 128, 128, 64]])
def test_backsolve_bf16_error_level(widths):
    c = backsolve_case(widths, dfx.Tsit5(), PID, TS6, 48, "bf16", seed=5)
    r = c["oracle"]
    same = np.all(c["stats"] == r["stats"], axis=1)
    e0, ep = rel(c["g_y0"], r["grad_y0"]), rel(c["g_params"], r["grad_params"])
    print(f"backsolve bf16 {widths}: same steps {same.mean():.2f}, dL/dy0 {e0:.2e}, "
          f"dL/dtheta {ep:.2e}")
    # hi/lo BF16 products put the noise floor of the Tsit5 error estimate higher
    check_steps(c, False, 5, slack=5)
    assert e0 < 1e-3 and ep < 1e-3


def _c4_grad_ys(ys):
    # loss = sum over the saved points of mean(y^2) over batch and state
    B, _, D = ys.shape
    return 2.0 * ys / (B * D)


@pytest.mark.parametrize("seminorm", [False, True])
def test_backsolve_neural_ode_wide(seminorm):
    # 64-256-256-64 with BF16 weights (the oracle gets the same BF16 values),
    # 32 saved times on [0, 1], Tsit5 + PID(1e-5, 1e-7).
    ts = np.linspace(0.0, 1.0, 32)
    c = backsolve_case([64, 256, 256, 64], dfx.Tsit5(), PID, ts, 24, "bf16", seed=6,
                       seminorm=seminorm, bf16_weights=True, grad_ys=_c4_grad_ys)
    r = c["oracle"]
    same = np.all(c["stats"] == r["stats"], axis=1)
    e0, ep = rel(c["g_y0"], r["grad_y0"]), rel(c["g_params"], r["grad_params"])
    print(f"backsolve 64-256-256-64 (seminorm={seminorm}): same steps {same.mean():.2f}, "
          f"dL/dy0 {e0:.2e}, dL/dtheta {ep:.2e}, bwd steps {c['stats'][:, 0].mean():.1f}")
    # under rms_norm the a_theta components dominate the norm and every
    # segment takes the FP64 oracle's two steps
    check_steps(c, not seminorm, 31)
    assert e0 < 1e-3 and ep < 1e-3


def test_backsolve_neural_ode_wide_fp32():
    ts = np.linspace(0.0, 1.0, 8)
    c = backsolve_case([64, 256, 256, 64], dfx.Tsit5(), PID, ts, 16, "fp32", seed=7)
    r = c["oracle"]
    check_steps(c, False, 7)
    assert rel(c["g_y0"], r["grad_y0"]) < 1e-4
    assert rel(c["g_params"], r["grad_params"]) < 1e-4


def test_backsolve_neural_ode_wide_finite_differences():
    # Central differences (eps = 1e-4) of the FP64 forward loss on 16 random
    # parameter directions against the GPU backsolve gradient.
    ts = np.linspace(0.0, 1.0, 32)
    widths = [64, 256, 256, 64]
    c = backsolve_case(widths, dfx.Tsit5(), PID, ts, 16, "bf16", seed=8, bf16_weights=True,
                       grad_ys=_c4_grad_ys)
    d = O.make_desc(**O.oracle_fields(c["sol"].lowered.fields))
    y0, P = c["y0"], c["params"]
    B, D = y0.shape

    def loss(p):
        f = O.solve(d, 0.0, 1.0, None, y0, params=p, ts=ts, nthreads=8)
        return float(np.sum(f["ys"] ** 2) / (B * D))

    rng = np.random.default_rng(9)
    eps = 1e-4
    errs = []
    for _ in range(16):
        v = rng.standard_normal(P.size)
        v /= np.linalg.norm(v)
        fd = (loss(P + eps * v) - loss(P - eps * v)) / (2 * eps)
        # relative to the directional derivative itself (|g.v| is ~|g|/sqrt(P))
        errs.append(abs(fd - c["g_params"] @ v) / abs(fd))
    print(f"backsolve vs central differences: per-direction rel err "
          f"{' '.join(f'{e:.1e}' for e in errs)}")
    assert max(errs) < 2e-3


def test_backsolve_plain_kernel():
    # The plain form (one trajectory per thread, FP32 CUDA-core products) of
    # the wide neural ODE's backsolve, against the FP64 oracle.
    ts = np.linspace(0.0, 1.0, 8)
    c = backsolve_case([64, 256, 256, 64], dfx.Tsit5(), PID, ts, 12, "fp32", seed=13,
                       grad_ys=_c4_grad_ys, kernel="plain")
    r = c["oracle"]
    e0, ep = rel(c["g_y0"], r["grad_y0"]), rel(c["g_params"], r["grad_params"])
    print(f"plain backsolve: dL/dy0 {e0:.2e}, dL/dtheta {ep:.2e}, "
          f"steps {c['stats'][:, 0].mean():.1f} (oracle {r['stats'][:, 0].mean():.1f})")
    assert np.all(c["result"] == 0)
    check_steps(c, False, 7)
    assert e0 < 1e-4 and ep < 1e-4


@pytest.mark.parametrize("throw", [True, False])
def test_backsolve_backward_failure(throw):
    # The reverse solve of BacksolveAdjoint(max_steps=2) cannot cross five
    # saved intervals.  With throw=True the backward raises, as the
    # reference's backward diffeqsolve does (diffrax/_adjoint.py:623-634);
    # with throw=False it returns and records max_steps_reached per trajectory.
    dev = torch.device("cuda")
    widths = [32, 64, 64, 32]
    Ws, bs = mlp_params(widths, 3)
    tW = [torch.tensor(W, dtype=torch.float32, device=dev, requires_grad=True) for W in Ws]
    tb = [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs]
    y0 = torch.tensor(np.random.default_rng(4).standard_normal((8, 32)), dtype=torch.float32,
                      device=dev)
    sol = dfx.diffeqsolve(dfx.ODETerm(dfx.MLPField(tW, tb)), dfx.Tsit5(), 0.0, 1.0, None, y0,
                          saveat=dfx.SaveAt(ts=TS6), stepsize_controller=PID,
                          adjoint=dfx.BacksolveAdjoint(max_steps=2, throw=throw))
    assert bool((sol.result == 0).all())
    loss = (sol.ys ** 2).sum()
    if throw:
        with pytest.raises(RuntimeError, match="maximum number of solver steps"):
            loss.backward()
    else:
        loss.backward()
        assert bool((sol.lowered.bwd_result == int(dfx.RESULTS.max_steps_reached)).all())
