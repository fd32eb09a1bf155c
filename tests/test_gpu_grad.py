"""GPU RecursiveCheckpointAdjoint gradients against the FP64 oracle's
discretise-then-optimise VJP (diffrax/_adjoint.py:179-312) on the same inputs.

With constant steps both sides differentiate the same step sequence, so the
FP32 parity mode must agree to FP32 accuracy; the BF16 tensor-core mode is
checked for its error level.  Checkpoint thinning (fewer slots than steps)
exercises the segment recomputation.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu


def bf16_round(a):
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).double().numpy()


def params_np(widths, seed, bias_scale=0.1):
    """BF16-valued weight matrices (the model's BF16 weights), FP32 biases."""
    rng = np.random.default_rng(seed)
    Ws, bs = [], []
    for i in range(len(widths) - 1):
        Ws.append(bf16_round(rng.standard_normal((widths[i + 1], widths[i]))
                             / np.sqrt(widths[i])))
        bs.append((rng.standard_normal(widths[i + 1]) * bias_scale)
                  .astype(np.float32).astype(np.float64))
    return Ws, bs


def grad_case(widths, solver, controller, saveat, t1, dt0, B, precision, checkpoints,
              seed=0, sde=False, max_steps=4096, kernel="fused"):
    dev = torch.device("cuda")
    rng = np.random.default_rng(seed + 100)
    D = widths[0]
    y0 = rng.standard_normal((B, D)).astype(np.float32).astype(np.float64)
    Ws, bs = params_np(widths, seed)
    tW = [torch.tensor(W, dtype=torch.float32, device=dev, requires_grad=True) for W in Ws]
    tb = [torch.tensor(b, dtype=torch.float32, device=dev, requires_grad=True) for b in bs]
    field = dfx.MLPField(tW, tb, precision=precision)
    flat = [np.concatenate([W.reshape(-1), b]) for W, b in zip(Ws, bs)]
    extra = []
    if sde:
        Wsig = bf16_round(rng.standard_normal((D, D)) / np.sqrt(D))
        bsig = (rng.standard_normal(D) * 0.1).astype(np.float32).astype(np.float64)
        tWs = torch.tensor(Wsig, dtype=torch.float32, device=dev, requires_grad=True)
        tbs = torch.tensor(bsig, dtype=torch.float32, device=dev, requires_grad=True)
        bm = dfx.VirtualBrownianTree(0.0, float(np.max(t1)), 1e-3, (D,), key=seed + 7)
        terms = dfx.MultiTerm(dfx.ODETerm(field), dfx.ControlTerm(
            dfx.TanhDiagonalDiffusion(tWs, tbs), bm))
        flat += [Wsig.reshape(-1), bsig]
        extra = [tWs, tbs]
    else:
        terms = dfx.ODETerm(field)
    params = np.concatenate(flat)
    y0_t = torch.tensor(y0, dtype=torch.float32, device=dev, requires_grad=True)
    t1_arg = torch.tensor(t1, dtype=torch.float64, device=dev) if isinstance(
        t1, np.ndarray) else t1
    sol = dfx.diffeqsolve(terms, solver, 0.0, t1_arg, dt0, y0_t, saveat=saveat,
                          stepsize_controller=controller, max_steps=max_steps,
                          adjoint=dfx.RecursiveCheckpointAdjoint(checkpoints=checkpoints),
                          kernel=kernel)
    n_save = sol.ys.shape[1]
    G = rng.standard_normal((B, n_save, D))
    loss = (sol.ys.double() * torch.tensor(G, device=dev)).sum()
    loss.backward()
    torch.cuda.synchronize()
    g_params = torch.cat([t.grad.reshape(-1) for pair in zip(tW, tb) for t in pair] +
                         [t.grad.reshape(-1) for t in extra]).double().cpu().numpy()
    g_y0 = y0_t.grad.double().cpu().numpy()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(terms, solver, controller, saveat, dim=D, dtype=torch.float32,
                       max_steps=max_steps, n_ts=0 if ts is None else ts.size)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.grad_recursive(d, 0.0, t1, dt0, y0, G, params=params, ts=ts, nthreads=8)
    steps = sol.stats["num_steps"].cpu().numpy()
    return g_y0, g_params, r, steps


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("solver", [dfx.Tsit5(), dfx.Dopri5(), dfx.Heun(), dfx.Euler()])
def test_grad_constant_steps_fp32(solver):
    ts = np.array([0.3, 0.55, 1.0])
    g_y0, g_p, r, steps = grad_case([64, 128, 128, 64], solver, dfx.ConstantStepSize(),
                                    dfx.SaveAt(ts=ts, t1=True), 1.0, 0.05, 70, "fp32",
                                    checkpoints=64, seed=1)
    assert np.array_equal(steps, r["stats"][:, 0])
    e0, ep = rel(g_y0, r["grad_y0"]), rel(g_p, r["grad_params"])
    print(f"grad {solver} constant fp32: dL/dy0 rel {e0:.2e}, dL/dtheta rel {ep:.2e}")
    assert e0 < 1e-4 and ep < 1e-4


@pytest.mark.parametrize("checkpoints", [2, 5, 16])
def test_grad_checkpoint_thinning_fp32(checkpoints):
    # 60 steps with few checkpoint slots: strides 32, 16, 8 and segment recompute.
    g_y0, g_p, r, steps = grad_case([32, 64, 64, 32], dfx.Tsit5(), dfx.ConstantStepSize(),
                                    dfx.SaveAt(t1=True, ts=np.array([0.5])), 1.2, 0.02, 40,
                                    "fp32", checkpoints=checkpoints, seed=2)
    assert steps.max() == 60
    e0, ep = rel(g_y0, r["grad_y0"]), rel(g_p, r["grad_params"])
    print(f"grad thinning C={checkpoints}: dL/dy0 rel {e0:.2e}, dL/dtheta rel {ep:.2e}")
    assert e0 < 1e-4 and ep < 1e-4


def test_grad_pid_coarse_fp32():
    # PID at a coarse tolerance: the FP32 and FP64 controllers take the same
    # number of steps, but their step sizes differ at the tolerance level, and
    # so do the gradients of the two discrete maps.
    g_y0, g_p, r, steps = grad_case([64, 128, 128, 64], dfx.Tsit5(),
                                    dfx.PIDController(rtol=1e-3, atol=1e-4),
                                    dfx.SaveAt(t1=True), 2.0, None, 64, "fp32",
                                    checkpoints=64, seed=3)
    same = steps == r["stats"][:, 0]
    assert same.mean() > 0.9
    rows = np.abs(g_y0 - r["grad_y0"]).max(axis=1) / np.abs(r["grad_y0"]).max()
    print(f"grad PID fp32: identical steps {same.mean():.2f}, dL/dy0 rel (same steps) "
          f"{rows[same].max():.2e}")
    assert rows[same].max() < 1e-2


def test_grad_uneven_t1_fp32():
    t1 = np.random.default_rng(9).uniform(0.3, 1.5, 90)
    g_y0, g_p, r, steps = grad_case([64, 128, 128, 64], dfx.Dopri5(), dfx.ConstantStepSize(),
                                    dfx.SaveAt(t1=True), t1, 0.05, 90, "fp32", checkpoints=8,
                                    seed=4)
    e0, ep = rel(g_y0, r["grad_y0"]), rel(g_p, r["grad_params"])
    assert e0 < 1e-4 and ep < 1e-4


@pytest.mark.parametrize("solver", [dfx.Heun(), dfx.Euler()])
def test_grad_neural_sde_fp32(solver):
    # Neural SDE shape: drift 32-64-64-32, diffusion 0.1 tanh(W y + b), dt = 0.01.
    g_y0, g_p, r, steps = grad_case([32, 64, 64, 32], solver, dfx.ConstantStepSize(),
                                    dfx.SaveAt(t1=True), 1.0, 0.01, 48, "fp32",
                                    checkpoints=12, seed=5, sde=True)
    e0, ep = rel(g_y0, r["grad_y0"]), rel(g_p, r["grad_params"])
    print(f"grad SDE {solver} fp32: dL/dy0 rel {e0:.2e}, dL/dtheta rel {ep:.2e}")
    assert e0 < 1e-4 and ep < 1e-4


@pytest.mark.parametrize("widths,sde", [([64, 128, 128, 64], False), ([32, 64, 64, 32], True)])
def test_grad_bf16_error_level(widths, sde):
    dt0 = 0.01 if sde else 0.05
    solver = dfx.Heun() if sde else dfx.Tsit5()
    g_y0, g_p, r, steps = grad_case(widths, solver, dfx.ConstantStepSize(), dfx.SaveAt(t1=True),
                                    1.0, dt0, 128, "bf16", checkpoints=64, seed=6, sde=sde)
    e0, ep = rel(g_y0, r["grad_y0"]), rel(g_p, r["grad_params"])
    print(f"grad bf16 {widths}: dL/dy0 rel {e0:.2e}, dL/dtheta rel {ep:.2e}")
    # BF16 weights and three-piece BF16 activations and cotangents: the
    # products are exact up to FP32 accumulation
    assert e0 < 1e-4 and ep < 1e-4


@pytest.mark.parametrize("sde", [False, True])
def test_grad_plain_kernel(sde):
    # The plain form (one trajectory per thread, FP32 CUDA-core products, full
    # tape): the neural ODE 64-128-128-64 with Tsit5 + PID and the neural SDE
    # 32-64-64-32 with Heun, against the FP64 oracle.
    if sde:
        g_y0, g_p, r, steps = grad_case([32, 64, 64, 32], dfx.Heun(), dfx.ConstantStepSize(),
                                        dfx.SaveAt(t1=True), 1.0, 0.01, 40, "fp32",
                                        checkpoints=16, seed=11, sde=True, kernel="plain")
    else:
        g_y0, g_p, r, steps = grad_case([64, 128, 128, 64], dfx.Tsit5(), dfx.ConstantStepSize(),
                                        dfx.SaveAt(t1=True, ts=np.array([0.4, 0.7])), 1.0, 0.05,
                                        40, "fp32", checkpoints=64, seed=12, kernel="plain")
    assert np.array_equal(steps, r["stats"][:, 0])
    e0, ep = rel(g_y0, r["grad_y0"]), rel(g_p, r["grad_params"])
    print(f"plain backward (sde={sde}): dL/dy0 rel {e0:.2e}, dL/dtheta rel {ep:.2e}")
    assert e0 < 1e-4 and ep < 1e-4


def _loss_grad_case(widths, solver, controller, dt0, B, checkpoints, sde, seed, kernel,
                    precision):
    """dL/dy0 and dL/dtheta of loss = mean(y(t1)^2) through diffeqsolve and
    backward(), against the FP64 oracle's gradient of the same loss (its
    cotangent from its own forward)."""
    dev = torch.device("cuda")
    rng = np.random.default_rng(seed + 100)
    D = widths[0]
    y0 = rng.standard_normal((B, D)).astype(np.float32).astype(np.float64)
    Ws, bs = params_np(widths, seed, bias_scale=0.0)
    tW = [torch.tensor(W, dtype=torch.float32, device=dev, requires_grad=True) for W in Ws]
    tb = [torch.tensor(b, dtype=torch.float32, device=dev, requires_grad=True) for b in bs]
    field = dfx.MLPField(tW, tb, precision=precision)
    flat = [np.concatenate([W.reshape(-1), b]) for W, b in zip(Ws, bs)]
    extra = []
    if sde:
        Wsig = bf16_round(rng.standard_normal((D, D)) / np.sqrt(D))
        bsig = np.zeros(D)
        tWs = torch.tensor(Wsig, dtype=torch.float32, device=dev, requires_grad=True)
        tbs = torch.tensor(bsig, dtype=torch.float32, device=dev, requires_grad=True)
        bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (D,), key=seed + 7)
        terms = dfx.MultiTerm(dfx.ODETerm(field), dfx.ControlTerm(
            dfx.TanhDiagonalDiffusion(tWs, tbs), bm))
        flat += [Wsig.reshape(-1), bsig]
        extra = [tWs, tbs]
    else:
        terms = dfx.ODETerm(field)
    params = np.concatenate(flat)
    y0_t = torch.tensor(y0, dtype=torch.float32, device=dev, requires_grad=True)
    sol = dfx.diffeqsolve(terms, solver, 0.0, 1.0, dt0, y0_t, stepsize_controller=controller,
                          adjoint=dfx.RecursiveCheckpointAdjoint(checkpoints=checkpoints),
                          kernel=kernel)
    loss = (sol.ys ** 2).mean()
    loss.backward()
    torch.cuda.synchronize()
    g_params = torch.cat([t.grad.reshape(-1) for pair in zip(tW, tb) for t in pair] +
                         [t.grad.reshape(-1) for t in extra]).double().cpu().numpy()
    fields = dfx.lower(terms, solver, controller, dfx.SaveAt(t1=True), dim=D,
                       dtype=torch.float32, max_steps=4096, n_ts=0)
    d = O.make_desc(**O.oracle_fields(fields))
    ref = O.solve(d, 0.0, 1.0, dt0, y0, params=params, nthreads=8)
    G = 2.0 * ref["ys"] / ref["ys"].size
    r = O.grad_recursive(d, 0.0, 1.0, dt0, y0, G, params=params, nthreads=8)
    g_y0 = y0_t.grad.double().cpu().numpy()
    e0 = float((np.abs(g_y0 - r["grad_y0"]).max(axis=1)
                / np.abs(r["grad_y0"]).max(axis=1)).max())
    return e0, rel(g_params, r["grad_params"])


@pytest.mark.parametrize("sde", [False, True])
def test_grad_product_precision_matches_plain_error(sde):
    # The gradient workloads as specified, at a reduced batch: the neural ODE
    # 64-128-128-64 with Tsit5 + PID(1e-5, 1e-7) and RecursiveCheckpointAdjoint(64),
    # and the neural SDE 32-64-64-32 (diffusion 0.1 tanh(W y + b)) with Heun,
    # dt 0.01, VBT tol 1e-3 and the default checkpoints.  The BF16 tensor-core
    # form must be as accurate against the FP64 oracle as the plain FP32 form
    # on the same inputs (within 2x: both solve in FP32 state and their FP32
    # controllers take the same steps, which differ from the FP64 oracle's).
    if sde:
        args = ([32, 64, 64, 32], dfx.Heun(), dfx.ConstantStepSize(), 0.01, 128, None, True, 31)
    else:
        args = ([64, 128, 128, 64], dfx.Tsit5(), dfx.PIDController(rtol=1e-5, atol=1e-7), None,
                128, 64, False, 32)
    f0, fp = _loss_grad_case(*args, kernel="fused", precision="bf16")
    p0, pp = _loss_grad_case(*args, kernel="plain", precision="fp32")
    print(f"product-precision gradients (sde={sde}): fused BF16 dL/dy0 {f0:.2e} "
          f"dL/dtheta {fp:.2e}; plain FP32 dL/dy0 {p0:.2e} dL/dtheta {pp:.2e}")
    assert f0 <= 2 * p0 + 1e-6 and fp <= 2 * pp + 1e-6
