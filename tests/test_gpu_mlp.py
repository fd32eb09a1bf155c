"""GPU parity of the MLP-field row-tile integrator against the FP64 oracle.

The FP32 parity mode (FP32 products) must match the oracle to FP32-state
accuracy; the BF16 tensor-core mode is checked for its expected error level
(BF16 operands carry 8 significant bits).  SDE runs feed the oracle the same
counter-based Brownian path the kernel draws.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu


def bf16_round(a):
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).double().numpy()


def mlp_params(widths, seed, bias_scale=0.0):
    """W ~ N(0, 1/fan_in) as BF16 values (the neural-ODE configs' BF16
    weights), biases zero (or small) in FP32."""
    rng = np.random.default_rng(seed)
    Ws, bs = [], []
    for i in range(len(widths) - 1):
        Ws.append(bf16_round(rng.standard_normal((widths[i + 1], widths[i])) / np.sqrt(widths[i])))
        bs.append(rng.standard_normal(widths[i + 1]) * bias_scale)
    return Ws, bs


def flat(Ws, bs):
    return np.concatenate([np.concatenate([W.reshape(-1), b]) for W, b in zip(Ws, bs)])


def run_mlp(widths, solver, controller, saveat, t0, t1, dt0, y0, precision, seed=0,
            diffusion=None, bm=None, max_steps=4096, bias_scale=0.0):
    """The GPU solve and the FP64 oracle's on the same inputs."""
    dev = torch.device("cuda")
    Ws, bs = mlp_params(widths, seed, bias_scale)
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
    tt = lambda x: torch.tensor(x, dtype=torch.float64, device=dev) if isinstance(  # noqa
        x, np.ndarray) else x
    sol = dfx.diffeqsolve(terms, solver, tt(t0), tt(t1), dt0,
                          torch.tensor(y0, dtype=torch.float32, device=dev),
                          saveat=saveat, stepsize_controller=controller,
                          max_steps=max_steps, throw=False)
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(terms, solver, controller, saveat, dim=y0.shape[1],
                       dtype=torch.float32, max_steps=max_steps,
                       n_ts=0 if ts is None else ts.size)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, t0, t1, dt0, y0, params=params, ts=ts, nthreads=8)
    return sol, r


def per_traj_err(sol, r):
    ys = sol.ys.cpu().double().numpy()
    assert np.array_equal(np.isfinite(ys), np.isfinite(r["ys"]))
    fin = np.isfinite(r["ys"])
    a = np.where(fin, ys, 0)
    b = np.where(fin, r["ys"], 0)
    return np.abs(a - b).max(axis=(1, 2)) / np.abs(b).max(axis=(1, 2))


@pytest.mark.parametrize("solver", [dfx.Tsit5(), dfx.Dopri5()])
def test_mlp_64_128_fp32_matches_oracle(solver):
    # Neural-ODE shape 64 -> 128 -> 128 -> 64, Tsit5/Dopri5 + PID(1e-5, 1e-7), t in [0, 1].
    rng = np.random.default_rng(10)
    y0 = rng.standard_normal((100, 64))
    ts = np.linspace(0.0, 1.0, 9)
    sol, r = run_mlp([64, 128, 128, 64], solver, dfx.PIDController(rtol=1e-5, atol=1e-7),
                     dfx.SaveAt(ts=ts, t1=True), 0.0, 1.0, None, y0, "fp32", seed=1,
                     bias_scale=0.1)
    assert (sol.result == 0).all()
    err = per_traj_err(sol, r)
    steps = sol.stats["num_steps"].cpu().numpy()
    print(f"MLP 64-128 fp32 {solver}: max rel err {err.max():.2e}, steps {steps.mean():.1f} "
          f"(oracle {r['stats'][:, 0].mean():.1f})")
    assert err.max() < 2e-5
    # With atol 1e-7 the FP32 rounding of the embedded error estimate is of the
    # order of the tolerance for small components, so the FP32 controller may
    # take a few more steps than the FP64 one.
    assert steps.mean() < 1.6 * r["stats"][:, 0].mean()


@pytest.mark.parametrize("solver", [dfx.Tsit5(), dfx.Dopri5()])
def test_mlp_fp32_controller_matches_oracle_step_for_step(solver):
    # At a tolerance well above FP32 rounding the PID decisions are identical.
    rng = np.random.default_rng(19)
    y0 = rng.standard_normal((100, 64))
    sol, r = run_mlp([64, 128, 128, 64], solver, dfx.PIDController(rtol=1e-3, atol=1e-4),
                     dfx.SaveAt(t1=True), 0.0, 3.0, None, y0, "fp32", seed=1, bias_scale=0.1)
    steps = sol.stats["num_steps"].cpu().numpy()
    same = steps == r["stats"][:, 0]
    err = per_traj_err(sol, r)
    print(f"controller parity {solver}: {same.mean():.3f} identical step counts")
    assert same.mean() > 0.95
    # Equal step counts, but the FP32 controller's step sizes differ from the
    # FP64 ones at the tolerance level, and so do the solutions.
    assert err.max() < 1e-2


def test_mlp_64_256_fp32_saveat_ts_matches_oracle():
    # Backsolve-config shape 64 -> 256 -> 256 -> 64 with 32 save points.
    rng = np.random.default_rng(11)
    y0 = rng.standard_normal((40, 64))
    ts = np.linspace(0.0, 1.0, 32)
    sol, r = run_mlp([64, 256, 256, 64], dfx.Tsit5(), dfx.PIDController(rtol=1e-5, atol=1e-7),
                     dfx.SaveAt(ts=ts), 0.0, 1.0, None, y0, "fp32", seed=2)
    err = per_traj_err(sol, r)
    print(f"MLP 64-256 fp32: max rel err {err.max():.2e}")
    assert err.max() < 2e-5
    assert np.array_equal(sol.ts.cpu().numpy(), r["ts"])


@pytest.mark.parametrize("solver", [dfx.Euler(), dfx.Heun()])
def test_mlp_constant_step_fp32(solver):
    rng = np.random.default_rng(12)
    y0 = rng.standard_normal((70, 32))
    sol, r = run_mlp([32, 64, 64, 32], solver, dfx.ConstantStepSize(),
                     dfx.SaveAt(t1=True, t0=True), 0.0, 1.0, 0.02, y0, "fp32", seed=3)
    err = per_traj_err(sol, r)
    assert err.max() < 1e-5
    assert np.array_equal(sol.stats["num_steps"].cpu().numpy(), r["stats"][:, 0])


def test_mlp_uneven_t1_row_refill():
    # Per-trajectory t1 and a batch that is not a multiple of the row tile:
    # rows finish at different steps and are refilled from the queue.
    rng = np.random.default_rng(13)
    B = 333
    y0 = rng.standard_normal((B, 64))
    t1 = rng.uniform(0.1, 2.0, B)
    sol, r = run_mlp([64, 128, 128, 64], dfx.Tsit5(), dfx.PIDController(rtol=1e-5, atol=1e-7),
                     dfx.SaveAt(t1=True), 0.0, t1, None, y0, "fp32", seed=4)
    err = per_traj_err(sol, r)
    assert err.max() < 2e-5
    assert np.array_equal(sol.ts.cpu().numpy(), r["ts"])


@pytest.mark.parametrize("widths", [[64, 128, 128, 64], [64, 256, 256, 64], [32, 64, 64, 32]])
def test_mlp_bf16_error_level(widths):
    # BF16 tensor-core products of the BF16 weights with activations held as
    # three BF16 pieces (24 bits): the solve matches the FP64 oracle with the
    # same weights to FP32-state accuracy.
    rng = np.random.default_rng(14)
    y0 = rng.standard_normal((256, widths[0]))
    sol, r = run_mlp(widths, dfx.Tsit5(), dfx.PIDController(rtol=1e-5, atol=1e-7),
                     dfx.SaveAt(t1=True), 0.0, 1.0, None, y0, "bf16", seed=5)
    assert (sol.result == 0).all()
    err = per_traj_err(sol, r)
    print(f"MLP {widths} bf16: rel err vs FP64 oracle median {np.median(err):.2e} "
          f"max {err.max():.2e}")
    assert err.max() < 2e-5
    # A smooth field keeps the step count near the FP64 controller's.  On this
    # easy problem the FP64 controller grows dt by its 10x cap from dt0 = 0.01;
    # FP32 stage rounding gives Tsit5's error estimate (error weights
    # |e|_2 ~ 0.76) a noise floor that limits the growth, so an FP32-state
    # solve takes more steps.  Pure BF16 activations took 90x.
    steps = sol.stats["num_steps"].cpu().numpy()
    print(f"attempted steps {steps.mean():.2f}, FP64 oracle {r['stats'][:, 0].mean():.2f}")
    assert steps.mean() < 2.5 * r["stats"][:, 0].mean()


def sde_setup(seed):
    rng = np.random.default_rng(seed)
    Wsig = bf16_round(rng.standard_normal((32, 32)) / np.sqrt(32))
    bsig = rng.standard_normal(32) * 0.1
    return Wsig, bsig.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("solver", [dfx.Heun(), dfx.Euler()])
def test_neural_sde_fp32_matches_oracle(solver):
    # Neural Stratonovich SDE: drift MLP 32 -> 64 -> 64 -> 32, diffusion
    # 0.1 tanh(W y + b), ConstantStepSize dt = 0.01, VBT tol 1e-3 on [0, 1].
    rng = np.random.default_rng(15)
    y0 = rng.standard_normal((96, 32))
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (32,), key=1234)
    sol, r = run_mlp([32, 64, 64, 32], solver, dfx.ConstantStepSize(),
                     dfx.SaveAt(t1=True, ts=np.array([0.25, 0.5])), 0.0, 1.0, 0.01, y0, "fp32",
                     seed=6, diffusion=sde_setup(16), bm=bm)
    err = per_traj_err(sol, r)
    print(f"neural SDE fp32 {solver}: max rel err vs FP64 oracle {err.max():.2e}")
    assert err.max() < 1e-4


def test_neural_sde_bf16_error_level():
    rng = np.random.default_rng(17)
    y0 = rng.standard_normal((256, 32))
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (32,), key=99)
    sol, r = run_mlp([32, 64, 64, 32], dfx.Heun(), dfx.ConstantStepSize(),
                     dfx.SaveAt(t1=True), 0.0, 1.0, 0.01, y0, "bf16", seed=7,
                     diffusion=sde_setup(18), bm=bm)
    err = per_traj_err(sol, r)
    print(f"neural SDE bf16: median rel err {np.median(err):.2e} max {err.max():.2e}")
    assert err.max() < 1e-4


@pytest.mark.parametrize("widths", [[64, 128, 128, 64], [64, 256, 256, 64]])
def test_mlp_adaptive_solve_is_deterministic(widths):
    # the PID error norm sums its per-tile partials in a fixed order, so
    # repeated solves give bit-identical saves and step counts
    dev = torch.device("cuda")
    rng = np.random.default_rng(31)
    Ws, bs = mlp_params(widths, 9, bias_scale=0.1)
    field = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                         [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs])
    y0 = torch.tensor(rng.standard_normal((1024, 64)), dtype=torch.float32, device=dev)
    t1 = torch.tensor(rng.uniform(0.5, 2.0, 1024), dtype=torch.float64, device=dev)
    runs = [dfx.diffeqsolve(dfx.ODETerm(field), dfx.Tsit5(), 0.0, t1, None, y0,
                            saveat=dfx.SaveAt(ts=[0.25, 0.5], t1=True),
                            stepsize_controller=dfx.PIDController(rtol=1e-5, atol=1e-7))
            for _ in range(3)]
    for r in runs[1:]:
        assert torch.equal(r.ys, runs[0].ys)
        assert torch.equal(r.stats["num_steps"], runs[0].stats["num_steps"])
