"""The MLP-field forward on the fifth-generation tensor cores (kernel="tc":
tcgen05.mma with TMEM accumulators and stage vectors, one trajectory per
thread) against the FP64 oracle and against the mma.sync row-tile kernel, on
the neural-ODE shape 64 -> 128 -> 128 -> 64 with Tsit5 + PID."""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O
from test_gpu_mlp import flat, mlp_params, per_traj_err

pytestmark = pytest.mark.gpu


def solve(kernel, y0, saveat, ctrl, seed=5, t1=1.0, bias_scale=0.0, solver=None):
    solver = dfx.Tsit5() if solver is None else solver
    dev = torch.device("cuda")
    Ws, bs = mlp_params([64, 128, 128, 64], seed, bias_scale)
    Ws = [W.astype(np.float32).astype(np.float64) for W in Ws]
    bs = [b.astype(np.float32).astype(np.float64) for b in bs]
    field = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                         [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs])
    tt = lambda x: torch.tensor(x, dtype=torch.float64, device=dev) if isinstance(  # noqa
        x, np.ndarray) else x
    sol = dfx.diffeqsolve(dfx.ODETerm(field), solver, 0.0, tt(t1), None,
                          torch.tensor(y0, dtype=torch.float32, device=dev), saveat=saveat,
                          stepsize_controller=ctrl, throw=False, kernel=kernel)
    torch.cuda.synchronize()
    return sol, field, flat(Ws, bs)


def oracle(field, params, y0, saveat, ctrl, t1=1.0, solver=None):
    solver = dfx.Tsit5() if solver is None else solver
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(dfx.ODETerm(field), solver, ctrl, saveat, dim=64,
                       dtype=torch.float32, max_steps=4096, n_ts=0 if ts is None else ts.size)
    d = O.make_desc(**O.oracle_fields(fields))
    return O.solve(d, 0.0, t1, None, y0, params=params, ts=ts, nthreads=8)


def test_tc_matches_oracle_and_rowtile():
    rng = np.random.default_rng(61)
    y0 = rng.standard_normal((300, 64))  # 3 tiles, the last one partial
    pid = dfx.PIDController(rtol=1e-5, atol=1e-7)
    saveat = dfx.SaveAt(t0=True, ts=np.linspace(0.0, 1.0, 9), t1=True)
    sol, field, params = solve("tc", y0, saveat, pid)
    ref, _, _ = solve("fused", y0, saveat, pid)
    r = oracle(field, params, y0, saveat, pid)
    assert (sol.result == 0).all()
    err = per_traj_err(sol, r)
    print(f"tc: rel err vs FP64 oracle median {np.median(err):.2e} max {err.max():.2e}; "
          f"steps {sol.stats['num_steps'].float().mean():.2f} (row tile "
          f"{ref.stats['num_steps'].float().mean():.2f}, oracle {r['stats'][:, 0].mean():.2f})")
    # BF16 weights and three-piece activations, as the row-tile kernel:
    # FP32-state accuracy
    assert err.max() < 2e-5
    assert np.array_equal(sol.ts.cpu().numpy(), r["ts"])
    steps = sol.stats["num_steps"].cpu().numpy()
    assert steps.mean() < 2.5 * r["stats"][:, 0].mean()
    d = (sol.ys - ref.ys).abs().max() / ref.ys.abs().max()
    assert float(d) < 1e-4


def test_tc_uneven_t1_refill_and_constant_steps():
    # Per-trajectory t1 (rows finish at different steps and refill from the
    # queue) and a constant-step solve.
    rng = np.random.default_rng(62)
    B = 700
    y0 = rng.standard_normal((B, 64))
    t1 = rng.uniform(0.2, 2.0, B)
    pid = dfx.PIDController(rtol=1e-4, atol=1e-6)
    sol, field, params = solve("tc", y0, dfx.SaveAt(t1=True), pid, seed=6, t1=t1,
                               bias_scale=0.1)
    r = oracle(field, params, y0, dfx.SaveAt(t1=True), pid, t1=t1)
    assert (sol.result == 0).all()
    err = per_traj_err(sol, r)
    assert err.max() < 1e-3, err.max()
    assert np.array_equal(sol.ts.cpu().numpy(), r["ts"])
    y0c = rng.standard_normal((200, 64))
    const = dfx.ConstantStepSize()
    dev = torch.device("cuda")
    Ws, bs = mlp_params([64, 128, 128, 64], 7)
    fld = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                       [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs])
    a = dfx.diffeqsolve(dfx.ODETerm(fld), dfx.Tsit5(), 0.0, 1.0, 0.05,
                        torch.tensor(y0c, dtype=torch.float32, device=dev),
                        stepsize_controller=const, kernel="tc")
    b = dfx.diffeqsolve(dfx.ODETerm(fld), dfx.Tsit5(), 0.0, 1.0, 0.05,
                        torch.tensor(y0c, dtype=torch.float32, device=dev),
                        stepsize_controller=const, kernel="fused")
    assert (a.stats["num_steps"] == 20).all()
    assert float((a.ys - b.ys).abs().max() / b.ys.abs().max()) < 2e-5


def test_tc_dopri5_matches_oracle_and_rowtile():
    # Dopri5 on the tensor-core tiles: its quartic interpolant for the ts saves
    rng = np.random.default_rng(62)
    y0 = rng.standard_normal((300, 64))
    pid = dfx.PIDController(rtol=1e-5, atol=1e-7)
    saveat = dfx.SaveAt(t0=True, ts=np.linspace(0.0, 1.0, 9), t1=True)
    sol, field, params = solve("tc", y0, saveat, pid, solver=dfx.Dopri5(), bias_scale=0.1)
    ref, _, _ = solve("fused", y0, saveat, pid, solver=dfx.Dopri5(), bias_scale=0.1)
    r = oracle(field, params, y0, saveat, pid, solver=dfx.Dopri5())
    assert (sol.result == 0).all()
    err = per_traj_err(sol, r)
    err_ref = per_traj_err(ref, r)
    print(f"tc Dopri5: rel err vs FP64 oracle median {np.median(err):.2e} max {err.max():.2e} "
          f"(row tile {np.median(err_ref):.2e} / {err_ref.max():.2e})")
    # the solve's tolerance level (FP32 and FP64 controllers take different
    # steps), and the row-tile kernel's
    assert err.max() < 5e-5 and err.max() < 1.5 * err_ref.max()
    d = (sol.ys - ref.ys).abs().max() / ref.ys.abs().max()
    assert float(d) < 1e-4
