"""The Ornstein-Uhlenbeck SDE dy = theta (mu - y) dt + sigma dW on the
analytic-field kernels (MultiTerm(ODETerm, ControlTerm) with a
VirtualBrownianTree, diffrax/_term.py:271-731, diffrax/_brownian/tree.py)
against the FP64 oracle fed the identical Brownian path, and against the
process's known law."""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu


def solve_pair(solver, ctrl, dt0, y0, args, bm, kernel, saveat=None, max_steps=4096):
    dev = torch.device("cuda")
    saveat = saveat or dfx.SaveAt(t1=True)
    terms = dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                          dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))
    sol = dfx.diffeqsolve(terms, solver, bm.t0, bm.t1, dt0,
                          torch.tensor(y0, dtype=torch.float32, device=dev),
                          torch.tensor(args, dtype=torch.float32, device=dev), saveat=saveat,
                          stepsize_controller=ctrl, max_steps=max_steps, throw=False,
                          kernel=kernel)
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(terms, solver, ctrl, saveat, dim=y0.shape[1], dtype=torch.float32,
                       max_steps=max_steps, n_ts=0 if ts is None else ts.size)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, bm.t0, bm.t1, dt0, y0, args=args, ts=ts, nthreads=8)
    return sol, r


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("solver, dim", [("heun", 2), ("euler", 4), ("heun", 4)])
def test_ou_sde_matches_oracle_on_the_same_path(kernel, solver, dim):
    rng = np.random.default_rng(51)
    B = 2048
    y0 = rng.uniform(-2, 2, (B, dim))
    args = np.array([1.5, 0.5, 0.3])
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (dim,), key=7)
    s = {"heun": dfx.Heun(), "euler": dfx.Euler()}[solver]
    saveat = dfx.SaveAt(ts=np.linspace(0.0, 1.0, 11), t1=True)
    sol, r = solve_pair(s, dfx.ConstantStepSize(), 0.01, y0, args, bm, kernel, saveat)
    assert (sol.result.cpu().numpy() == 0).all()
    assert np.array_equal(sol.stats["num_steps"].cpu().numpy(), r["stats"][:, 0])
    ys = sol.ys.cpu().double().numpy()
    # FP32 state and FP32 tree values against the FP64 oracle on the same
    # integer stream
    err = np.abs(ys - r["ys"]).max() / np.abs(r["ys"]).max()
    assert err < 2e-5, err


def test_ou_sde_adaptive_heun_matches_oracle():
    # Heun with a PID controller (adaptive SDE stepping, error order 1,
    # _integrate.py:1145-1151 allows it for Heun).  The FP32-state controller
    # forms its step factor in FP32, so step ends differ from the FP64
    # oracle's by ~1e-7 relative, and on a Brownian path (Hoelder 1/2) that
    # moves the increments by ~sqrt(1e-7 dt): the step sequences part after a
    # while.  Both are then discretisations of the same path at the same
    # tolerance: compare the solutions and the step counts statistically.
    rng = np.random.default_rng(52)
    B = 1024
    y0 = rng.uniform(-2, 2, (B, 2))
    args = np.array([2.0, -0.3, 0.2])
    bm = dfx.VirtualBrownianTree(0.0, 2.0, 1e-4, (2,), key=11)
    sol, r = solve_pair(dfx.Heun(), dfx.PIDController(rtol=1e-3, atol=1e-4), 0.01, y0, args,
                        bm, "fused", max_steps=16384)
    assert (sol.result.cpu().numpy() == 0).all()
    n_gpu = sol.stats["num_steps"].cpu().numpy().mean()
    assert abs(n_gpu / r["stats"][:, 0].mean() - 1) < 0.05
    ys = sol.ys.cpu().double().numpy()[:, 0]
    per = np.abs(ys - r["ys"][:, 0]).max(axis=1) / np.abs(r["ys"]).max()
    assert np.median(per) < 5e-3 and per.max() < 5e-2, (np.median(per), per.max())


def test_ou_sde_law():
    # Heun dt = 0.01 on [0, 1] from y0 = 2: mean mu + (y0 - mu) e^{-theta t},
    # variance sigma^2 (1 - e^{-2 theta t}) / (2 theta), over 65536 paths.
    B, theta, mu, sigma = 65536, 1.5, 0.5, 0.3
    dev = torch.device("cuda")
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), key=3)
    terms = dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                          dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))
    sol = dfx.diffeqsolve(terms, dfx.Heun(), 0.0, 1.0, 0.01,
                          torch.full((B, 2), 2.0, dtype=torch.float32, device=dev),
                          torch.tensor([theta, mu, sigma], dtype=torch.float32, device=dev))
    y = sol.ys[:, 0].double().cpu().numpy().reshape(-1)
    m = mu + (2.0 - mu) * np.exp(-theta)
    v = sigma ** 2 * (1 - np.exp(-2 * theta)) / (2 * theta)
    n = y.size
    assert abs(y.mean() - m) < 5 * np.sqrt(v / n) + 1e-3
    assert abs(y.var() / v - 1) < 0.03
