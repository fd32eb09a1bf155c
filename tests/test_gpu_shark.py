"""The additive-noise SRKs (ShARK, SRA1, SEA) and the virtual Brownian tree
with space-time Levy area on the analytic-field kernels
(diffrax/_solver/{shark,sra1,sea}.py, the additive-noise branch of
diffrax/_solver/srk.py:335-671, diffrax/_brownian/tree.py:94-126, 562-603,
727-750), against the FP64 oracle fed the identical integer stream, and
against the Ornstein-Uhlenbeck process's known law."""
import math

import numpy as np
import pytest
import scipy.stats
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu


def _terms(bm):
    return dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                         dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))


def solve_pair(solver, ctrl, t0, t1, dt0, y0, args, bm, kernel, saveat=None, max_steps=4096):
    dev = torch.device("cuda")
    saveat = saveat or dfx.SaveAt(t1=True)
    terms = _terms(bm)
    sol = dfx.diffeqsolve(terms, solver, t0, t1, dt0,
                          torch.tensor(y0, dtype=torch.float32, device=dev),
                          torch.tensor(args, dtype=torch.float32, device=dev), saveat=saveat,
                          stepsize_controller=ctrl, max_steps=max_steps, throw=False,
                          kernel=kernel)
    torch.cuda.synchronize()
    ts = None if saveat.ts is None else np.asarray(saveat.ts, dtype=np.float64)
    fields = dfx.lower(terms, solver, ctrl, saveat, dim=y0.shape[1], dtype=torch.float32,
                       max_steps=max_steps, n_ts=0 if ts is None else ts.size)
    d = O.make_desc(**O.oracle_fields(fields))
    r = O.solve(d, t0, t1, dt0, y0, args=args, ts=ts, nthreads=8)
    return sol, r


def test_device_levy_tree_matches_oracle():
    # One ShARK step of the Ornstein-Uhlenbeck SDE from y0 = 0 with mu = 0,
    # sigma = 1 and h = 1: theta = 0 gives y1 = W, theta = 1 gives
    # y1 = (W - H) / 2.  So two solves read the device tree's (W, H) of
    # [0.3, 1.3] (inside a tree on [0, 2]) for every trajectory.
    B = 65536
    bm = dfx.VirtualBrownianTree(0.0, 2.0, 2 ** -12, (2,), key=21,
                                 levy_area=dfx.SpaceTimeLevyArea)
    dev = torch.device("cuda")
    y0 = torch.zeros(B, 2, dtype=torch.float32, device=dev)

    def one_step(theta):
        args = torch.tensor([theta, 0.0, 1.0], dtype=torch.float32, device=dev)
        sol = dfx.diffeqsolve(_terms(bm), dfx.ShARK(), 0.3, 1.3, 1.0, y0, args)
        return sol.ys[:, 0].double().cpu().numpy()
    w = one_step(0.0)
    h = w - 2 * one_step(1.0)
    d = O.make_desc(dim=2, vbt_t0=0.0, vbt_t1=2.0, vbt_tol=2 ** -12, seed=21)
    n = 4096
    wo, ho = O.vbt_levy_increments(d, np.arange(n), np.full(n, 0.3), np.full(n, 1.3))
    # FP32 descent and Chen's relation against FP64
    assert np.abs(w[:n] - wo).max() < 2e-5, np.abs(w[:n] - wo).max()
    assert np.abs(h[:n] - ho).max() < 1e-4, np.abs(h[:n] - ho).max()
    # the law (test/test_brownian.py:120-175): W ~ N(0, 1), H ~ N(0, 1/12)
    assert scipy.stats.kstest(w.reshape(-1), "norm").pvalue > 1e-3
    assert scipy.stats.kstest(h.reshape(-1), scipy.stats.norm(0, math.sqrt(1 / 12)).cdf).pvalue > 1e-3
    assert abs(np.mean(w * h)) < 0.01


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("solver, dim", [("shark", 2), ("shark", 4), ("sra1", 2), ("sea", 4),
                                         ("heun", 2), ("euler", 4)])
def test_levy_tree_solvers_match_oracle_on_the_same_path(kernel, solver, dim):
    rng = np.random.default_rng(61)
    B = 2048
    y0 = rng.uniform(-2, 2, (B, dim))
    args = np.array([1.5, 0.5, 0.6])
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (dim,), key=9,
                                 levy_area=dfx.SpaceTimeLevyArea)
    s = {"shark": dfx.ShARK(), "sra1": dfx.SRA1(), "sea": dfx.SEA(), "heun": dfx.Heun(),
         "euler": dfx.Euler()}[solver]
    saveat = dfx.SaveAt(ts=np.linspace(0.0, 1.0, 11), t1=True)
    sol, r = solve_pair(s, dfx.ConstantStepSize(), 0.0, 1.0, 0.02, y0, args, bm, kernel, saveat)
    assert (sol.result.cpu().numpy() == 0).all()
    assert np.array_equal(sol.stats["num_steps"].cpu().numpy(), r["stats"][:, 0])
    ys = sol.ys.cpu().double().numpy()
    err = np.abs(ys - r["ys"]).max() / np.abs(r["ys"]).max()
    assert err < 5e-5, err


def test_shark_reverse_time_matches_oracle():
    # t0 > t1: the increments are the forward real interval's times the
    # direction (_term.py:742-745), and the drift's control is the loop's step
    # (srk.py:364), as the oracle restates.
    rng = np.random.default_rng(62)
    B = 1024
    y0 = rng.uniform(-2, 2, (B, 2))
    args = np.array([1.2, -0.5, 0.4])
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), key=4,
                                 levy_area=dfx.SpaceTimeLevyArea)
    saveat = dfx.SaveAt(ts=np.linspace(1.0, 0.0, 6), t1=True)
    sol, r = solve_pair(dfx.ShARK(), dfx.ConstantStepSize(), 1.0, 0.0, -0.05, y0, args, bm,
                        "fused", saveat)
    assert (sol.result.cpu().numpy() == 0).all()
    assert np.array_equal(sol.stats["num_steps"].cpu().numpy(), r["stats"][:, 0])
    ys = sol.ys.cpu().double().numpy()
    err = np.abs(ys - r["ys"]).max() / np.abs(r["ys"]).max()
    assert err < 5e-5, err


@pytest.mark.parametrize("solver", [dfx.ShARK(), dfx.SRA1()])
def test_srk_adaptive_matches_oracle(solver):
    # ShARK / SRA1 with a PID controller (error order strong_order + 1/2 = 2,
    # base.py:292-301).  As for Heun, FP32 step factors part the step
    # sequences from the FP64 oracle's after a while on a Brownian path:
    # compare the step counts and solutions statistically.
    rng = np.random.default_rng(63)
    B = 1024
    y0 = rng.uniform(-2, 2, (B, 2))
    args = np.array([2.0, -0.3, 0.2])
    bm = dfx.VirtualBrownianTree(0.0, 2.0, 1e-4, (2,), key=13,
                                 levy_area=dfx.SpaceTimeLevyArea)
    sol, r = solve_pair(solver, dfx.PIDController(rtol=1e-3, atol=1e-4), 0.0, 2.0, 0.01,
                        y0, args, bm, "fused", max_steps=16384)
    assert (sol.result.cpu().numpy() == 0).all()
    n_gpu = sol.stats["num_steps"].cpu().numpy().mean()
    assert abs(n_gpu / r["stats"][:, 0].mean() - 1) < 0.05
    ys = sol.ys.cpu().double().numpy()[:, 0]
    per = np.abs(ys - r["ys"][:, 0]).max(axis=1) / np.abs(r["ys"]).max()
    assert np.median(per) < 5e-3 and per.max() < 5e-2, (np.median(per), per.max())


def test_shark_ou_law():
    # ShARK dt = 0.05 on [0, 1] from y0 = 2: mean mu + (y0 - mu) e^{-theta t},
    # variance sigma^2 (1 - e^{-2 theta t}) / (2 theta), over 65536 paths.
    B, theta, mu, sigma = 65536, 1.5, 0.5, 0.3
    dev = torch.device("cuda")
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), key=3,
                                 levy_area=dfx.SpaceTimeLevyArea)
    sol = dfx.diffeqsolve(_terms(bm), dfx.ShARK(), 0.0, 1.0, 0.05,
                          torch.full((B, 2), 2.0, dtype=torch.float32, device=dev),
                          torch.tensor([theta, mu, sigma], dtype=torch.float32, device=dev))
    y = sol.ys[:, 0].double().cpu().numpy().reshape(-1)
    m = mu + (2.0 - mu) * np.exp(-theta)
    v = sigma ** 2 * (1 - np.exp(-2 * theta)) / (2 * theta)
    n = y.size
    assert abs(y.mean() - m) < 5 * np.sqrt(v / n) + 1e-3
    assert abs(y.var() / v - 1) < 0.03
