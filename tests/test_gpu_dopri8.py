"""GPU parity of the Dopri8 solver (diffrax/_solver/dopri8.py: 14-stage 8(7)
pair, FSAL/SSAL, Bogacki--Shampine dense output) on the analytic-field kernels
against the FP64 oracle, which is pinned for Dopri8 to the reference's order,
DETEST and dense-output tests in tests/test_oracle_pins.py.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O
from test_gpu_dense import rows_close, solve_pair

pytestmark = pytest.mark.gpu

LV_ARGS = np.array([0.1, 0.02, 0.4, 0.02])


def same_steps(sol, r):
    same = sol.stats["num_steps"].cpu().numpy() == r["stats"][:, 0]
    same &= sol.stats["num_accepted_steps"].cpu().numpy() == r["stats"][:, 1]
    assert same.mean() >= 0.95, f"only {same.mean():.3f} took the oracle's steps"
    return same


@pytest.mark.parametrize("kernel", ["plain", "fused"])
@pytest.mark.parametrize("controller", ["pid", "constant"])
def test_dopri8_fp64_matches_oracle(kernel, controller):
    # Lotka-Volterra on [0, 140], 100 ts saves (the interpolant) and t1.
    rng = np.random.default_rng(41)
    y0 = rng.uniform(5, 15, (128, 2))
    ctrl = (dfx.PIDController(rtol=1e-9, atol=1e-11) if controller == "pid"
            else dfx.ConstantStepSize())
    saveat = dfx.SaveAt(ts=np.linspace(0.0, 140.0, 100), t1=True)
    sol, r, d = solve_pair(dfx.LotkaVolterra(), dfx.Dopri8(), ctrl, saveat, 0.0, 140.0, 0.25,
                           y0, LV_ARGS, torch.float64, kernel)
    same = same_steps(sol, r)
    rows_close(sol.ys.cpu().numpy(), r["ys"], same, 1e-9)
    assert np.array_equal(sol.result.cpu().numpy(), r["result"])
    assert (r["result"] == 0).all()


def test_dopri8_dense_and_event():
    # Dense output and an event located by Newton on the Dopri8 interpolant.
    rng = np.random.default_rng(42)
    B = 64
    y0 = rng.uniform(-2, 2, (B, 2))
    mu = np.exp(rng.uniform(np.log(0.1), np.log(3.0), (B, 1)))
    saveat = dfx.SaveAt(t1=True, dense=True)
    sol, r, d = solve_pair(dfx.VanDerPol(), dfx.Dopri8(),
                           dfx.PIDController(rtol=1e-9, atol=1e-11), saveat, 0.0, 15.0, None,
                           y0, mu, torch.float64, "fused")
    same = same_steps(sol, r)
    # Van der Pol at rtol 1e-9 over hundreds of steps: GPU and host FP64 pow
    # differ by an ulp now and then, and a step sequence that differs by one
    # ulp somewhere moves every later step (records then differ by up to ~1e-4
    # relative, as perturbing the oracle's PID factor by one ulp shows).  So
    # the records are compared on the trajectories whose step times equal the
    # oracle's, and the evaluation against the oracle's DenseInterpolation
    # over the GPU's own records.
    it = sol.interpolation
    tsg = it.ts.cpu().numpy()
    ident = same & np.all((tsg == r["dense_ts"]) | (np.isinf(tsg) & np.isinf(r["dense_ts"])),
                          axis=1)
    assert ident.mean() >= 0.5
    rows_close(it.infos.cpu().numpy(), r["dense_info"], ident, 1e-9, min_frac=ident.mean())
    mine = dict(dense_ts=it.ts.cpu().numpy(), dense_info=it.infos.cpu().numpy(),
                dense_n=it.ts_size.cpu().numpy())
    q = np.linspace(0.0, 15.0, 61)
    everyone = np.ones(B, dtype=bool)
    for order in (0, 1):
        got = (sol.evaluate if order == 0 else sol.derivative)(torch.tensor(q))
        rows_close(got.cpu().numpy(), O.dense_evaluate(d, 0.0, 15.0, y0, mine, q, order=order),
                   everyone, 1e-10, min_frac=1.0, loose=1e-10)
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-10, 1e-10), direction=False)
    dev = torch.device("cuda")
    sol = dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri8(), 0.0, 15.0, None,
                          torch.tensor(y0, device=dev), torch.tensor(mu, device=dev),
                          stepsize_controller=dfx.PIDController(rtol=1e-9, atol=1e-11),
                          event=ev, throw=False, kernel="fused")
    fired = sol.event_mask.cpu().numpy() & (sol.result.cpu().numpy() == 3)
    assert fired.mean() > 0.5
    assert np.abs(sol.ys.cpu().numpy()[fired, 0, 0]).max() < 1e-9


def test_dopri8_fp32_fused_van_der_pol():
    # FP32 state (FP64 time), the headline workload's shape at Dopri8.
    rng = np.random.default_rng(43)
    B = 1024
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), (B, 1)))
    y0 = rng.uniform(-2, 2, (B, 2))
    t1 = rng.uniform(5, 50, B)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    sol, r, d = solve_pair(dfx.VanDerPol(), dfx.Dopri8(), pid, dfx.SaveAt(t1=True), 0.0, t1,
                           None, y0, mu, torch.float32, "fused")
    got = sol.ys.cpu().double().numpy()
    per = np.abs(got - r["ys"]).max(axis=(1, 2)) / np.abs(r["ys"]).max(axis=(1, 2))
    assert (sol.result.cpu().numpy() == 0).all()
    assert np.median(per) < 1e-4 and per.max() < 5e-2, (np.median(per), per.max())
