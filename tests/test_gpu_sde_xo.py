"""SaveAt(steps=n), SaveAt(dense=True), ClipStepSizeController and events on
the Ornstein-Uhlenbeck SDE (diffrax/_integrate.py:492-540, 542-821,
diffrax/_step_size_controller/clip.py), on the W-only and the space-time Levy
area trees, against the FP64 oracle fed the identical Brownian path."""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu

ARGS = np.array([1.5, 0.5, 0.6])


def _terms(levy, key=17, dim=2, t1=1.0):
    bm = dfx.VirtualBrownianTree(0.0, t1, 1e-3, (dim,), key=key, levy_area=levy)
    return dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                         dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))


def _pair(solver, levy, saveat, ctrl, dt0, y0, max_steps=128, event=None, step_ts=None,
          jump_ts=None):
    dev = torch.device("cuda")
    terms = _terms(levy, dim=y0.shape[1])
    sol = dfx.diffeqsolve(terms, solver, 0.0, 1.0, dt0,
                          torch.tensor(y0, dtype=torch.float32, device=dev),
                          torch.tensor(ARGS, dtype=torch.float32, device=dev), saveat=saveat,
                          stepsize_controller=ctrl, max_steps=max_steps, throw=False,
                          event=event)
    torch.cuda.synchronize()
    fields = dfx.lower(terms, solver, ctrl, saveat, dim=y0.shape[1], dtype=torch.float32,
                       max_steps=max_steps, n_ts=0 if saveat.ts is None else len(saveat.ts),
                       event=event)
    d = O.make_desc(**O.oracle_fields(fields))
    ts = None if saveat.ts is None else np.asarray(saveat.ts, np.float64)
    r = O.solve(d, 0.0, 1.0, dt0, y0, args=ARGS, ts=ts, nthreads=8, step_ts=step_ts,
                jump_ts=jump_ts)
    return sol, r, d


@pytest.mark.parametrize("solver, levy", [(dfx.Heun(), dfx.BrownianIncrement),
                                          (dfx.ShARK(), dfx.SpaceTimeLevyArea),
                                          (dfx.SEA(), dfx.SpaceTimeLevyArea)])
def test_sde_saveat_steps(solver, levy):
    rng = np.random.default_rng(71)
    y0 = rng.uniform(-2, 2, (1024, 2))
    sol, r, _ = _pair(solver, levy, dfx.SaveAt(steps=2, t1=True), dfx.ConstantStepSize(),
                      0.02, y0)
    assert (sol.result.cpu().numpy() == 0).all()
    ts = sol.ts.cpu().numpy()
    assert np.array_equal(ts, r["ts"])  # the constant-step grid, inf past the saves
    fin = np.isfinite(r["ts"])
    ys = sol.ys.cpu().double().numpy()
    assert np.isinf(ys[~fin]).all()
    err = np.abs(ys[fin] - r["ys"][fin]).max() / np.abs(r["ys"][fin]).max()
    assert err < 5e-5, err


@pytest.mark.parametrize("solver, levy", [(dfx.Heun(), dfx.BrownianIncrement),
                                          (dfx.SRA1(), dfx.SpaceTimeLevyArea)])
def test_sde_dense_output(solver, levy):
    # the dense records of the step grid, and their evaluation (Heun: the
    # Hermite interpolant of its noisy stages; the SRKs: linear) against the
    # oracle's evaluation of its own records
    rng = np.random.default_rng(72)
    y0 = rng.uniform(-2, 2, (512, 2))
    sol, r, d = _pair(solver, levy, dfx.SaveAt(dense=True, t1=True), dfx.ConstantStepSize(),
                      0.05, y0, max_steps=64)
    assert (sol.result.cpu().numpy() == 0).all()
    interp = sol.interpolation
    assert np.array_equal(interp.ts.cpu().numpy(), r["dense_ts"])
    q = np.linspace(0.0, 1.0, 37)
    yq = interp.evaluate(torch.tensor(q, device="cuda")).double().cpu().numpy()
    rq = O.dense_evaluate(d, 0.0, 1.0, y0, r, q)
    err = np.abs(yq - rq).max() / np.abs(rq).max()
    assert err < 5e-5, err


def test_sde_clip_controller_lands_on_step_ts():
    # ShARK with PID inside ClipStepSizeController: every step time is a step
    # end, the steps skip over each jump time, and the step counts agree with
    # the oracle's statistically (FP32 step factors part the sequences).
    rng = np.random.default_rng(73)
    y0 = rng.uniform(-2, 2, (512, 2))
    step_ts = np.linspace(0.0, 1.0, 21)
    jump_ts = np.array([0.33, 0.71])
    pid = dfx.PIDController(rtol=1e-3, atol=1e-4)
    ctrl = dfx.ClipStepSizeController(pid, step_ts=step_ts, jump_ts=jump_ts)
    sol, r, _ = _pair(dfx.ShARK(), dfx.SpaceTimeLevyArea, dfx.SaveAt(dense=True, t1=True),
                      ctrl, 0.01, y0, max_steps=2048, step_ts=step_ts, jump_ts=jump_ts)
    assert (sol.result.cpu().numpy() == 0).all()
    dts = sol.interpolation.ts.cpu().numpy()
    n = sol.interpolation.ts_size.cpu().numpy()
    for b in range(0, 512, 37):
        t = dts[b, :n[b]]
        assert np.isin(step_ts, t).all()
        for j in jump_ts:  # no step ends exactly at a jump: it ends just below
            assert not np.isin(j, t)
    n_gpu = sol.stats["num_steps"].cpu().numpy().mean()
    assert abs(n_gpu / r["stats"][:, 0].mean() - 1) < 0.05


def test_sde_event_with_root():
    # Heun with constant steps; y_0 crosses 1 upwards; Newton root on the
    # step's interpolant.  Same path and step grid: the same trajectories
    # fire, at the same times.
    rng = np.random.default_rng(74)
    y0 = rng.uniform(-2, 0.5, (2048, 2))
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0], offset=-1.0), dfx.Newton(1e-6, 1e-6),
                   direction=True)
    sol, r, _ = _pair(dfx.Heun(), dfx.BrownianIncrement, dfx.SaveAt(t1=True),
                      dfx.ConstantStepSize(), 0.02, y0, event=ev)
    fired = sol.event_mask.cpu().numpy()
    ref = r["event_index"] == 0
    assert 0.05 < fired.mean() < 0.95
    assert (fired == ref).mean() > 0.99
    both = fired & ref
    tg = sol.ts.cpu().numpy()[both, 0]
    assert np.median(np.abs(tg - r["ts"][both, 0])) < 1e-5
