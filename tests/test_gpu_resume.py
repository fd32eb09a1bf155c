"""Resuming a solve from its saved solver and controller states
(diffeqsolve's solver_state / controller_state / made_jump inputs and the
SaveAt(solver_state=, controller_state=, made_jump=) outputs,
diffrax/_integrate.py:1252-1271, 1309, 1489-1500), against the FP64 oracle
given the same resume records.

FP64 states must reproduce the oracle's records and step counts; FP32 states
agree within the solve's tolerance.
"""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx
import oracle as O

pytestmark = pytest.mark.gpu

STATES = dict(solver_state=True, controller_state=True, made_jump=True)


def _oracle(field, solver, controller, saveat, dim, dtype, max_steps, **kw):
    fields = dfx.lower(dfx.ODETerm(field), solver, controller, saveat, dim=dim, dtype=dtype,
                       max_steps=max_steps, n_ts=0)
    return O.solve(O.make_desc(**O.oracle_fields(fields)), nthreads=8, want_state=True, **kw)


def _record(sol):
    """The [B, 7 + dim] record gbdx_solve_fwd_ex wrote."""
    return sol.lowered.state_record.cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("solver", ["dopri5", "tsit5", "dopri8"])
def test_pid_resume_matches_oracle(solver, dtype):
    # Van der Pol mu = 1, PID(1e-6, 1e-8): leg 1 on [0, 3], then leg 2 on
    # [3, 7] resumed from leg 1's states (FSAL f0, PID errors), dt0 = 0.05.
    solver = {"dopri5": dfx.Dopri5(), "tsit5": dfx.Tsit5(), "dopri8": dfx.Dopri8()}[solver]
    ctrl = dfx.PIDController(rtol=1e-6, atol=1e-8, pcoeff=0.2, icoeff=0.4)
    rng = np.random.default_rng(3)
    B, D = 96, 2
    y0 = rng.uniform(-2, 2, (B, D))
    mu = np.array([1.0])
    dev = torch.device("cuda")
    field = dfx.VanDerPol()
    sa1 = dfx.SaveAt(t1=True, **STATES)
    s1 = dfx.diffeqsolve(dfx.ODETerm(field), solver, 0.0, 3.0, 0.05,
                         torch.tensor(y0, dtype=dtype, device=dev),
                         torch.tensor(mu, dtype=dtype, device=dev), saveat=sa1,
                         stepsize_controller=ctrl, max_steps=4096)
    r1 = _oracle(field, solver, ctrl, sa1, D, dtype, 4096, t0=0.0, t1=3.0, dt0=0.05, y0=y0,
                 args=mu)
    rec1 = _record(s1)
    # the record: passed flag, first_step (an FSAL value is present), made_jump
    assert np.array_equal(rec1[:, 4:7], r1["state"][:, 4:7])
    assert (rec1[:, 5] == 0).all()
    if dtype == torch.float64:
        # f0 and the PID errors follow the oracle's step sequence (a
        # trajectory whose accept/reject sequence is ulp-sensitive may take
        # another).  f0 is the field at the final state (1e-9); the errors are
        # ratios of an embedded error estimate, a sum of cancelling stage
        # terms, so ulp-level stage differences move them by far more (1e-4).
        same = s1.stats["num_steps"].cpu().numpy() == r1["stats"][:, 0]
        f0s = np.abs(r1["state"][:, 7:]).max()
        f0_ok = (np.abs(rec1[:, 7:] - r1["state"][:, 7:]) <= 1e-9 * f0s).all(axis=1)
        pid_ok = (np.abs(rec1[:, :3] - r1["state"][:, :3]) <= 1e-4 * np.abs(r1["state"][:, :3])
                  ).all(axis=1)
        print(f"leg 1: steps equal {same.mean():.3f}, f0 {f0_ok.mean():.3f}, "
              f"PID errors {pid_ok.mean():.3f}")
        assert (same & f0_ok).mean() >= 0.95
        # a final step clipped to t1 can be tiny, with an error estimate at
        # the rounding level: its PID entries then carry no digits
        assert (same & pid_ok).mean() >= 0.85
    # the Solution's tuples hold the same record
    cs, ss, mj = s1.controller_state, s1.solver_state, s1.made_jump
    assert len(cs) == 3 and cs[2].dtype == torch.bool and not bool(mj.any())
    assert ss[1].shape == (B, D) and ss[1].dtype == dtype and not bool(ss[0].any())

    sa2 = dfx.SaveAt(t1=True, **STATES)
    s2 = dfx.diffeqsolve(dfx.ODETerm(field), solver, 3.0, 7.0, 0.05, s1.ys[:, -1],
                         torch.tensor(mu, dtype=dtype, device=dev), saveat=sa2,
                         stepsize_controller=ctrl, max_steps=4096,
                         solver_state=ss, controller_state=cs, made_jump=mj)
    torch.cuda.synchronize()
    r2 = _oracle(field, solver, ctrl, sa2, D, dtype, 4096, t0=3.0, t1=7.0, dt0=0.05,
                 y0=s1.ys[:, -1].double().cpu().numpy(), args=mu, state_in=rec1)
    ys = s2.ys.double().cpu().numpy()
    scale = np.abs(r2["ys"]).max()
    err = np.abs(ys - r2["ys"]).max() / scale
    steps = s2.stats["num_steps"].cpu().numpy()
    print(f"resume {dtype}: max rel err {err:.2e}, steps equal "
          f"{(steps == r2['stats'][:, 0]).mean():.3f}")
    if dtype == torch.float64:
        assert err < 1e-9
        assert (steps == r2["stats"][:, 0]).mean() >= 0.95
    else:
        assert err < 2e-4
    # the passed PID state steers the steps: a fresh solve from the same point
    # takes another step sequence
    r3 = _oracle(field, solver, ctrl, sa2, D, dtype, 4096, t0=3.0, t1=7.0, dt0=0.05,
                 y0=s1.ys[:, -1].double().cpu().numpy(), args=mu)
    assert not np.array_equal(r3["ys"], r2["ys"])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("solver", ["euler", "heun", "tsit5"])
def test_constant_step_resume_continues_the_grid(solver, dtype):
    # Lotka-Volterra, ConstantStepSize dt0 = 0.1 on [0, 20]: leg 1 stops at
    # max_steps = 70 (throw=False); leg 2 resumes from step 70 with leg 1's
    # states and finishes the grid t0 + (t1 - t0) k / 200.
    solver = {"euler": dfx.Euler(), "heun": dfx.Heun(), "tsit5": dfx.Tsit5()}[solver]
    ctrl = dfx.ConstantStepSize()
    rng = np.random.default_rng(5)
    B, D = 64, 2
    y0 = rng.uniform(5, 15, (B, D))
    lv = np.array([0.1, 0.02, 0.4, 0.02])
    dev = torch.device("cuda")
    field = dfx.LotkaVolterra()
    args = torch.tensor(lv, dtype=dtype, device=dev)
    sa1 = dfx.SaveAt(steps=True, **STATES)
    s1 = dfx.diffeqsolve(dfx.ODETerm(field), solver, 0.0, 20.0, 0.1,
                         torch.tensor(y0, dtype=dtype, device=dev), args, saveat=sa1,
                         stepsize_controller=ctrl, max_steps=70, throw=False)
    assert (s1.result.cpu().numpy() == int(dfx.RESULTS.max_steps_reached)).all()
    # steps_completed starts at 1 (the first step is planned at init,
    # constant.py:30-55) and counts one more per step taken
    sc, nc, t0s, t1s = s1.controller_state
    assert (sc.cpu().numpy() == 71).all() and (nc.cpu().numpy() == 200).all()
    assert (t0s.cpu().numpy() == 0.0).all() and (t1s.cpu().numpy() == 20.0).all()
    r1 = _oracle(field, solver, ctrl, sa1, D, dtype, 70, t0=0.0, t1=20.0, dt0=0.1, y0=y0,
                 args=lv)
    rec1 = _record(s1)
    assert np.array_equal(rec1[:, :7], r1["state"][:, :7])

    t_m = s1.ts[:, 69].contiguous()
    y_m = s1.ys[:, 69].contiguous()
    sa2 = dfx.SaveAt(t1=True, **STATES)
    s2 = dfx.diffeqsolve(dfx.ODETerm(field), solver, t_m, 20.0, 0.1, y_m, args, saveat=sa2,
                         stepsize_controller=ctrl, max_steps=4096,
                         solver_state=s1.solver_state, controller_state=s1.controller_state,
                         made_jump=s1.made_jump)
    full = dfx.diffeqsolve(dfx.ODETerm(field), solver, 0.0, 20.0, 0.1,
                           torch.tensor(y0, dtype=dtype, device=dev), args,
                           saveat=dfx.SaveAt(t1=True), stepsize_controller=ctrl,
                           max_steps=4096)
    torch.cuda.synchronize()
    # 70 + 130 steps: the resumed leg follows the full solve's grid
    assert (s2.stats["num_steps"].cpu().numpy() == 130).all()
    assert (s2.controller_state[0].cpu().numpy() == 201).all()
    a, b = s2.ys[:, -1].double().cpu().numpy(), full.ys[:, -1].double().cpu().numpy()
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    assert np.abs(a - b).max() / np.abs(b).max() < tol
    r2 = _oracle(field, solver, ctrl, sa2, D, dtype, 4096, t0=t_m.cpu().numpy(), t1=20.0,
                 dt0=0.1, y0=y_m.double().cpu().numpy(), args=lv, state_in=rec1)
    err = np.abs(s2.ys.double().cpu().numpy() - r2["ys"]).max() / np.abs(r2["ys"]).max()
    assert err < (1e-12 if dtype == torch.float64 else 1e-5)
    assert np.array_equal(_record(s2)[:, :2], r2["state"][:, :2])


def test_states_alone_save_no_ys_and_unsupported_forms_raise():
    dev = torch.device("cuda")
    y0 = torch.ones((4, 2), dtype=torch.float64, device=dev)
    mu = torch.ones((1,), dtype=torch.float64, device=dev)
    ctrl = dfx.PIDController(rtol=1e-6, atol=1e-8)
    sol = dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Heun(), 0.0, 1.0, 0.1, y0, mu,
                          saveat=dfx.SaveAt(controller_state=True, solver_state=True),
                          stepsize_controller=ctrl)
    assert sol.ys is None and sol.ts is None
    assert sol.solver_state is None  # Heun keeps no FSAL value
    assert len(sol.controller_state) == 3
    with pytest.raises(ValueError, match="controller_state must hold 3"):
        dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Heun(), 0.0, 1.0, 0.1, y0, mu,
                        stepsize_controller=ctrl, controller_state=(1.0, 1.0))
    with pytest.raises(ValueError, match="no solver state"):
        dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Heun(), 0.0, 1.0, 0.1, y0, mu,
                        stepsize_controller=ctrl, solver_state=(False, y0))
    clip = dfx.ClipStepSizeController(ctrl, step_ts=[0.5])
    with pytest.raises(NotImplementedError, match="ClipStepSizeController"):
        dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Heun(), 0.0, 1.0, 0.1, y0, mu,
                        stepsize_controller=clip, saveat=dfx.SaveAt(t1=True, made_jump=True))


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_mlp_resume_matches_oracle(precision):
    # 64 -> 128 -> 128 -> 64 (BF16 weights), Tsit5 + PID(1e-5, 1e-7): leg 1 on
    # [0, 0.5] saving the states, leg 2 on [0.5, 1] resumed from them, against
    # the oracle resumed from the same records
    from test_gpu_mlp import mlp_params, flat
    dev = torch.device("cuda")
    rng = np.random.default_rng(61)
    B, D = 128, 64
    y0 = rng.standard_normal((B, D))
    Ws, bs = mlp_params([64, 128, 128, 64], 13, bias_scale=0.1)
    Ws = [W.astype(np.float32).astype(np.float64) for W in Ws]
    bs = [b.astype(np.float32).astype(np.float64) for b in bs]
    field = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                         [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs],
                         precision=precision)
    ctrl = dfx.PIDController(rtol=1e-5, atol=1e-7)
    sa = dfx.SaveAt(t1=True, **STATES)
    s1 = dfx.diffeqsolve(dfx.ODETerm(field), dfx.Tsit5(), 0.0, 0.5, 0.05,
                         torch.tensor(y0, dtype=torch.float32, device=dev), saveat=sa,
                         stepsize_controller=ctrl)
    rec1 = _record(s1)
    assert (rec1[:, 4] == 1).all() and (rec1[:, 5] == 0).all()  # states and an FSAL value
    s2 = dfx.diffeqsolve(dfx.ODETerm(field), dfx.Tsit5(), 0.5, 1.0, 0.05, s1.ys[:, -1],
                         saveat=sa, stepsize_controller=ctrl, solver_state=s1.solver_state,
                         controller_state=s1.controller_state, made_jump=s1.made_jump)
    torch.cuda.synchronize()
    fields = dfx.lower(dfx.ODETerm(field), dfx.Tsit5(), ctrl, sa, dim=D, dtype=torch.float32,
                       max_steps=4096, n_ts=0)
    d = O.make_desc(**O.oracle_fields(fields))
    r2 = O.solve(d, 0.5, 1.0, 0.05, s1.ys[:, -1].double().cpu().numpy(),
                 params=flat(Ws, bs), state_in=rec1, want_state=True, nthreads=8)
    ys = s2.ys.double().cpu().numpy()
    err = np.abs(ys - r2["ys"]).max() / np.abs(r2["ys"]).max()
    print(f"MLP resume {precision}: max rel err {err:.2e}")
    assert err < 2e-5
    # the FSAL value in the record is the field at the final state
    rec2 = _record(s2)
    f_end = rec2[:, 7:]
    fr = r2["state"][:, 7:]
    assert np.abs(f_end - fr).max() < 1e-4 * np.abs(fr).max()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_split_equals_whole_on_the_gpu(dtype):
    # the GPU form of the oracle pin: a PID solve stopped after k attempted
    # steps and resumed from its records (dt0 = the whole solve's next step)
    # takes the whole solve's remaining steps bit for bit
    dev = torch.device("cuda")
    y0 = torch.tensor([[1.2, -0.3], [-0.8, 0.6]], dtype=dtype, device=dev)
    mu = torch.tensor([1.5], dtype=dtype, device=dev)
    ctrl = dfx.PIDController(rtol=1e-6, atol=1e-8)
    term = dfx.ODETerm(dfx.VanDerPol())

    def run(t0, dt0, y, k, **kw):
        return dfx.diffeqsolve(term, dfx.Tsit5(), t0, 3.0, dt0, y, mu,
                               saveat=dfx.SaveAt(steps=1, **STATES), stepsize_controller=ctrl,
                               max_steps=k, throw=False, **kw)
    whole = run(0.0, 0.05, y0, 4096)
    acc = [run(0.0, 0.05, y0, k).stats["num_accepted_steps"].cpu().numpy() for k in range(1, 41)]
    k = next(k for k in range(10, 40)
             if (acc[k - 1] == acc[k - 2] + 1).all() and (acc[k] == acc[k - 1] + 1).all())
    leg1 = run(0.0, 0.05, y0, k)
    ka = leg1.stats["num_accepted_steps"].cpu().numpy().astype(np.int64)  # per trajectory
    rows = torch.arange(2, device=dev)
    kk = torch.tensor(ka, device=dev)
    wts = whole.ts
    tk = wts[rows, kk - 1].contiguous()
    assert torch.equal(leg1.ts[rows, kk - 1], tk)
    leg2 = run(tk, (wts[rows, kk] - tk).contiguous(), leg1.ys[rows, kk - 1].contiguous(), 4096,
               solver_state=leg1.solver_state, controller_state=leg1.controller_state,
               made_jump=leg1.made_jump)
    n = whole.stats["num_accepted_steps"].cpu().numpy()
    if dtype == torch.float64:
        for b in range(2):
            m = int(n[b] - ka[b])
            assert int(leg2.stats["num_accepted_steps"][b]) == m
            assert torch.equal(leg2.ts[b, :m], wts[b, ka[b]:n[b]])
            assert torch.equal(leg2.ys[b, :m], whole.ys[b, ka[b]:n[b]])
        assert np.array_equal(_record(leg2), _record(whole))
    else:
        # the FP32 kernels carry the controller's step size instead of
        # re-forming it from the step's times, so the resumed leg's first
        # step size can differ from the whole solve's in its last bits
        m2 = leg2.stats["num_accepted_steps"].cpu().numpy()
        assert (np.abs(m2 - (n - ka)) <= 1).all()
        rows = torch.arange(2, device=dev)
        last2 = leg2.ys[torch.arange(2, device=dev), torch.tensor(m2 - 1, device=dev)]
        lastw = whole.ys[torch.arange(2, device=dev), torch.tensor(n - 1, device=dev)]
        assert float((last2 - lastw).abs().max()) < 1e-5 * float(lastw.abs().max())
