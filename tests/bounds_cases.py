"""Solves run under both the release library and the bounds-checked one
(libgbdx_bounds.so, GBDX_BOUNDS=1): every kernel family and extended output,
on small seeded inputs.  ``run_cases()`` returns the outputs by name; run as a
script it writes them to the .npz file named on the command line (the
bounds-checked library is chosen per process, so the bounds-checked side runs
in a child process)."""
import sys

import numpy as np
import torch

import diffrax_gb300 as dfx


# outputs summed across trajectories in work-stealing order (not bitwise
# reproducible from run to run)
REDUCED = ("mlp_rc_dW1", "mlp_bs_dW1")


def _bf16(a):
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).float()


def _mlp(widths, seed, dev, grad=False):
    g = np.random.default_rng(seed)
    Ws = [_bf16(g.standard_normal((widths[i + 1], widths[i])) / np.sqrt(widths[i])).to(dev)
          for i in range(len(widths) - 1)]
    bs = [torch.tensor(g.standard_normal(widths[i + 1]) * 0.1, dtype=torch.float32,
                       device=dev) for i in range(len(widths) - 1)]
    if grad:
        for t in Ws + bs:
            t.requires_grad_(True)
    return Ws, bs


def run_cases():
    dev = torch.device("cuda")
    out = {}
    g = np.random.default_rng(11)
    B = 512
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    vdp = dfx.ODETerm(dfx.VanDerPol())
    y0 = torch.tensor(g.uniform(-2, 2, (B, 2)), dtype=torch.float32, device=dev)
    mu = torch.tensor(g.uniform(0.5, 2.0, (B, 1)), dtype=torch.float32, device=dev)
    t1 = torch.tensor(g.uniform(2.0, 8.0, B), dtype=torch.float64, device=dev)
    ts = np.linspace(0.0, 2.0, 9)
    # K1 fused and K0 plain, FP32 and FP64, SaveAt(t0, ts, t1)
    for kern in ("fused", "plain"):
        for dt in (torch.float32, torch.float64):
            sol = dfx.diffeqsolve(vdp, dfx.Dopri5(), 0.0, t1, None, y0.to(dt), mu.to(dt),
                                  saveat=dfx.SaveAt(t0=True, ts=ts, t1=True),
                                  stepsize_controller=pid, kernel=kern, throw=False)
            out[f"vdp_{kern}_{dt}"] = sol.ys
    # the extended outputs: steps, dense, clip, event, resume records
    sol = dfx.diffeqsolve(vdp, dfx.Tsit5(), 0.0, 4.0, None, y0, mu[:1].reshape(1),
                          saveat=dfx.SaveAt(steps=2, t1=True, dense=True),
                          stepsize_controller=pid, max_steps=512, throw=False)
    out["xo_steps"] = sol.ys
    out["xo_dense"] = sol.evaluate(torch.linspace(0.0, 4.0, 17, dtype=torch.float64,
                                                  device=dev))
    clip = dfx.ClipStepSizeController(pid, step_ts=np.linspace(0.5, 3.5, 7), jump_ts=[2.25])
    out["xo_clip"] = dfx.diffeqsolve(vdp, dfx.Dopri5(), 0.0, 4.0, None, y0,
                                     mu[:1].reshape(1), stepsize_controller=clip,
                                     throw=False).ys
    ev = dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-5, 1e-5), direction=True)
    sol = dfx.diffeqsolve(vdp, dfx.Dopri5(), 0.0, 8.0, None, y0, mu[:1].reshape(1),
                          stepsize_controller=pid, event=ev, throw=False)
    out["xo_event"] = sol.ys
    sol = dfx.diffeqsolve(vdp, dfx.Dopri5(), 0.0, 2.0, 0.05, y0, mu,
                          saveat=dfx.SaveAt(t1=True, solver_state=True, controller_state=True,
                                            made_jump=True), stepsize_controller=pid)
    out["resume_leg1"] = sol.lowered.state_record
    sol = dfx.diffeqsolve(vdp, dfx.Dopri5(), 2.0, 4.0, 0.05, sol.ys[:, -1], mu,
                          stepsize_controller=pid, solver_state=sol.solver_state,
                          controller_state=sol.controller_state, made_jump=sol.made_jump)
    out["resume_leg2"] = sol.ys
    # analytic-field adjoints (gradients with respect to y0 and args)
    lv = dfx.ODETerm(dfx.LotkaVolterra())
    y0l = torch.tensor(g.uniform(5, 15, (64, 2)), dtype=torch.float64, device=dev)
    for name, adj in (("rc", dfx.RecursiveCheckpointAdjoint()),
                      ("bs", dfx.BacksolveAdjoint())):
        yg = y0l.clone().requires_grad_(True)
        ag = torch.tensor([0.1, 0.02, 0.4, 0.02], dtype=torch.float64, device=dev,
                          requires_grad=True)
        sol = dfx.diffeqsolve(lv, dfx.Tsit5(), 0.0, 10.0, 0.1, yg, ag,
                              saveat=dfx.SaveAt(ts=np.linspace(0, 10, 5)),
                              stepsize_controller=dfx.PIDController(rtol=1e-8, atol=1e-8),
                              adjoint=adj)
        sol.ys.square().sum().backward()
        out[f"lv_{name}_dy0"], out[f"lv_{name}_dargs"] = yg.grad, ag.grad
    # MLP fields: K2 forward, K5 tcgen05 forward, K3 and K4 gradients, the SDE
    Bm = 256
    ym = torch.tensor(g.standard_normal((Bm, 64)), dtype=torch.float32, device=dev)
    pidm = dfx.PIDController(rtol=1e-5, atol=1e-7)
    Ws, bs = _mlp([64, 128, 128, 64], 1, dev)
    for kern in ("fused", "tc"):
        sol = dfx.diffeqsolve(dfx.ODETerm(dfx.MLPField(Ws, bs)), dfx.Tsit5(), 0.0, 1.0, None,
                              ym, saveat=dfx.SaveAt(t0=True, ts=[0.25, 0.5], t1=True),
                              stepsize_controller=pidm, kernel=kern)
        out[f"mlp_{kern}"] = sol.ys
    for name, adj in (("rc", dfx.RecursiveCheckpointAdjoint(checkpoints=8)),
                      ("bs", dfx.BacksolveAdjoint())):
        Wg, bg = _mlp([64, 128, 128, 64], 2, dev, grad=True)
        yg = ym.clone().requires_grad_(True)
        sol = dfx.diffeqsolve(dfx.ODETerm(dfx.MLPField(Wg, bg)), dfx.Tsit5(), 0.0, 1.0, None,
                              yg, saveat=dfx.SaveAt(ts=[0.5, 1.0]), stepsize_controller=pidm,
                              adjoint=adj)
        sol.ys.square().sum().backward()
        out[f"mlp_{name}_dy0"], out[f"mlp_{name}_dW1"] = yg.grad, Wg[1].grad
    Wd, bd = _mlp([32, 64, 64, 32], 3, dev)
    Wsig, bsig = _mlp([32, 32], 4, dev)
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (32,), key=5)
    terms = dfx.MultiTerm(dfx.ODETerm(dfx.MLPField(Wd, bd)),
                          dfx.ControlTerm(dfx.TanhDiagonalDiffusion(Wsig[0], bsig[0]), bm))
    ys = torch.tensor(g.standard_normal((Bm, 32)), dtype=torch.float32, device=dev)
    out["nsde"] = dfx.diffeqsolve(terms, dfx.Heun(), 0.0, 1.0, 0.05, ys).ys
    torch.cuda.synchronize()
    return {k: v.detach().cpu().numpy() for k, v in out.items()}


if __name__ == "__main__":
    np.savez(sys.argv[1], **run_cases())
