#!/usr/bin/env python
"""Benchmark of the batched diffeqsolve hot path on GB300.

Workload (the uneven-batching configuration): Van der Pol x' = y,
y' = mu (1 - x^2) y - x with mu ~ LogUniform[0.1, 10], (x0, y0) ~ U[-2, 2]^2,
per-trajectory t1 ~ U[5, 50], batch 65536 per GPU; Dopri5 with
PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4), dt0=None,
SaveAt(t1=True); FP32 state with FP64 t/dt; one persistent launch captured as a
CUDA graph.  Inputs are seeded synthetic draws of exactly that distribution.

One step = one solve of the whole batch.  `value` is trajectories/s with
inputs resident in HBM (fused kernel K1); `e2e` is the same metric through the
public API for a repeated solve, GraphedSolve(host_io=True) (one solve captured
as a CUDA graph, the counterpart of a jitted diffeqsolve; its kernels read the
page-locked host inputs and write the results into page-locked host memory in
place over NVLink-C2C -- or, where the GPU does not map them, the graph copies
them in and out) every step; `e2e_eager` the same through a fresh
diffeqsolve call every step.  The plain one-trajectory-per-thread kernel K0 is timed the
same way and reported beside it, together with the max relative error of both
against the FP64 oracle and the oracle's own throughput on the host cores.

`--impl reference` times the reference path's CPU implementation -- the FP64
oracle restatement of Diffrax's loop (the reference itself is JAX and cannot
be installed here) -- on all host cores, on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "trajectories/s (Van der Pol, Dopri5+PID rtol 1e-6, uneven t1, batch 65536)"
UNIT = "trajectories/s"
WORKLOAD = "vdp_dopri5_pid_uneven_t1_b65536"
# Algorithmic work per attempted Dopri5 step on Van der Pol (d = 2), counting
# an FMA as 2 flops: 6 field evaluations x 5, 7 stage scalings x 2, 20
# nonzero stage coefficients x 2 dims x 2 + 12 adds, 6 error terms x 2 x 2,
# and ~26 for the scaled RMS norm and PID factor.
FP32_FLOPS_PER_STEP = 6 * 5 + 14 + 92 + 24 + 26
FP64_OPS_PER_STEP = 6      # dt, t + dt, dt * factor, clip compare, loop compare, min
BYTES_PER_TRAJ = 8 + 4 + 8 + 8 + 8 + 4 + 12  # y0, mu, t1, ys, ts, result, stats
FP32_PEAK_TFLOPS_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12
FP64_PEAK_TFLOPS_NOMINAL = 1.25


def vdp_inputs(B: int, seed: int):
    rng = np.random.default_rng(seed)
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), B))
    y0 = rng.uniform(-2.0, 2.0, (B, 2))
    t1 = rng.uniform(5.0, 50.0, B)
    return mu, y0, t1


def oracle_solve(mu, y0, t1, nthreads):
    import oracle as O
    d = O.make_desc(solver=O.DOPRI5, controller=O.PID, field=O.VAN_DER_POL, dim=2,
                    rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4, save_t1=1, n_args=1)
    return O.solve(d, 0.0, t1, None, y0, args=mu[:, None], nthreads=nthreads)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the fused kernel on this workload, from an ncu capture of the same command
# (bench.py --profile fused); not measured in a bench run (a run under ncu is
# never timed).
NCU_TRAFFIC_BYTES_PER_LAUNCH = 2119936.0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, period_ms: int = 20):
        self.index = index
        self.period_ms = period_ms
        self.proc = None
        self.path = None
        self.first = 0

    def _rows(self):
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        return rows

    def start(self):
        """Starts nvidia-smi and returns once it has written its first sample,
        so that the samples after this call fall inside the timed region."""
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", str(self.period_ms)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        deadline = time.perf_counter() + 10.0
        while time.perf_counter() < deadline and self.proc.poll() is None:
            if self._rows():
                break
            time.sleep(0.005)
        self.first = len(self._rows())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        every = self._rows()
        os.unlink(self.path)
        # the samples written during the timed region; a region shorter than
        # the sampling period keeps the sample nearest its start
        rows = every[self.first:] or every[-1:]
        in_region = len(every) - self.first
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": max(in_region, 0), "period_ms": self.period_ms}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    """CPU implementation of the path (the FP64 oracle restatement) on all host
    cores, `sample` trajectories per step."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = args.ref_sample if args.ref_sample > 0 else args.batch
    mu, y0, t1 = vdp_inputs(args.batch, args.seed)
    mu, y0, t1 = mu[:sample], y0[:sample], t1[:sample]
    for _ in range(args.warmup):
        oracle_solve(mu, y0, t1, cores)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle_solve(mu, y0, t1, cores)
        times.append(time.perf_counter() - t)
    v = sample / statistics.mean(times)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch_per_gpu": args.batch,
                   "batch_per_step": sample,
                   "note": "Diffrax (JAX) is not installable offline; this is the FP64 C "
                           "restatement of its solve loop with OpenMP over trajectories"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{sample} trajectories of the workload per step"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---------------------------------------------------------------------------
# The other configurations, measured beside the headline workload.
# ---------------------------------------------------------------------------

def _events_time(fn, steps, warmup, flush):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return statistics.median(ms)


def _bf16_values(a):
    """The nearest BF16 values of an array, as float32."""
    import torch
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).float().numpy()


def _mlp_np(widths, seed):
    """eqx.nn.MLP-style weights N(0, 1/fan_in) from a seed, held as BF16 values
    (the workloads' BF16 weights: the fused, plain and oracle solves all see
    the same values), zero biases."""
    rng = np.random.default_rng(seed)
    Ws = [_bf16_values(rng.standard_normal((widths[i + 1], widths[i])) / np.sqrt(widths[i]))
          for i in range(len(widths) - 1)]
    bs = [np.zeros(widths[i + 1], np.float32) for i in range(len(widths) - 1)]
    return Ws, bs


def _rel_per_traj(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ax = tuple(range(1, a.ndim))
    return np.abs(a - b).max(axis=ax) / np.abs(b).max(axis=ax)


def _oracle_rate(fn, n, cores):
    t = time.perf_counter()
    fn()
    dt = time.perf_counter() - t
    return {"value": n / dt, "cores": cores, "kind": "port",
            "sample": f"{n} trajectories, FP64 oracle, {dt:.2f} s"}


def workload_lotka_volterra(dev, flush, steps, warmup):
    """Lotka-Volterra, Tsit5 + PID(1e-6, 1e-8), batch 1024, 100 ts on [0, 140]."""
    import torch
    import diffrax_gb300 as dfx
    import oracle as O
    from diffrax_gb300._integrate import Lowered
    B = 1024
    rng = np.random.default_rng(11)
    y0 = rng.uniform(5, 15, (B, 2))
    ts = np.linspace(0.0, 140.0, 100)
    args = np.array([0.1, 0.02, 0.4, 0.02])
    pid = dfx.PIDController(rtol=1e-6, atol=1e-8)
    out = {"workload": "lotka_volterra_tsit5_pid_b1024_ts100"}
    ref = O.solve(O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.LOTKA_VOLTERRA,
                              dim=2, rtol=1e-6, atol=1e-8, n_ts=100, save_t1=0, n_args=4),
                  0.0, 140.0, 0.1, y0, args=args, ts=ts, nthreads=os.cpu_count() or 1)
    for dt_name, dtype in (("f32", torch.float32), ("f64", torch.float64)):
        for kern in ("fused", "plain"):
            low = Lowered(dfx.ODETerm(dfx.LotkaVolterra()), dfx.Tsit5(), 0.0, 140.0, 0.1,
                          torch.tensor(y0, dtype=dtype, device=dev),
                          torch.tensor(args, dtype=dtype, device=dev), dfx.SaveAt(ts=ts), pid,
                          None, 4096, kern, 0, 0)
            ms = _events_time(low.run_forward, steps, warmup, flush)
            ys = low.run_forward()[0].double().cpu().numpy()
            e = _rel_per_traj(ys, ref["ys"])
            out[f"{kern}_{dt_name}"] = {"traj_per_s": B / (ms / 1e3), "ms": ms,
                                        "max_rel_err_vs_fp64_oracle": float(e.max())}
    out["fused_over_plain_f32"] = out["fused_f32"]["traj_per_s"] / out["plain_f32"]["traj_per_s"]
    cores = os.cpu_count() or 1
    out["cpu_baseline"] = _oracle_rate(lambda: O.solve(
        O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.LOTKA_VOLTERRA, dim=2, rtol=1e-6,
                    atol=1e-8, n_ts=100, save_t1=0, n_args=4),
        0.0, 140.0, 0.1, y0, args=args, ts=ts, nthreads=cores), B, cores)
    return out


def profile_backsolve(dev, B, seminorm, n):
    """n forward + BacksolveAdjoint backward solves of the wide neural ODE
    (64-256-256-64, Tsit5 PID(1e-5, 1e-7), 32 ts) at batch B, for ncu."""
    import torch
    import diffrax_gb300 as dfx
    from diffrax_gb300._integrate import Lowered
    widths = [64, 256, 256, 64]
    Ws, bs = _mlp_np(widths, 22)
    y0 = np.random.default_rng(23).standard_normal((B, 64)).astype(np.float32)
    field = dfx.MLPField([torch.tensor(W, device=dev) for W in Ws],
                         [torch.tensor(b, device=dev) for b in bs])
    ctrl = dfx.PIDController(rtol=1e-5, atol=1e-7)
    adj = dfx.BacksolveAdjoint(stepsize_controller=dfx.PIDController(
        rtol=1e-5, atol=1e-7, norm=dfx.adjoint_rms_seminorm)) if seminorm else \
        dfx.BacksolveAdjoint()
    low = Lowered(dfx.ODETerm(field), dfx.Tsit5(), 0.0, 1.0, None,
                  torch.tensor(y0, device=dev), None, dfx.SaveAt(ts=np.linspace(0, 1, 32)),
                  ctrl, adj, 4096, "fused", 0, 0, want_grad=True)
    for _ in range(n):
        ys, ts, res, _ = low.run_forward()
        _, _, bres, _ = low.run_backsolve(ts, ys, ys * (2.0 / ys.numel()), low.params)
    torch.cuda.synchronize()
    ok = bool((res == 0).all().item()) and bool((bres == 0).all().item())
    print(json.dumps({"profile": "backsolve", "seminorm": seminorm, "solves": n,
                      "all_successful": ok}))
    if not ok:
        sys.exit(1)


def profile_saveat_steps(dev, n):
    """`--profile saveat_steps`: n rounds of the SaveAt(t1) and the
    SaveAt(steps=3) solves of the Van der Pol rows of workload_next_rows
    (batch 16384, t in [0, 10]), alternating, for a launch-by-launch
    comparison of the plain and the extended-output fused kernels."""
    import torch
    import diffrax_gb300 as dfx
    from diffrax_gb300._integrate import Lowered
    B = 16384
    rng = np.random.default_rng(7)
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), B))
    y0 = rng.uniform(-2, 2, (B, 2))
    y0_d = torch.tensor(y0, dtype=torch.float32, device=dev)
    mu_d = torch.tensor(mu[:, None], dtype=torch.float32, device=dev)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    lows = [Lowered(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(), 0.0, 10.0, None, y0_d, mu_d,
                    sa, pid, None, 1024, "fused", 0, 0)
            for sa in (dfx.SaveAt(t1=True), dfx.SaveAt(steps=3, t1=True))]
    ok = True
    for _ in range(n):
        for low in lows:
            ok = ok and bool((low.run_forward()[2] == 0).all().item())
    torch.cuda.synchronize()
    print(json.dumps({"profile": "saveat_steps", "rounds": n, "all_successful": ok}))
    if not ok:
        sys.exit(1)


def profile_neural(dev, which, B, n):
    """n fused solves of a neural workload at batch B, for ncu: the forward of
    the neural ODE (64-128-128-64, row-tile or tcgen05 kernel), its forward +
    RecursiveCheckpointAdjoint backward, the wide neural ODE forward, or the
    neural SDE forward (and its forward + RecursiveCheckpointAdjoint
    backward)."""
    import torch
    import diffrax_gb300 as dfx
    from diffrax_gb300._integrate import Lowered
    wide, sde = which == "neural_ode_wide", which in ("neural_sde", "neural_sde_grad")
    widths = [64, 256, 256, 64] if wide else ([32, 64, 64, 32] if sde else [64, 128, 128, 64])
    D = widths[0]
    Ws, bs = _mlp_np(widths, 21)
    y0 = torch.tensor(np.random.default_rng(24).standard_normal((B, D)).astype(np.float32),
                      device=dev)
    field = dfx.MLPField([torch.tensor(W, device=dev) for W in Ws],
                         [torch.tensor(b, device=dev) for b in bs])
    if sde:
        rng = np.random.default_rng(25)
        Wsig = torch.tensor(_bf16_values(rng.standard_normal((D, D)) / np.sqrt(D)), device=dev)
        bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (D,), key=23)
        terms = dfx.MultiTerm(dfx.ODETerm(field), dfx.ControlTerm(
            dfx.TanhDiagonalDiffusion(Wsig, torch.zeros(D, device=dev)), bm))
        solver, ctrl, dt0, saveat = dfx.Heun(), dfx.ConstantStepSize(), 0.01, dfx.SaveAt(t1=True)
    else:
        terms = dfx.ODETerm(field)
        solver, ctrl, dt0 = dfx.Tsit5(), dfx.PIDController(rtol=1e-5, atol=1e-7), None
        saveat = dfx.SaveAt(ts=np.linspace(0, 1, 32)) if wide else dfx.SaveAt(t1=True)
    grad = which in ("neural_ode_grad", "neural_sde_grad")
    adjoint = dfx.RecursiveCheckpointAdjoint() if sde else \
        dfx.RecursiveCheckpointAdjoint(checkpoints=64)
    low = Lowered(terms, solver, 0.0, 1.0, dt0, y0, None, saveat, ctrl, adjoint, 4096,
                  "tc" if which == "neural_ode_tc" else "fused", 0, 0, want_grad=grad)
    for _ in range(n):
        if grad:
            ys, _, res, _, ws = low.run_forward(keep_workspace=True)
            low.run_backward(ws, ys * (2.0 / ys.numel()), low.y0, low.params)
        else:
            ys, _, res, _ = low.run_forward()
    torch.cuda.synchronize()
    ok = bool((res == 0).all().item())
    print(json.dumps({"profile": which, "solves": n, "all_successful": ok}))
    if not ok:
        sys.exit(1)


RESULT_NAMES_BENCH = {0: "successful", 1: "max_steps_reached", 2: "dt_min_reached",
                      3: "event_occurred", 4: "max_steps_rejected", 5: "internal_error",
                      6: "nonlinear_max_steps_reached"}


def workload_next_rows(dev, flush, steps, warmup):
    """The solve features beyond the headline path, each timed on the device
    (CUDA events, L2 flushed) beside the same solve without it, with its
    parity against the FP64 oracle on the first 256 trajectories.

    ODE rows: Van der Pol, Dopri5 + PID(1e-6, 1e-9, p=.3, i=.4), mu ~
    LogU[0.1, 10], (x0, y0) ~ U[-2, 2]^2, t in [0, 10], batch 16384, FP32
    state, max_steps 1024: SaveAt(steps=3), SaveAt(dense=True) (+ evaluation
    at 64 times), ClipStepSizeController(step_ts = 101-point grid, jump_ts =
    2.5, 5, 7.5), Event(x crosses 0 upwards, Newton(1e-5, 1e-5) root), Dopri8.
    SDE rows: Ornstein-Uhlenbeck dim 2 (theta 1.5, mu 0.5, sigma 0.6) on
    [0, 1], dt 0.01, tree tol 1e-3, batch 16384: Heun on the W-only tree,
    Heun / ShARK / SRA1 / SEA on the space-time Levy area tree.
    MLP rows: the neural-ODE field (64 -> 128 -> 128 -> 64), Tsit5 + PID(1e-5,
    1e-7), batch 8192: SaveAt(steps=1), SaveAt(dense=True), the clip
    controller, a linear event with Newton root finding (final values against
    the oracle on 64 trajectories)."""
    import torch
    import diffrax_gb300 as dfx
    import oracle as O
    from diffrax_gb300._integrate import Lowered
    B, n_chk, t1 = 16384, 256, 10.0
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(7)
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), B))
    y0 = rng.uniform(-2, 2, (B, 2))
    y0_d = torch.tensor(y0, dtype=torch.float32, device=dev)
    mu_d = torch.tensor(mu[:, None], dtype=torch.float32, device=dev)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    term = dfx.ODETerm(dfx.VanDerPol())
    out = {"workload": "vdp_dopri5_pid_t10_b16384, ou_sde_dt0.01_b16384 and "
                       "neural_ode_64_128_b8192",
           "ode": {}, "sde": {}}

    def ode_row(solver, saveat, ctrl, event=None):
        low = Lowered(term, solver, 0.0, t1, None, y0_d, mu_d, saveat, ctrl, None, 1024,
                      "fused", 0, 0, event=event)
        ex = saveat.dense or event is not None
        run = low.run_forward_ex if ex else low.run_forward
        ms = _events_time(run, steps, warmup, flush)
        outs = run()
        ts_ = np.asarray(saveat.ts) if saveat.ts is not None else None
        d = O.make_desc(**O.oracle_fields(low.fields))
        kw = {}
        if isinstance(ctrl, dfx.ClipStepSizeController):
            kw = dict(step_ts=ctrl.step_ts, jump_ts=ctrl.jump_ts)
        r = O.solve(d, 0.0, t1, None, y0[:n_chk], args=mu[:n_chk, None], ts=ts_,
                    nthreads=cores, **kw)
        res = outs[2].cpu().numpy()
        codes, counts = np.unique(res, return_counts=True)
        row = {"traj_per_s": B / (ms / 1e3), "ms": ms,
               "mean_attempted_steps": float(outs[3][:, 0].float().mean().item()),
               "results": {RESULT_NAMES_BENCH.get(int(c), str(c)): int(n)
                           for c, n in zip(codes, counts)}}
        # the final value (the last written save: saves are compacted and the
        # slots after them hold inf) against the oracle's
        def final(ys_, ts_):
            k = np.isfinite(ts_).sum(axis=1) - 1
            return ys_[np.arange(ys_.shape[0]), k]
        last = final(outs[0][:n_chk].double().cpu().numpy(), outs[1][:n_chk].cpu().numpy())
        ref_last = final(r["ys"], r["ts"])
        e = np.abs(last - ref_last).max(axis=1) / np.abs(ref_last).max()
        row["t1_rel_err_vs_fp64_oracle"] = {"median": float(np.median(e)), "max": float(e.max())}
        return low, outs, r, row

    base = ode_row(dfx.Dopri5(), dfx.SaveAt(t1=True), pid)[3]
    out["ode"]["base_saveat_t1"] = base
    for name, solver, saveat, ctrl, event in (
            ("saveat_steps3", dfx.Dopri5(), dfx.SaveAt(steps=3, t1=True), pid, None),
            ("saveat_dense", dfx.Dopri5(), dfx.SaveAt(dense=True, t1=True), pid, None),
            ("clip_controller", dfx.Dopri5(), dfx.SaveAt(t1=True),
             dfx.ClipStepSizeController(pid, step_ts=np.linspace(0.0, t1, 101),
                                        jump_ts=np.array([2.5, 5.0, 7.5])), None),
            ("event_x_up_newton", dfx.Dopri5(), dfx.SaveAt(t1=True), pid,
             dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-5, 1e-5),
                       direction=True)),
            ("dopri8", dfx.Dopri8(), dfx.SaveAt(t1=True), pid, None)):
        low, outs, r, row = ode_row(solver, saveat, ctrl, event)
        row["time_over_base"] = row["ms"] / base["ms"]
        if saveat.dense:
            interp = outs[4]
            q = torch.linspace(0.0, t1, 64, dtype=torch.float64, device=dev)
            ms_q = _events_time(lambda: interp.evaluate(q), steps, warmup, flush)
            yq = interp.evaluate(q)[:n_chk].double().cpu().numpy()
            d = O.make_desc(**O.oracle_fields(low.fields))
            rq = O.dense_evaluate(d, 0.0, t1, y0[:n_chk], r, q.cpu().numpy())
            eq = np.abs(yq - rq).max(axis=(1, 2)) / np.abs(rq).max()
            row["dense_bytes"] = int(outs[4].infos.numel() * outs[4].infos.element_size())
            row["evaluate_64_times"] = {
                "ms": ms_q, "rel_err_vs_fp64_oracle": {"median": float(np.median(eq)),
                                                       "max": float(eq.max())}}
        if event is not None:
            ev = outs[5][:n_chk].cpu().numpy()
            row["event_fired_frac"] = float((outs[5] >= 0).float().mean().item())
            row["event_index_agrees_with_oracle"] = float((ev == r["event_index"]).mean())
            tg = outs[1][:n_chk, -1].cpu().numpy()
            row["event_time_abs_diff"] = {"median": float(np.median(np.abs(tg - r["ts"][:, -1]))),
                                          "max": float(np.abs(tg - r["ts"][:, -1]).max())}
        out["ode"][name] = row

    # SDE rows
    ys0 = rng.uniform(-2, 2, (B, 2))
    ys0_d = torch.tensor(ys0, dtype=torch.float32, device=dev)
    sargs = np.array([1.5, 0.5, 0.6])
    sargs_d = torch.tensor(sargs, dtype=torch.float32, device=dev)
    sde_base = None
    for name, solver, levy in (("heun_w_tree", dfx.Heun(), dfx.BrownianIncrement),
                               ("heun_levy_tree", dfx.Heun(), dfx.SpaceTimeLevyArea),
                               ("shark", dfx.ShARK(), dfx.SpaceTimeLevyArea),
                               ("sra1", dfx.SRA1(), dfx.SpaceTimeLevyArea),
                               ("sea", dfx.SEA(), dfx.SpaceTimeLevyArea)):
        bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), key=5, levy_area=levy)
        terms = dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                              dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))
        low = Lowered(terms, solver, 0.0, 1.0, 0.01, ys0_d, sargs_d, dfx.SaveAt(t1=True),
                      dfx.ConstantStepSize(), None, 4096, "fused", 0, 0)
        ms = _events_time(low.run_forward, steps, warmup, flush)
        ys_ = low.run_forward()[0][:n_chk, 0].double().cpu().numpy()
        r = O.solve(O.make_desc(**O.oracle_fields(low.fields)), 0.0, 1.0, 0.01, ys0[:n_chk],
                    args=sargs, nthreads=cores)
        e = np.abs(ys_ - r["ys"][:, 0]).max(axis=1) / np.abs(r["ys"][:, 0]).max()
        row = {"traj_per_s": B / (ms / 1e3), "ms": ms,
               "t1_rel_err_vs_fp64_oracle": {"median": float(np.median(e)), "max": float(e.max())},
               "steps": 100}
        if sde_base is None:
            sde_base = ms
        row["time_over_heun_w_tree"] = ms / sde_base
        out["sde"][name] = row

    # MLP rows: the neural-ODE field 64 -> 128 -> 128 -> 64 (BF16 weights,
    # three-piece operands), Tsit5 + PID(1e-5, 1e-7) on [0, 1], batch 8192
    Bm, n_m = 8192, 64
    Ws, bs = _mlp_np([64, 128, 128, 64], 21)
    field = dfx.MLPField([torch.tensor(W, dtype=torch.float32, device=dev) for W in Ws],
                         [torch.tensor(b, dtype=torch.float32, device=dev) for b in bs])
    params = np.concatenate([np.concatenate([W.reshape(-1), b]) for W, b in zip(Ws, bs)])
    ym = rng.standard_normal((Bm, 64)).astype(np.float32).astype(np.float64)
    ym_d = torch.tensor(ym, dtype=torch.float32, device=dev)
    pidm = dfx.PIDController(rtol=1e-5, atol=1e-7)
    mterm = dfx.ODETerm(field)
    out["mlp"] = {"workload": "neural_ode_64_128_tsit5_pid_b8192"}
    mbase = None
    for name, saveat, ctrl, event in (
            ("base_saveat_t1", dfx.SaveAt(t1=True), pidm, None),
            ("saveat_steps1", dfx.SaveAt(steps=1, t1=True), pidm, None),
            ("saveat_dense", dfx.SaveAt(dense=True, t1=True), pidm, None),
            ("clip_controller", dfx.SaveAt(t1=True),
             dfx.ClipStepSizeController(pidm, step_ts=np.linspace(0.0, 1.0, 11),
                                        jump_ts=np.array([0.5])), None),
            ("event_linear_newton", dfx.SaveAt(t1=True), pidm,
             dfx.Event(dfx.LinearCondition([1.0, 0.5], offset=-0.25),
                       dfx.Newton(1e-5, 1e-5)))):
        low = Lowered(mterm, dfx.Tsit5(), 0.0, 1.0, None, ym_d, None, saveat, ctrl, None, 256,
                      "fused", 0, 0, event=event)
        ex = saveat.dense or event is not None
        run = low.run_forward_ex if ex else low.run_forward
        ms = _events_time(run, steps, warmup, flush)
        outs = run()
        kw = {}
        if isinstance(ctrl, dfx.ClipStepSizeController):
            kw = dict(step_ts=ctrl.step_ts, jump_ts=ctrl.jump_ts)
        r = O.solve(O.make_desc(**O.oracle_fields(low.fields)), 0.0, 1.0, None, ym[:n_m],
                    params=params, nthreads=cores, **kw)
        k = np.isfinite(outs[1][:n_m].cpu().numpy()).sum(axis=1) - 1
        last = outs[0][:n_m].double().cpu().numpy()[np.arange(n_m), k]
        kr = np.isfinite(r["ts"]).sum(axis=1) - 1
        ref = r["ys"][np.arange(n_m), kr]
        e = np.abs(last - ref).max(axis=1) / np.abs(ref).max()
        row = {"traj_per_s": Bm / (ms / 1e3), "ms": ms,
               "mean_attempted_steps": float(outs[3][:, 0].float().mean().item()),
               "final_rel_err_vs_fp64_oracle": {"median": float(np.median(e)),
                                                "max": float(e.max())}}
        if mbase is None:
            mbase = ms
        row["time_over_base"] = ms / mbase
        if event is not None:
            row["event_fired_frac"] = float((outs[5] >= 0).float().mean().item())
            row["event_index_agrees_with_oracle"] = float(
                (outs[5][:n_m].cpu().numpy() == r["event_index"]).mean())
        out["mlp"][name] = row
    return out


def workload_analytic_grads(dev, flush, steps, warmup):
    """Gradients of the analytic fields, forward + backward timed on the
    device, errors (per trajectory, relative to the batch's largest gradient)
    against the FP64 oracle's gradients on 256 trajectories; loss = sum of
    y(t1)^2, gradients with respect to y0 and the per-trajectory args.

    vdp: the uneven Van der Pol batch (mu ~ LogU[0.1, 10], (x0, y0) ~
    U[-2, 2]^2, t1 ~ U[5, 50], Dopri5 + PID(1e-6, 1e-9, p=.3, i=.4), B =
    65 536, FP32 state) through RecursiveCheckpointAdjoint (the full step
    tape), fused and plain forms.  BacksolveAdjoint is not run on it: the
    Van der Pol limit cycle attracts forward in time and repels backward, so
    the reverse solve of y diverges over these horizons (in the oracle too).
    lv: Lotka-Volterra (args 0.1, 0.02, 0.4, 0.02 x U[0.8, 1.2] per
    trajectory, y0 ~ U[5, 15]^2, t in [0, 20], Tsit5 + PID(1e-6, 1e-8), B =
    65 536, FP32 state) through both adjoints."""
    import torch
    import diffrax_gb300 as dfx
    import oracle as O
    from diffrax_gb300._integrate import Lowered
    B, n_chk = 65536, 256
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(2024)
    cases = {}
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), B))
    cases["vdp"] = dict(term=dfx.ODETerm(dfx.VanDerPol()), solver=dfx.Dopri5(),
                        ctrl=dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4),
                        y0=rng.uniform(-2, 2, (B, 2)), args=mu[:, None],
                        t1=rng.uniform(5.0, 50.0, B),
                        rows=(("recursive_fused", dfx.RecursiveCheckpointAdjoint(), "fused"),
                              ("recursive_plain", dfx.RecursiveCheckpointAdjoint(), "plain")))
    lv = np.array([0.1, 0.02, 0.4, 0.02])
    cases["lv"] = dict(term=dfx.ODETerm(dfx.LotkaVolterra()), solver=dfx.Tsit5(),
                       ctrl=dfx.PIDController(rtol=1e-6, atol=1e-8),
                       y0=rng.uniform(5, 15, (B, 2)), args=lv * rng.uniform(0.8, 1.2, (B, 4)),
                       t1=np.full(B, 20.0),
                       rows=(("recursive_fused", dfx.RecursiveCheckpointAdjoint(), "fused"),
                             ("backsolve_fused", dfx.BacksolveAdjoint(), "fused")))
    out = {"workload": "vdp_dopri5_pid_uneven_t1_b65536 and lv_tsit5_pid_t20_b65536, "
                       "loss sum y(t1)^2, gradients wrt y0 and args",
           "unit": "trajectory gradients/s"}
    for cname, c in cases.items():
        y0_d = torch.tensor(c["y0"], dtype=torch.float32, device=dev)
        a_d = torch.tensor(c["args"], dtype=torch.float32, device=dev)
        t1_d = torch.tensor(c["t1"], dtype=torch.float64, device=dev)
        res_c, ref = {}, {}
        for name, adjoint, kernel in c["rows"]:
            low = Lowered(c["term"], c["solver"], 0.0, t1_d, None, y0_d, a_d,
                          dfx.SaveAt(t1=True), c["ctrl"], adjoint, 4096, kernel, 0, 0,
                          want_grad=True)
            backsolve = isinstance(adjoint, dfx.BacksolveAdjoint)

            def step():
                if backsolve:
                    ys, ts_out, _, _ = low.run_forward()
                    return low.run_backsolve_args(ts_out, ys, 2.0 * ys, low.args)
                ys, _, _, _, ws = low.run_forward(keep_workspace=True)
                return low.run_backward_args(ws, 2.0 * ys, low.y0, low.args)
            ms = _events_time(step, steps, warmup, flush)
            ys, ts_out, res, _ = low.run_forward()
            g = step()
            torch.cuda.synchronize()
            kind = "backsolve" if backsolve else "recursive"
            if kind not in ref:
                G = 2.0 * ys[:n_chk].double().cpu().numpy()
                if backsolve:
                    d = O.make_desc(**O.oracle_fields(low.bwd_fields))
                    ref[kind] = O.backsolve(d, 0.0, c["t1"][:n_chk], None,
                                            ts_out[:n_chk].cpu().numpy(),
                                            ys[:n_chk].double().cpu().numpy(), G,
                                            args=c["args"][:n_chk], nthreads=cores)
                else:
                    d = O.make_desc(**O.oracle_fields(low.fields))
                    ref[kind] = O.grad_recursive(d, 0.0, c["t1"][:n_chk], None,
                                                 c["y0"][:n_chk], G, args=c["args"][:n_chk],
                                                 nthreads=cores)
                    # the CPU baseline: the oracle's forward + backward on a
                    # larger sample of the same batch (the library is loaded)
                    n_cpu = 16384
                    Gc = 2.0 * ys[:n_cpu].double().cpu().numpy()
                    t = time.perf_counter()
                    O.grad_recursive(d, 0.0, c["t1"][:n_cpu], None, c["y0"][:n_cpu], Gc,
                                     args=c["args"][:n_cpu], nthreads=cores)
                    ref["cpu_s"] = time.perf_counter() - t
                    ref["cpu_n"] = n_cpu
            r = ref[kind]
            gy = g[0][:n_chk].double().cpu().numpy()
            ga = g[1][:n_chk].double().cpu().numpy()
            ey = np.abs(gy - r["grad_y0"]).max(axis=1) / np.abs(r["grad_y0"]).max()
            ea = np.abs(ga - r["grad_args"]).max(axis=1) / np.abs(r["grad_args"]).max()
            res_c[name] = {"grads_per_s": B / (ms / 1e3), "ms": ms,
                           "all_successful": bool((res == 0).all().item()),
                           "dL_dy0_rel_err_vs_fp64_oracle": {"median": float(np.median(ey)),
                                                             "max": float(ey.max())},
                           "dL_dargs_rel_err_vs_fp64_oracle": {"median": float(np.median(ea)),
                                                               "max": float(ea.max())}}
        res_c["cpu_baseline"] = {"value": ref["cpu_n"] / ref["cpu_s"],
                                 "unit": "trajectory gradients/s", "cores": cores,
                                 "kind": "port",
                                 "sample": f"{ref['cpu_n']} trajectories forward + recursive "
                                           f"backward, FP64 oracle, {ref['cpu_s']:.2f} s"}
        out[cname] = res_c
    v = out["vdp"]
    v["recursive_fused_over_plain"] = (v["recursive_fused"]["grads_per_s"] /
                                       v["recursive_plain"]["grads_per_s"])
    return out


def _per_row_max(a, b):
    """max over rows of max|a - b| / max|b| within the row."""
    return float(_rel_per_traj(a, b).max())


def _vec_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


class _NeuralCase:
    """One neural workload: its inputs, its Lowered solves per kernel form and
    precision, and the FP64 oracle on a subset of its trajectories."""

    def __init__(self, dev, kind):
        import torch
        import diffrax_gb300 as dfx
        self.dev, self.kind = dev, kind
        self.cores = os.cpu_count() or 1
        if kind == "ode":
            self.widths, self.B, seed = [64, 128, 128, 64], 8192, 21
            self.solver, self.ctrl, self.dt0 = (dfx.Tsit5(),
                                                dfx.PIDController(rtol=1e-5, atol=1e-7), None)
            self.ts, self.sde = None, False
            self.adjoint = dfx.RecursiveCheckpointAdjoint(checkpoints=64)
            self.name = "neural_ode_64_128_tsit5_pid_b8192_recursive64"
        elif kind == "wide":
            self.widths, self.B, seed = [64, 256, 256, 64], 16384, 22
            self.solver, self.ctrl, self.dt0 = (dfx.Tsit5(),
                                                dfx.PIDController(rtol=1e-5, atol=1e-7), None)
            self.ts, self.sde = np.linspace(0.0, 1.0, 32), False
            self.adjoint = dfx.BacksolveAdjoint()
            self.name = "neural_ode_64_256_tsit5_pid_b16384_ts32_backsolve"
        else:
            self.widths, self.B, seed = [32, 64, 64, 32], 32768, 23
            self.solver, self.ctrl, self.dt0 = dfx.Heun(), dfx.ConstantStepSize(), 0.01
            self.ts, self.sde = None, True
            # the default checkpoint count (ceil(log2(max_steps)))
            self.adjoint = dfx.RecursiveCheckpointAdjoint()
            self.name = "neural_sde_32_64_heun_dt0.01_vbt1e-3_b32768_recursive"
        self.saveat = dfx.SaveAt(ts=self.ts) if self.ts is not None else dfx.SaveAt(t1=True)
        w, D = self.widths, self.widths[0]
        self.D, self.seed = D, seed
        Ws, bs = _mlp_np(w, seed)
        rng = np.random.default_rng(seed + 1)
        self.y0 = rng.standard_normal((self.B, D)).astype(np.float32)
        params = [np.concatenate([W.reshape(-1), b]) for W, b in zip(Ws, bs)]
        self.tW = [torch.tensor(W, device=dev) for W in Ws]
        self.tb = [torch.tensor(b, device=dev) for b in bs]
        if self.sde:
            Wsig = _bf16_values(rng.standard_normal((D, D)) / np.sqrt(D))
            bsig = np.zeros(D, np.float32)
            self.tWs, self.tbs = torch.tensor(Wsig, device=dev), torch.tensor(bsig, device=dev)
            params += [Wsig.reshape(-1), bsig]
        self.params = np.concatenate(params).astype(np.float64)
        self.y0_d = torch.tensor(self.y0, device=dev)
        self.fl_eval = 2 * sum(w[i] * w[i + 1] for i in range(len(w) - 1)) + (
            2 * D * D if self.sde else 0)
        self.evals = 2 if self.sde else 6

    def terms(self, prec):
        import diffrax_gb300 as dfx
        field = dfx.MLPField(self.tW, self.tb, precision=prec)
        if not self.sde:
            return dfx.ODETerm(field)
        bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (self.D,), key=self.seed)
        return dfx.MultiTerm(dfx.ODETerm(field), dfx.ControlTerm(
            dfx.TanhDiagonalDiffusion(self.tWs, self.tbs), bm))

    def lowered(self, kern, grad, prec="bf16", n=None, adjoint=None):
        from diffrax_gb300._integrate import Lowered
        y0 = self.y0_d if n is None else self.y0_d[:n].contiguous()
        return Lowered(self.terms(prec), self.solver, 0.0, 1.0, self.dt0, y0, None,
                       self.saveat, self.ctrl, adjoint or self.adjoint, 4096, kern, 0, 0,
                       want_grad=grad)

    def desc(self, fields):
        import oracle as O
        return O.make_desc(**O.oracle_fields(fields))

    def oracle_forward(self, n, params=None):
        import oracle as O
        low = self.lowered("fused", False, n=1)
        return O.solve(self.desc(low.fields), 0.0, 1.0, self.dt0,
                       self.y0[:n].astype(np.float64),
                       params=self.params if params is None else params, ts=self.ts,
                       nthreads=self.cores)

    def grad_ys(self, ys):
        """Cotangent of loss = mean(y^2) over the whole batch (and over the
        saved points: sum)."""
        return 2.0 * ys / (self.B * self.D)


def _neural_forward(case, flush, steps, warmup, n_chk=256):
    """The forward solve in the fused (BF16 tensor-core) and plain (FP32
    one-trajectory-per-thread) forms, each with its error against the FP64
    oracle on the first n_chk trajectories; when the fused form's error is
    above the plain form's, the fused kernel's FP32 mode is timed too (the
    comparison at equal accuracy)."""
    peaks, src = measured_peaks()
    ref = case.oracle_forward(n_chk)
    out = {}
    for form, kern, prec, reps in (("fused", "fused", "bf16", steps),
                                   ("plain", "plain", "fp32", max(2, steps // 4))):
        low = case.lowered(kern, False, prec)
        ms = _events_time(low.run_forward, reps, min(warmup, 1) if form == "plain" else warmup,
                          flush)
        ys, _, res, st = low.run_forward()
        e = _rel_per_traj(ys[:n_chk].double().cpu().numpy(), ref["ys"])
        out[form] = {"traj_per_s": case.B / (ms / 1e3), "ms": ms,
                     "max_rel_err_vs_fp64_oracle": float(e.max()),
                     "median_rel_err_vs_fp64_oracle": float(np.median(e)),
                     "mean_attempted_steps": float(st[:, 0].float().mean().item()),
                     "all_successful": bool((res == 0).all().item())}
    f = out["fused"]
    alg = case.B * f["mean_attempted_steps"] * case.evals * case.fl_eval / (f["ms"] / 1e3) / 1e12
    peak = peaks.get("bf16_tflops", 1900.0)
    f["roofline"] = {
        "bound": "tensor", "achieved": alg, "peak": peak, "unit": "TFLOP/s",
        "frac": alg / peak, "peak_source": src,
        "work": f"{case.fl_eval} flop per field evaluation x {case.evals} evaluations per "
                f"attempted step (algorithmic; the three-piece operands execute 3x that)"}
    out["fused_over_plain"] = out["plain"]["ms"] / f["ms"]
    out["fused_err_le_plain_err"] = (f["max_rel_err_vs_fp64_oracle"]
                                     <= out["plain"]["max_rel_err_vs_fp64_oracle"])
    if not out["fused_err_le_plain_err"]:
        low = case.lowered("fused", False, "fp32")
        ms = _events_time(low.run_forward, steps, warmup, flush)
        ys = low.run_forward()[0]
        e = _rel_per_traj(ys[:n_chk].double().cpu().numpy(), ref["ys"])
        out["fused_fp32"] = {"traj_per_s": case.B / (ms / 1e3), "ms": ms,
                             "max_rel_err_vs_fp64_oracle": float(e.max()),
                             "median_rel_err_vs_fp64_oracle": float(np.median(e))}
        out["fused_fp32_over_plain"] = out["plain"]["ms"] / ms
        out["fused_fp32_err_le_plain_err"] = (float(e.max())
                                              <= out["plain"]["max_rel_err_vs_fp64_oracle"])
    cpu_n = 512
    out["cpu_baseline"] = _oracle_rate(lambda: case.oracle_forward(cpu_n), cpu_n, case.cores)
    return out


def _recursive_grad(case, flush, steps, warmup, n_g=64):
    """Forward + RecursiveCheckpointAdjoint backward of loss = mean(y(t1)^2):
    gradients/s of the fused and plain forms over the whole batch, and each
    form's dL/dy0 and dL/dtheta against the FP64 oracle's discretise-then-
    optimise gradient on the first n_g trajectories (end to end: each side's
    cotangent comes from its own forward)."""
    import torch
    import oracle as O
    ref_f = case.oracle_forward(n_g)
    low1 = case.lowered("fused", True, n=1)
    r = O.grad_recursive(case.desc(low1.fields), 0.0, 1.0, case.dt0,
                         case.y0[:n_g].astype(np.float64), case.grad_ys(ref_f["ys"]),
                         params=case.params, ts=case.ts, nthreads=case.cores)
    out = {}

    def run(kern, prec, n=None):
        low = case.lowered(kern, True, prec, n=n)

        def fwd_bwd():
            ys_, _, _, _, ws = low.run_forward(keep_workspace=True)
            return low.run_backward(ws, case.grad_ys(ys_), low.y0, low.params)
        return low, fwd_bwd

    def errs(kern, prec):
        _, fb = run(kern, prec, n_g)
        gy0, gp = fb()
        return (_per_row_max(gy0.double().cpu().numpy(), r["grad_y0"]),
                _vec_rel(gp.double().cpu().numpy(), r["grad_params"]))

    forms = [("fused", "fused", "bf16", steps, warmup),
             ("plain", "plain", "fp32", max(2, steps // 2), 1)]
    for form, kern, prec, reps, wu in forms:
        _, fb = run(kern, prec)
        ms = _events_time(fb, reps, wu, flush)
        e0, ep = errs(kern, prec)
        out[form] = {"grads_per_s": case.B / (ms / 1e3), "ms": ms,
                     "unit": "trajectory gradients/s",
                     "dL_dy0_max_rel_err_vs_fp64_oracle": e0,
                     "dL_dtheta_rel_err_vs_fp64_oracle": ep}
    f, p = out["fused"], out["plain"]
    out["fused_over_plain"] = p["ms"] / f["ms"]
    out["fused_err_le_plain_err"] = (
        f["dL_dy0_max_rel_err_vs_fp64_oracle"] <= p["dL_dy0_max_rel_err_vs_fp64_oracle"] and
        f["dL_dtheta_rel_err_vs_fp64_oracle"] <= p["dL_dtheta_rel_err_vs_fp64_oracle"])
    if not out["fused_err_le_plain_err"]:
        _, fb = run("fused", "fp32")
        ms = _events_time(fb, steps, warmup, flush)
        e0, ep = errs("fused", "fp32")
        out["fused_fp32"] = {"grads_per_s": case.B / (ms / 1e3), "ms": ms,
                             "dL_dy0_max_rel_err_vs_fp64_oracle": e0,
                             "dL_dtheta_rel_err_vs_fp64_oracle": ep}
        out["fused_fp32_over_plain"] = p["ms"] / ms
        out["fused_fp32_err_le_plain_err"] = (
            e0 <= p["dL_dy0_max_rel_err_vs_fp64_oracle"] and
            ep <= p["dL_dtheta_rel_err_vs_fp64_oracle"])
    out["oracle_fp64_grad_norm"] = float(np.linalg.norm(r["grad_params"]))
    t = time.perf_counter()
    O.grad_recursive(case.desc(low1.fields), 0.0, 1.0, case.dt0,
                     case.y0[:n_g].astype(np.float64), case.grad_ys(ref_f["ys"]),
                     params=case.params, ts=case.ts, nthreads=case.cores)
    dt = time.perf_counter() - t
    out["cpu_baseline"] = {"value": n_g / dt, "unit": "trajectory gradients/s",
                           "cores": case.cores, "kind": "port",
                           "sample": f"{n_g} trajectories forward + backward, FP64 oracle, "
                                     f"{dt:.2f} s"}
    return out


def _backsolve_grad(case, flush, steps, warmup, n_g=32):
    """Forward + BacksolveAdjoint backward of loss = sum over the saved points
    of mean(y^2), under the reference's default rms_norm (a_theta in the error
    norm, streamed from HBM) and under adjoint_rms_seminorm.  Gradients/s of
    the fused and plain forms over the whole batch; each form's dL/dy0 and
    dL/dtheta against the FP64 oracle (forward with the config's FP32 weights,
    backsolve from its own saves) on the first n_g trajectories."""
    import diffrax_gb300 as dfx
    import oracle as O
    ref_f = case.oracle_forward(n_g)
    out = {}
    for name, adj in (("rms_norm", dfx.BacksolveAdjoint()),
                      ("seminorm", dfx.BacksolveAdjoint(stepsize_controller=dfx.PIDController(
                          rtol=case.ctrl.rtol, atol=case.ctrl.atol,
                          norm=dfx.adjoint_rms_seminorm)))):
        bdesc = case.desc(case.lowered("fused", True, n=1, adjoint=adj).bwd_fields)
        t = time.perf_counter()
        r = O.backsolve(bdesc, 0.0, 1.0, None, ref_f["ts"], ref_f["ys"],
                        case.grad_ys(ref_f["ys"]), params=case.params, nthreads=case.cores)
        dt_cpu = time.perf_counter() - t

        def run(kern, prec, n=None):
            low = case.lowered(kern, True, prec, n=n, adjoint=adj)

            def fwd_bwd():
                ys_, ts_, _, _ = low.run_forward()
                return low.run_backsolve(ts_, ys_, case.grad_ys(ys_), low.params)
            return low, fwd_bwd

        def errs(kern, prec):
            low, fb = run(kern, prec, n_g)
            gy0, gp, res, _ = fb()
            return (_per_row_max(gy0.double().cpu().numpy(), r["grad_y0"]),
                    _vec_rel(gp.double().cpu().numpy(), r["grad_params"]), low)

        ent = {}
        forms = [("fused", "fused", "bf16", steps, warmup)]
        if name == "rms_norm":
            forms.append(("plain", "plain", "fp32", 1, 0))  # one ~40 s solve
        for form, kern, prec, reps, wu in forms:
            low, fb = run(kern, prec)
            ms = _events_time(fb, reps, wu, flush)
            gy0, gp, res, st = fb()
            e0, ep, _ = errs(kern, prec)
            ent[form] = {"grads_per_s": case.B / (ms / 1e3), "ms": ms,
                         "unit": "trajectory gradients/s",
                         "mean_backward_steps": float(st[:, 0].float().mean().item()),
                         "backward_failures": int((res != 0).sum().item()),
                         "dL_dy0_max_rel_err_vs_fp64_oracle": e0,
                         "dL_dtheta_rel_err_vs_fp64_oracle": ep}
            if form == "fused" and name == "rms_norm":
                peaks, src = measured_peaks()
                n_par = int(low.params.numel())
                stream = float(st[:, 0].double().sum().item()) * 2 * 4 * n_par
                peak = peaks.get("hbm_gbs", 6800.0)
                ent["roofline"] = {
                    "bound": "hbm", "achieved": stream / (ms / 1e3) / 1e9, "peak": peak,
                    "unit": "GB/s", "frac": stream / (ms / 1e3) / 1e9 / peak,
                    "peak_source": src, "a_theta_stream_bytes": stream,
                    "work": "a_theta double buffer: 8 bytes per parameter per "
                            "trajectory-step (read a_theta0, write the candidate); timed "
                            "region = forward + backward"}
        if "plain" in ent:
            f, p = ent["fused"], ent["plain"]
            ent["fused_over_plain"] = p["ms"] / f["ms"]
            ent["fused_err_le_plain_err"] = (
                f["dL_dy0_max_rel_err_vs_fp64_oracle"] <= p["dL_dy0_max_rel_err_vs_fp64_oracle"]
                and f["dL_dtheta_rel_err_vs_fp64_oracle"]
                <= p["dL_dtheta_rel_err_vs_fp64_oracle"])
            if not ent["fused_err_le_plain_err"]:
                low, fb = run("fused", "fp32")
                ms = _events_time(fb, max(2, steps // 2), 1, flush)
                e0, ep, _ = errs("fused", "fp32")
                ent["fused_fp32"] = {"grads_per_s": case.B / (ms / 1e3), "ms": ms,
                                     "dL_dy0_max_rel_err_vs_fp64_oracle": e0,
                                     "dL_dtheta_rel_err_vs_fp64_oracle": ep}
                ent["fused_fp32_over_plain"] = p["ms"] / ms
                ent["fused_fp32_err_le_plain_err"] = (
                    e0 <= p["dL_dy0_max_rel_err_vs_fp64_oracle"] and
                    ep <= p["dL_dtheta_rel_err_vs_fp64_oracle"])
        ent["oracle_mean_backward_steps"] = float(r["stats"][:, 0].mean())
        ent["cpu_baseline"] = {"value": n_g / dt_cpu, "unit": "trajectory gradients/s",
                               "cores": case.cores, "kind": "port",
                               "sample": f"{n_g} trajectories backward only, FP64 oracle, "
                                         f"{dt_cpu:.2f} s"}
        out[f"backsolve_{name}"] = ent
    return out


def workload_neural(dev, flush, steps, warmup, kind):
    """Neural ODE (64-128-128-64, Tsit5 PID(1e-5, 1e-7), batch 8192, t1 save,
    RecursiveCheckpointAdjoint(64), loss mean y(t1)^2), the wide neural ODE
    (64-256-256-64, batch 16384, 32 ts, BacksolveAdjoint, loss sum over the
    saves of mean y^2) or the neural SDE (drift 32-64-64-32, diffusion
    0.1 tanh(W y + b), Heun dt 0.01, VBT tol 1e-3, batch 32768,
    RecursiveCheckpointAdjoint, loss mean y(t1)^2): forward and gradient
    throughput of the fused and plain forms with their errors against the
    FP64 oracle."""
    import torch
    case = _NeuralCase(dev, kind)
    out = {"workload": case.name, "forward": _neural_forward(case, flush, steps, warmup)}
    if kind == "ode":
        # The same forward on the fifth-generation tensor cores (tcgen05.mma,
        # TMEM accumulators; 128 trajectories per CTA), at this batch (64
        # tiles) and at a batch filling every SM with one tile (152 x 128),
        # beside the mma.sync row-tile kernel at that batch.
        import oracle as O
        from diffrax_gb300._integrate import Lowered
        n_chk = 256
        ref = case.oracle_forward(n_chk)
        tc = case.lowered("tc", False)
        ms_t = _events_time(tc.run_forward, steps, warmup, flush)
        ys_t, _, _, st_t = tc.run_forward()
        e_t = _rel_per_traj(ys_t[:n_chk].double().cpu().numpy(), ref["ys"])
        peaks, src = measured_peaks()
        alg_t = (case.B * float(st_t[:, 0].float().mean().item()) * case.evals * case.fl_eval
                 / (ms_t / 1e3) / 1e12)
        out["forward"]["tc"] = {
            "traj_per_s": case.B / (ms_t / 1e3), "ms": ms_t,
            "max_rel_err_vs_fp64_oracle": float(e_t.max()),
            "roofline": {"bound": "tensor", "achieved": alg_t,
                         "frac": alg_t / peaks.get("bf16_tflops", 1900.0),
                         "unit": "TFLOP/s", "peak_source": src}}
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        Bf = 128 * sms
        yf = torch.tensor(np.random.default_rng(case.seed + 2).standard_normal((Bf, case.D)),
                          dtype=torch.float32, device=dev)
        full = {}
        for kern in ("fused", "tc"):
            lo = Lowered(case.terms("bf16"), case.solver, 0.0, 1.0, case.dt0, yf, None,
                         case.saveat, case.ctrl, None, 4096, kern, 0, 0)
            ms_k = _events_time(lo.run_forward, steps, warmup, flush)
            full[kern] = {"traj_per_s": Bf / (ms_k / 1e3), "ms": ms_k}
        full["tc_over_fused"] = full["fused"]["ms"] / full["tc"]["ms"]
        out[f"forward_batch_{Bf}"] = full
    if kind == "wide":
        out.update(_backsolve_grad(case, flush, steps, warmup))
    else:
        out["gradient"] = _recursive_grad(case, flush, steps, warmup)
    return out


def _summary(others, vdp_ratio, vdp_err, vdp_plain_err):
    """grads_per_s, fused_over_plain and errors (fused, plain) per config."""
    def g(d, *keys):
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    def r3(x):
        return None if x is None else float(f"{x:.3g}")
    grads, ratio, errs = {}, {"c2_vdp_fwd": r3(vdp_ratio)}, {
        "c2_vdp_fwd": [r3(vdp_err), r3(vdp_plain_err)]}
    lv = others.get("lotka_volterra", {})
    ratio["c1_lv_fwd"] = r3(g(lv, "fused_over_plain_f32"))
    errs["c1_lv_fwd"] = [r3(g(lv, "fused_f32", "max_rel_err_vs_fp64_oracle")),
                         r3(g(lv, "plain_f32", "max_rel_err_vs_fp64_oracle"))]
    e0 = "dL_dy0_max_rel_err_vs_fp64_oracle"
    for tag, key, gk in (("c3_node", "neural_ode", "gradient"),
                         ("c4_wide", "neural_ode_wide", "backsolve_rms_norm"),
                         ("c5_nsde", "neural_sde", "gradient")):
        c = others.get(key, {})
        fw = g(c, "forward")
        ratio[f"{tag}_fwd"] = r3(g(fw, "fused_over_plain"))
        errs[f"{tag}_fwd"] = [r3(g(fw, "fused", "max_rel_err_vs_fp64_oracle")),
                              r3(g(fw, "plain", "max_rel_err_vs_fp64_oracle"))]
        if g(fw, "fused_fp32") is not None:
            ratio[f"{tag}_fwd_fp32"] = r3(g(fw, "fused_fp32_over_plain"))
            errs[f"{tag}_fwd_fp32"] = r3(g(fw, "fused_fp32", "max_rel_err_vs_fp64_oracle"))
        gr = g(c, gk)
        grads[tag] = r3(g(gr, "fused", "grads_per_s"))
        grads[f"{tag}_plain"] = r3(g(gr, "plain", "grads_per_s"))
        ratio[f"{tag}_grad"] = r3(g(gr, "fused_over_plain"))
        errs[f"{tag}_grad_dy0"] = [r3(g(gr, "fused", e0)), r3(g(gr, "plain", e0))]
        errs[f"{tag}_grad_dtheta"] = [
            r3(g(gr, "fused", "dL_dtheta_rel_err_vs_fp64_oracle")),
            r3(g(gr, "plain", "dL_dtheta_rel_err_vs_fp64_oracle"))]
        if g(gr, "fused_fp32") is not None:
            grads[f"{tag}_fp32"] = r3(g(gr, "fused_fp32", "grads_per_s"))
            ratio[f"{tag}_grad_fp32"] = r3(g(gr, "fused_fp32_over_plain"))
            errs[f"{tag}_grad_fp32_dy0"] = r3(g(gr, "fused_fp32", e0))
            errs[f"{tag}_grad_fp32_dtheta"] = r3(
                g(gr, "fused_fp32", "dL_dtheta_rel_err_vs_fp64_oracle"))
    grads["c4_wide_seminorm"] = r3(g(others.get("neural_ode_wide", {}), "backsolve_seminorm",
                                     "fused", "grads_per_s"))
    return {"grads_per_s": grads, "fused_over_plain": ratio,
            "max_rel_err_fused_plain": errs}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbdx", choices=["gbdx", "reference"])
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--ref-sample", type=int, default=0,
                    help="trajectories per reference step (default: the whole batch)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the other configurations")
    ap.add_argument("--profile", default=None,
                    choices=["fused", "plain", "backsolve", "backsolve_seminorm", "neural_ode",
                             "neural_ode_tc", "neural_ode_grad", "neural_ode_wide",
                             "neural_sde", "neural_sde_grad", "saveat_steps"],
                    help="run warmup + steps eager solves of one kernel only (for ncu); "
                         "backsolve*: forward + backward of the wide neural ODE at --batch")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist

    import diffrax_gb300 as dfx
    from diffrax_gb300._integrate import Lowered

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    B = args.batch
    mu, y0, t1 = vdp_inputs(B, args.seed + rank)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)
    term = dfx.ODETerm(dfx.VanDerPol())
    y0_d = torch.tensor(y0, dtype=torch.float32, device=dev)
    mu_d = torch.tensor(mu[:, None], dtype=torch.float32, device=dev)
    t1_d = torch.tensor(t1, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def lowered(kernel):
        return Lowered(term, dfx.Dopri5(), 0.0, t1_d, None, y0_d, mu_d, dfx.SaveAt(t1=True),
                       pid, None, 4096, kernel, 0, 0)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def time_kernel(kernel, steps, sampler=None):
        low = lowered(kernel)
        for _ in range(args.warmup):
            low.run_forward()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            outs = low.run_forward()
        g.replay()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        barrier()
        if sampler:
            sampler.start()
        wall = time.perf_counter()
        for e0, e1 in evs:
            flush.fill_(1.0)          # evict L2 between timed solves (not timed)
            e0.record()
            g.replay()
            e1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall
        barrier()
        clocks = sampler.stop() if sampler else None
        ms = [a.elapsed_time(b) for a, b in evs]
        ms_step = statistics.mean(ms)
        if world > 1:
            t = torch.tensor([ms_step], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms_step = float(t.item())
        return ms_step, outs, clocks, wall

    if args.profile and args.profile.startswith("backsolve"):
        profile_backsolve(dev, B, args.profile == "backsolve_seminorm",
                          args.warmup + args.steps)
        return
    if args.profile and args.profile.startswith("neural"):
        profile_neural(dev, args.profile, B, args.warmup + args.steps)
        return
    if args.profile == "saveat_steps":
        profile_saveat_steps(dev, args.warmup + args.steps)
        return
    if args.profile:
        low = lowered(args.profile)
        for _ in range(args.warmup + args.steps):
            outs = low.run_forward()
        torch.cuda.synchronize()
        ok = bool((outs[2] == 0).all().item())
        print(json.dumps({"profile": args.profile, "solves": args.warmup + args.steps,
                          "all_successful": ok}))
        if not ok:
            sys.exit(1)
        return

    sampler = ClockSampler(local)
    ms_fused, outs, clocks, wall = time_kernel("fused", args.steps, sampler)
    ms_plain, outs_plain, _, _ = time_kernel("plain", max(3, args.steps // 2))
    value = B * world / (ms_fused / 1e3)
    plain_value = B * world / (ms_plain / 1e3)

    ys, ts_out, res, stats = outs
    steps_total = int(stats[:, 0].sum().item())
    ok = bool((res == 0).all().item())

    # End to end through the public call: pinned host inputs in, results out.
    y0_h = torch.tensor(y0, dtype=torch.float32).pin_memory()
    mu_h = torch.tensor(mu[:, None], dtype=torch.float32).pin_memory()
    t1_h = torch.tensor(t1, dtype=torch.float64).pin_memory()
    ys_h = torch.empty((B, 1, 2), dtype=torch.float32).pin_memory()
    res_h = torch.empty((B,), dtype=torch.int32).pin_memory()

    def eager_step():
        sol = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, t1_h, None, y0_h, mu_h,
                              stepsize_controller=pid, throw=False)
        ys_h.copy_(sol.ys, non_blocking=True)
        res_h.copy_(sol.result, non_blocking=True)
        torch.cuda.synchronize()

    # the page-locked inputs are the graph's staging buffers: each replay
    # solves with the kernels reading them and writing ys, ts, result and
    # stats into page-locked host tensors in place (one graph launch per
    # solve; copies in and out inside the graph where the GPU does not map
    # page-locked memory)
    graphed = dfx.GraphedSolve(term, dfx.Dopri5(), 0.0, t1_h, None, y0_h, mu_h,
                               stepsize_controller=pid, throw=False, host_io=True)
    graphed_out = {}

    def graphed_step():
        graphed_out["sol"] = graphed()

    def wall_time(step):
        for _ in range(args.warmup):
            step()
        barrier()
        ts_ = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t = time.perf_counter()
            step()
            ts_.append(time.perf_counter() - t)
        s_ = statistics.mean(ts_)
        if world > 1:
            t = torch.tensor([s_], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            s_ = float(t.item())
        return s_
    e2e_s = wall_time(graphed_step)
    gsol = graphed_out["sol"]
    e2e_ok = bool((gsol.result == 0).all()) and bool(torch.equal(gsol.ys, ys.cpu()))
    eager_s = wall_time(eager_step)
    h2d = B * (2 * 4 + 4 + 8)  # y0, mu, t1 (t0 = 0 is a cached device scalar)
    d2h = B * (2 * 4 + 4)      # eager: ys, result
    d2h_graphed = B * (2 * 4 + 8 + 4 + 3 * 4)  # ys, ts, result, stats

    # The kernel's own bound: no schedule finishes before its longest
    # trajectory, whose steps depend on one another.  That trajectory alone
    # (the same kernel, batch 1, CUDA events, median of the timed solves).
    crit = None
    if rank == 0:
        k_long = int(stats[:, 0].argmax().item())
        lone = Lowered(term, dfx.Dopri5(), 0.0, t1_d[k_long:k_long + 1].contiguous(), None,
                       y0_d[k_long:k_long + 1].contiguous(), mu_d[k_long:k_long + 1].contiguous(),
                       dfx.SaveAt(t1=True), pid, None, 4096, "fused", 0, 0)
        ms_lone = _events_time(lone.run_forward, 20, 3, flush)
        n_long = int(stats[k_long, 0].item())
        crit = {"trajectory": k_long, "attempted_steps": n_long, "alone_ms": ms_lone,
                "batch_ms": ms_fused, "frac": ms_lone / ms_fused}

    others = {}
    if rank == 0 and not args.headline_only:
        for key, fn in (("lotka_volterra", lambda: workload_lotka_volterra(dev, flush, 10, 3)),
                        ("neural_ode", lambda: workload_neural(dev, flush, 5, 3, "ode")),
                        ("neural_ode_wide", lambda: workload_neural(dev, flush, 5, 3, "wide")),
                        ("neural_sde", lambda: workload_neural(dev, flush, 5, 3, "sde")),
                        ("next_rows", lambda: workload_next_rows(dev, flush, 10, 3)),
                        ("analytic_grads", lambda: workload_analytic_grads(dev, flush, 5, 3))):
            try:
                others[key] = fn()
            except Exception as exc:  # report, never hide the headline line
                others[key] = {"error": f"{type(exc).__name__}: {exc}"}

    if rank == 0:
        peaks, src = measured_peaks()
        t_s = ms_fused / 1e3
        fp32 = steps_total * FP32_FLOPS_PER_STEP / t_s / 1e12
        fp64 = steps_total * FP64_OPS_PER_STEP / t_s / 1e12
        gbs = B * BYTES_PER_TRAJ / t_s / 1e9
        # The fused kernel's bound is the dependent-step latency of its longest
        # trajectory (critical_path: that trajectory alone / the whole batch),
        # not HBM (DRAM ~0.03 %) nor the FP32 pipe: the HBM line is kept in
        # the contract's form, with the critical path and the compute rates
        # beside it.
        hbm_peak = peaks.get("hbm_gbs", 6800.0)
        sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
        if crit is not None:
            crit["cycles_per_step_alone"] = (crit["alone_ms"] * 1e-3 * sm_mhz * 1e6
                                             / max(crit["attempted_steps"], 1))
            crit["sm_mhz"] = sm_mhz
        roofline = {
            "bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
            "frac": gbs / hbm_peak, "traffic": NCU_TRAFFIC_BYTES_PER_LAUNCH,
            "traffic_source": "ncu capture of this kernel on this workload, not this run",
            "peak_source": src,
            "work": f"{BYTES_PER_TRAJ} algorithmic bytes per trajectory x {B} per launch",
            "binding": "critical_path",
            "critical_path": crit,
            "fp32": {"achieved": fp32, "peak": FP32_PEAK_TFLOPS_NOMINAL, "unit": "TFLOP/s",
                     "frac": fp32 / FP32_PEAK_TFLOPS_NOMINAL,
                     "work": f"{FP32_FLOPS_PER_STEP} FP32 flop per attempted step x "
                             f"{steps_total} attempted steps per launch",
                     "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2 x 2.07 GHz), "
                                    "not measured"},
            "fp64": {"achieved": fp64, "peak": FP64_PEAK_TFLOPS_NOMINAL, "unit": "TFLOP/s",
                     "frac": fp64 / FP64_PEAK_TFLOPS_NOMINAL,
                     "peak_source": "nominal GB300 FP64 rate, not measured"},
        }
        # Accuracy of both kernels against the FP64 oracle on the same inputs.
        n_chk = min(B, 4096)
        ref = oracle_solve(mu[:n_chk], y0[:n_chk], t1[:n_chk], os.cpu_count() or 1)
        def err(o):
            a = o[0][:n_chk].double().cpu().numpy()
            per = np.abs(a - ref["ys"]).max(axis=(1, 2)) / np.abs(ref["ys"]).max(axis=(1, 2))
            return float(per.max()), float(np.median(per))
        fused_err = err(outs)
        plain_err = err(outs_plain)
        cpu = None
        if not args.no_cpu_baseline:
            # Whole batches of the same workload through the FP64 oracle on all
            # host cores until at least ~10 core-seconds of work are done.
            cores = os.cpu_count() or 1
            done, t = 0, time.perf_counter()
            while True:
                oracle_solve(mu, y0, t1, cores)
                done += B
                dt = time.perf_counter() - t
                if dt * cores >= 10.0 or dt > 30.0:
                    break
            cpu = {"value": done / dt, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": f"{done // B} full batch(es) of {B} trajectories, FP64 oracle, "
                             f"OpenMP over trajectories, {dt:.2f} s wall"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_fused,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 state, f64 time", "data": "synthetic",
            "config": {"workload": WORKLOAD, "batch_per_gpu": B, "solver": "Dopri5",
                       "controller": "PID(rtol=1e-6, atol=1e-9, pcoeff=0.3, icoeff=0.4)",
                       "saveat": "t1", "kernel": "fused persistent (CUDA graph)",
                       "l2": "256 MB buffer written between timed solves"},
            "e2e": {"value": B * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h_graphed, "api": "GraphedSolve(host_io=True)",
                    "transfer": ("kernels read and write page-locked host memory in place"
                                 if graphed.zero_copy else "copies inside the graph"),
                    "results_equal_device_run": e2e_ok},
            "e2e_eager": {"value": B * world / eager_s, "unit": UNIT,
                          "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                          "api": "diffeqsolve"},
            # per timed solve: the four longest-first work-order kernels and
            # the integrator (one graph replay)
            "gpu_launches": 5 * args.steps,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "plain": {"value": plain_value, "ms_per_step": ms_plain,
                      "max_rel_err_vs_fp64_oracle": plain_err[0],
                      "median_rel_err_vs_fp64_oracle": plain_err[1]},
            "max_rel_err_vs_fp64_oracle": fused_err[0],
            "median_rel_err_vs_fp64_oracle": fused_err[1],
            "all_successful": ok,
            "attempted_steps_per_launch": steps_total,
            "wall_s_timed_region": wall,
            "other_configs": others,
        }
        # The whole metric in brief, last on the line: gradients/s, fused over
        # plain and both forms' errors against the FP64 oracle per config.
        line.update(_summary(others, value / plain_value, fused_err[0], plain_err[0]))
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
