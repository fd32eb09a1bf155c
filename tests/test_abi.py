"""The C ABI: the library builds and loads, exports every symbol declared in
include/gbdx.h, agrees with the Python descriptor layout and validates problems
the way the reference raises ValueErrors.  No kernel runs here."""
import ctypes
import os
import re

import pytest
import torch

import diffrax_gb300 as dfx
from diffrax_gb300 import _lib
from diffrax_gb300._integrate import _host_checks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "gbdx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbdx_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = header_functions()
    assert "gbdx_solve_fwd" in names and len(names) >= 8
    for n in names:
        assert hasattr(lib, n), f"{n} declared in gbdx.h but not exported"


def test_descriptor_layout():
    lib = _lib.load()
    assert lib.gbdx_problem_desc_size() == ctypes.sizeof(_lib.ProblemDesc)
    assert lib.gbdx_version() >= 1


def _fields(**kw):
    base = dfx.lower(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(),
                     dfx.PIDController(rtol=1e-6, atol=1e-9), dfx.SaveAt(t1=True), dim=2,
                     dtype=torch.float32, max_steps=4096, n_ts=0)
    base.update(kw)
    return base


def test_problem_create_and_queries():
    p = _lib.Problem(_fields())
    assert p.n_save == 1
    assert p.workspace_size(1000) >= 8
    p2 = _lib.Problem(_fields(n_ts=7, save_t0=1))
    assert p2.n_save == 9


@pytest.mark.parametrize("bad, msg", [
    (dict(solver=0), "error estimates"),          # adaptive Euler (pid.py:437-447)
    (dict(solver=9), "unknown solver"),
    (dict(max_steps=0), "max_steps"),
    (dict(save_t1=0), "Empty saveat"),
    (dict(save_steps=-1), "steps"),
    (dict(dtype=7), "dtype"),
])
def test_problem_validation(bad, msg):
    with pytest.raises(ValueError, match=msg):
        _lib.Problem(_fields(**bad))


def test_unsupported_dimension():
    with pytest.raises(_lib.GbdxError):
        _lib.Problem(_fields(dim=3))


def test_sde_euler_adaptive_rejected():
    # _integrate.py:1145-1151
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (1,), key=0)
    terms = dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                          dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))
    with pytest.raises(ValueError, match="SDE"):
        dfx.lower(terms, dfx.Euler(), dfx.PIDController(rtol=1e-3, atol=1e-3),
                  dfx.SaveAt(t1=True), dim=1, dtype=torch.float32, max_steps=10, n_ts=0)


def test_host_checks():
    t0 = torch.tensor([0.1], dtype=torch.float64)
    t1 = torch.tensor([1.1], dtype=torch.float64)
    with pytest.raises(ValueError):
        _host_checks(t0, t1, torch.tensor([-0.1], dtype=torch.float64), None, 0)
    # test/test_saveat_solution.py:89-94: ts outside [t0, t1] raise RuntimeError.
    with pytest.raises(RuntimeError):
        _host_checks(t0, t1, None, torch.tensor([0.0], dtype=torch.float64), 0)
    with pytest.raises(RuntimeError):
        _host_checks(t0, t1, None, torch.tensor([3.0], dtype=torch.float64), 0)
    with pytest.raises(RuntimeError):
        _host_checks(t0, t1, None, torch.tensor([0.8, 0.5], dtype=torch.float64), 0)
    _host_checks(t0, t1, None, torch.tensor([0.5, 0.8], dtype=torch.float64), 0)
    # backwards in time: decreasing ts are valid
    _host_checks(t1, t0, None, torch.tensor([0.8, 0.5], dtype=torch.float64), 0)


def test_saveat_validation():
    with pytest.raises(ValueError):
        dfx.SaveAt()
    s = dfx.SaveAt(t1=True, solver_state=True)
    assert s.solver_state and not s.controller_state and not s.state_only
    assert dfx.SaveAt(made_jump=True).state_only
    # the states alone still save one point internally (the final state)
    f = dfx.lower(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(), dfx.ConstantStepSize(),
                  dfx.SaveAt(controller_state=True), dim=2, dtype=torch.float32,
                  max_steps=8, n_ts=0)
    assert f["save_t1"] == 1


def test_backsolve_kwargs_validation():
    with pytest.raises(ValueError):
        dfx.BacksolveAdjoint(foo=1)
    dfx.BacksolveAdjoint(solver=dfx.Dopri5())


def _mlp_fields(widths, solver, **kw):
    W = [torch.zeros(widths[i + 1], widths[i]) for i in range(3)]
    b = [torch.zeros(widths[i + 1]) for i in range(3)]
    f = dfx.lower(dfx.ODETerm(dfx.MLPField(W, b)), solver,
                  dfx.PIDController(rtol=1e-5, atol=1e-7), dfx.SaveAt(ts=[0.5, 1.0]),
                  dim=widths[0], dtype=torch.float32, max_steps=64, n_ts=2,
                  adjoint=dfx.BacksolveAdjoint())
    f.update(kw)
    return f


def test_backsolve_problem_creation():
    p = _lib.Problem(_mlp_fields([64, 256, 256, 64], dfx.Tsit5()))
    assert p.param_count() == 64 * 256 + 256 + 256 * 256 + 256 + 256 * 64 + 64
    _lib.Problem(_mlp_fields([32, 64, 64, 32], dfx.Heun()))
    _lib.Problem(_mlp_fields([32, 64, 64, 32], dfx.Tsit5(), norm=1))
    with pytest.raises(_lib.GbdxError, match="backsolve"):
        _lib.Problem(_mlp_fields([64, 256, 256, 64], dfx.Heun()))
    with pytest.raises(ValueError, match="norm"):
        _lib.Problem(_mlp_fields([32, 64, 64, 32], dfx.Tsit5(), norm=5))
    with pytest.raises(_lib.GbdxError, match="plain"):
        _lib.Problem(_mlp_fields([32, 64, 64, 32], dfx.Tsit5(), kernel=1))


def test_no_cpu_fallback():
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(), 0.0, 1.0, None,
                        torch.zeros(4, 2), torch.ones(1),
                        stepsize_controller=dfx.PIDController(rtol=1e-6, atol=1e-9))


@pytest.mark.parametrize("steps, t0, t1, n_ts, max_steps", [
    (1, 0, 1, 0, 4096), (2, 0, 1, 0, 4096), (3, 1, 1, 5, 4096), (3, 0, 0, 0, 10),
    (7, 1, 1, 0, 10), (0, 1, 1, 3, 100)])
def test_saveat_steps_output_length(steps, t0, t1, n_ts, max_steps):
    # _integrate.py:1273-1293, as the oracle restates it
    import oracle as O
    f = _fields(save_steps=steps, save_t0=t0, save_t1=t1, n_ts=n_ts, max_steps=max_steps)
    assert _lib.Problem(f).n_save == O.n_saves(O.make_desc(**O.oracle_fields(f)))


def test_saveat_steps_dense_scope():
    # forward solves of the analytic fields only; a dense or event problem is
    # solved by gbdx_solve_fwd_ex and evaluated by gbdx_dense_evaluate (no
    # kernel runs: the calls fail validation first)
    with pytest.raises(_lib.GbdxError, match="analytic"):
        _lib.Problem(_fields(save_steps=1, adjoint=1, checkpoints=8))
    assert _lib.Problem(_fields(save_dense=1, save_t1=0)).n_save == 0
    lib = _lib.load()
    p = _lib.Problem(_fields(save_dense=1))
    z = [None] * 16
    assert lib.gbdx_solve_fwd(p.handle, 1, *z[:3], 0, *z[:2], 0, *z[:7], 0, None) == -1
    assert "gbdx_solve_fwd_ex" in _lib.last_error()
    assert lib.gbdx_solve_fwd_ex(p.handle, 1, *z[:3], 0, *z[:2], 0, *z[:7], None, 0,
                                 None) == -1
    assert "dense_ts" in _lib.last_error()
    assert lib.gbdx_dense_evaluate(p.handle, 1, None, None, 0, None, None, None, None, 3,
                                   None, 5, 1, 0, None, None) == -1
    assert "query_stride" in _lib.last_error()
    q = _lib.Problem(_fields(n_event=1, ev_kind=[0], ev_coef=[1, 0, 0, 0, 0, 0]))
    assert lib.gbdx_solve_fwd(q.handle, 1, *z[:3], 0, *z[:2], 0, *z[:7], 0, None) == -1


@pytest.mark.parametrize("bad, msg", [
    (dict(n_event=5), "conditions"),
    (dict(n_event=1, ev_kind=[7]), "kind"),
    (dict(n_event=1, ev_dir=[3]), "direction"),
    (dict(n_event=1, event_root=1, newton_atol=0.0), "root finder"),
])
def test_event_validation(bad, msg):
    with pytest.raises(ValueError, match=msg):
        _lib.Problem(_fields(**bad))


def test_event_python_surface():
    with pytest.raises(ValueError, match="Missmatch"):
        dfx.Event([dfx.LinearCondition([1])], direction=[True, False])
    with pytest.raises(NotImplementedError):
        dfx.Event(lambda t, y, args, **kw: y)
    ev = dfx.Event([dfx.LinearCondition([1, 0], offset=-1.0),
                    dfx.LinearCondition([], t_coeff=1.0, offset=-3.0, boolean=True),
                    dfx.steady_state_event()], dfx.Newton(1e-6, 1e-7), direction=True)
    f = dfx.lower(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(),
                  dfx.PIDController(rtol=1e-6, atol=1e-9), dfx.SaveAt(t1=True), dim=2,
                  dtype=torch.float32, max_steps=64, n_ts=0, event=ev)
    assert f["n_event"] == 3 and f["ev_kind"] == [0, 1, 2] and f["ev_dir"] == [1, 1, 1]
    assert f["ev_coef"][:6] == [1.0, 0.0, 0.0, 0.0, 0.0, -1.0]
    assert f["ev_coef"][12:14] == [1e-6, 1e-9] and f["event_root"] == 1
    assert _lib.Problem(f).n_save == 1
    # steady_state_event without an adaptive controller needs its tolerances
    with pytest.raises(ValueError, match="steady_state_event"):
        dfx.lower(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(), dfx.ConstantStepSize(),
                  dfx.SaveAt(t1=True), dim=2, dtype=torch.float32, max_steps=64, n_ts=0,
                  event=dfx.Event(dfx.steady_state_event()))


def test_saveat_steps_dense_python_surface():
    with pytest.raises(ValueError, match="Empty saveat"):
        dfx.SaveAt()
    assert dfx.SaveAt(steps=True).steps == 1 and dfx.SaveAt(steps=4).steps == 4
    assert dfx.SaveAt(dense=True).dense
    f = dfx.lower(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(),
                  dfx.PIDController(rtol=1e-6, atol=1e-9), dfx.SaveAt(steps=3, dense=True),
                  dim=2, dtype=torch.float32, max_steps=64, n_ts=0)
    assert f["save_steps"] == 3 and f["save_dense"] == 1
    sol = dfx.Solution(t0=0.0, t1=1.0, ts=None, ys=None, stats={}, result=None)
    with pytest.raises(ValueError, match="dense=True"):
        sol.evaluate(0.5)


def test_autotune_cache_key_ignores_launch_shape():
    from diffrax_gb300 import _tune
    f = _fields()
    k1 = _tune._key(dict(f, block_threads=64, ctas_per_sm=2), 5000)
    k2 = _tune._key(dict(f, block_threads=0, ctas_per_sm=0), 8000)
    assert k1 == k2 and k1[1] == 8192
    assert _tune._key(f, 9000) != k2
    assert _tune.candidates(dict(f, field=3), 1024) == [("fused", 0, c) for c in (1, 2, 3, 4)]
    # the 64-128-128-64 Tsit5 BF16 forward may also take the tcgen05 tiles
    W = [torch.zeros(128, 64), torch.zeros(128, 128), torch.zeros(64, 128)]
    b = [torch.zeros(128), torch.zeros(128), torch.zeros(64)]
    mlp = dfx.lower(dfx.ODETerm(dfx.MLPField(W, b)), dfx.Tsit5(),
                    dfx.PIDController(rtol=1e-5, atol=1e-7), dfx.SaveAt(t1=True), dim=64,
                    dtype=torch.float32, max_steps=64, n_ts=0)
    assert _tune.tc_eligible(mlp) and ("tc", 0, 1) in _tune.candidates(mlp, 8192)
    assert ("tc", 0, 1) not in _tune.candidates(dict(mlp, kernel=2), 8192)
    assert _tune.tc_eligible(dict(mlp, solver=2))  # Dopri5
    assert not _tune.tc_eligible(dict(mlp, solver=1))  # Heun


def test_ou_sde_scope():
    # the Ornstein-Uhlenbeck SDE runs on the analytic kernels in FP32 state
    # with an even state dimension (the tree draws component pairs)
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), key=0)
    terms = dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                          dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))

    def fields(dim, dtype):
        return dfx.lower(terms, dfx.Heun(), dfx.ConstantStepSize(), dfx.SaveAt(t1=True),
                         dim=dim, dtype=dtype, max_steps=100, n_ts=0)
    assert _lib.Problem(fields(2, torch.float32)).n_save == 1
    assert _lib.Problem(fields(4, torch.float32)).n_save == 1
    with pytest.raises(_lib.GbdxError, match="FP32"):
        _lib.Problem(fields(2, torch.float64))
    with pytest.raises(_lib.GbdxError, match="dim 2 or 4"):
        _lib.Problem(fields(3, torch.float32))


def test_tc_kernel_scope():
    # kernel="tc": BF16 forward solves of 64 -> 128 -> 128 -> 64 MLP fields
    # with Tsit5 or Dopri5; anything else is rejected at problem creation
    W = [torch.zeros(128, 64), torch.zeros(128, 128), torch.zeros(64, 128)]
    b = [torch.zeros(128), torch.zeros(128), torch.zeros(64)]
    term = dfx.ODETerm(dfx.MLPField(W, b))
    pid = dfx.PIDController(rtol=1e-5, atol=1e-7)

    def fields(solver, **kw):
        return dfx.lower(term, solver, pid, dfx.SaveAt(t1=True), dim=64, dtype=torch.float32,
                         max_steps=64, n_ts=0, kernel="tc", **kw)
    assert _lib.Problem(fields(dfx.Tsit5())).n_save == 1
    assert _lib.Problem(fields(dfx.Dopri5())).n_save == 1
    with pytest.raises(_lib.GbdxError, match="Tsit5 or Dopri5"):
        _lib.Problem(fields(dfx.Heun()))
    with pytest.raises(_lib.GbdxError, match="adjoint"):
        _lib.Problem(fields(dfx.Tsit5(), adjoint=dfx.RecursiveCheckpointAdjoint(8)))
    with pytest.raises(_lib.GbdxError, match="MLP"):
        _lib.Problem(_fields(kernel=3))


def test_shark_and_levy_tree_scope():
    # ShARK needs an SDE whose tree has the space-time Levy area
    # (srk.py:374-379); the Levy area tree drives the Ornstein-Uhlenbeck SDE
    # kernels (Euler, Heun, Dopri5, Tsit5 use its W).
    def terms(levy):
        bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), key=0, levy_area=levy)
        return dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                             dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))

    def fields(solver, levy, ctrl=None):
        return dfx.lower(terms(levy), solver, ctrl or dfx.ConstantStepSize(),
                         dfx.SaveAt(t1=True), dim=2, dtype=torch.float32, max_steps=100,
                         n_ts=0)
    f = fields(dfx.ShARK(), dfx.SpaceTimeLevyArea)
    assert f["solver"] == 5 and f["levy_area"] == 1
    assert _lib.Problem(f).n_save == 1
    assert _lib.Problem(fields(dfx.ShARK(), dfx.SpaceTimeLevyArea,
                               dfx.PIDController(rtol=1e-3, atol=1e-3))).n_save == 1
    assert _lib.Problem(fields(dfx.Heun(), dfx.SpaceTimeLevyArea)).n_save == 1
    assert fields(dfx.Heun(), dfx.BrownianIncrement)["levy_area"] == 0
    with pytest.raises(ValueError, match="minimal Levy Area"):
        fields(dfx.ShARK(), dfx.BrownianIncrement)
    for solver, sid in ((dfx.SRA1(), 6), (dfx.SEA(), 7)):
        g = fields(solver, dfx.SpaceTimeLevyArea)
        assert g["solver"] == sid and _lib.Problem(g).n_save == 1
        with pytest.raises(ValueError, match="minimal Levy Area"):
            fields(solver, dfx.BrownianIncrement)
    assert _lib.Problem(fields(dfx.SRA1(), dfx.SpaceTimeLevyArea,
                               dfx.PIDController(rtol=1e-3, atol=1e-3))).n_save == 1
    with pytest.raises(ValueError, match="error estimates"):
        _lib.Problem(fields(dfx.SEA(), dfx.SpaceTimeLevyArea,
                            dfx.PIDController(rtol=1e-3, atol=1e-3)))
    with pytest.raises(ValueError, match="SDE"):
        dfx.lower(dfx.ODETerm(dfx.OrnsteinUhlenbeck()), dfx.ShARK(), dfx.ConstantStepSize(),
                  dfx.SaveAt(t1=True), dim=2, dtype=torch.float32, max_steps=100, n_ts=0)
    with pytest.raises(ValueError, match="levy_area"):
        dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), levy_area=int)
    # the C ABI checks the same
    with pytest.raises(ValueError, match="levy_area=SpaceTimeLevyArea"):
        _lib.Problem(dict(f, levy_area=0))
    with pytest.raises(ValueError, match="unknown levy_area"):
        _lib.Problem(dict(f, levy_area=2))
    g = dfx.lower(dfx.ODETerm(dfx.OrnsteinUhlenbeck()), dfx.Heun(), dfx.ConstantStepSize(),
                  dfx.SaveAt(t1=True), dim=2, dtype=torch.float32, max_steps=100, n_ts=0)
    with pytest.raises(ValueError, match="Brownian tree of an SDE"):
        _lib.Problem(dict(g, levy_area=1))
    # the extended outputs serve the Ornstein-Uhlenbeck SDE too
    assert _lib.Problem(dfx.lower(terms(dfx.SpaceTimeLevyArea), dfx.ShARK(),
                                  dfx.ConstantStepSize(), dfx.SaveAt(dense=True), dim=2,
                                  dtype=torch.float32, max_steps=100, n_ts=0)).n_save == 0


def test_sde_extended_output_scope():
    # SaveAt(steps / dense), the clip controller and events serve the
    # Ornstein-Uhlenbeck SDE on either tree; the MLP SDE keeps SaveAt(ts / t0 / t1)
    pid = dfx.PIDController(rtol=1e-3, atol=1e-3)
    for levy, solver in ((dfx.BrownianIncrement, dfx.Heun()),
                         (dfx.SpaceTimeLevyArea, dfx.ShARK())):
        bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (2,), key=0, levy_area=levy)
        terms = dfx.MultiTerm(dfx.ODETerm(dfx.OrnsteinUhlenbeck()),
                              dfx.ControlTerm(dfx.OrnsteinUhlenbeck(), bm))
        for saveat, ctrl, event in (
                (dfx.SaveAt(steps=2, t1=True), dfx.ConstantStepSize(), None),
                (dfx.SaveAt(dense=True), dfx.ConstantStepSize(), None),
                (dfx.SaveAt(t1=True), dfx.ClipStepSizeController(pid, step_ts=[0.5]), None),
                (dfx.SaveAt(t1=True), dfx.ConstantStepSize(),
                 dfx.Event(dfx.LinearCondition([1.0, 0.0]), dfx.Newton(1e-5, 1e-5)))):
            f = dfx.lower(terms, solver, ctrl, saveat, dim=2, dtype=torch.float32,
                          max_steps=64, n_ts=0, event=event)
            p = _lib.Problem(f)
            assert p.n_save == (32 if saveat.steps else (0 if saveat.dense else 1))
    # the MLP SDE: step saves, dense steps, the clip controller and events on
    # the fused kernel; not on the plain or tensor-core kernels
    W = [torch.zeros(64, 32), torch.zeros(64, 64), torch.zeros(32, 64)]
    b = [torch.zeros(64), torch.zeros(64), torch.zeros(32)]
    bm = dfx.VirtualBrownianTree(0.0, 1.0, 1e-3, (32,), key=0)
    terms = dfx.MultiTerm(dfx.ODETerm(dfx.MLPField(W, b)),
                          dfx.ControlTerm(dfx.TanhDiagonalDiffusion(torch.zeros(32, 32),
                                                                    torch.zeros(32)), bm))
    for saveat in (dfx.SaveAt(steps=2, t1=True), dfx.SaveAt(dense=True)):
        f = dfx.lower(terms, dfx.Heun(), dfx.ConstantStepSize(), saveat, dim=32,
                      dtype=torch.float32, max_steps=64, n_ts=0)
        assert _lib.Problem(f).n_save == (32 if saveat.steps else 0)
        with pytest.raises(_lib.GbdxError, match="fused kernel"):
            _lib.Problem(dict(f, kernel=1))
    f = dfx.lower(terms, dfx.Heun(), dfx.ClipStepSizeController(pid, step_ts=[0.5]),
                  dfx.SaveAt(t1=True), dim=32, dtype=torch.float32, max_steps=64, n_ts=0)
    assert _lib.Problem(f).n_save == 1
    with pytest.raises(_lib.GbdxError, match="fused kernel"):
        _lib.Problem(dict(f, kernel=3))
    f = dfx.lower(terms, dfx.Heun(), pid, dfx.SaveAt(t1=True), dim=32, dtype=torch.float32,
                  max_steps=64, n_ts=0, event=dfx.Event(dfx.steady_state_event()))
    assert _lib.Problem(f).n_save == 1
    with pytest.raises(_lib.GbdxError, match="fused kernel"):
        _lib.Problem(dict(f, kernel=1))


def test_autotune_cache_round_trip(tmp_path, monkeypatch):
    # GBDX_AUTOTUNE_CACHE: choices written by one process are read by the next
    # (keyed by GPU name, problem and batch class); other GPUs' entries and
    # a corrupt file are ignored.
    from diffrax_gb300 import _tune
    fields = dfx.lower(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(),
                       dfx.PIDController(rtol=1e-6, atol=1e-9), dfx.SaveAt(t1=True), dim=2,
                       dtype=torch.float32, max_steps=4096, n_ts=0)
    key = _tune._key(fields, 65536)
    path = str(tmp_path / "tune.json")
    monkeypatch.setattr(_tune, "_TUNED", {key: ("fused", 128, 4)})
    _tune.save_cache(path, "GPU-A")
    monkeypatch.setattr(_tune, "_TUNED", {})
    assert _tune.load_cache(path, "GPU-B") == 0
    assert _tune.load_cache(path, "GPU-A") == 1
    assert _tune._TUNED[key] == ("fused", 128, 4)
    # a second problem merges into the same file
    f2 = dict(fields, rtol=1e-5)
    k2 = _tune._key(f2, 1000)
    _tune._TUNED[k2] = ("fused", 64, 2)
    _tune.save_cache(path, "GPU-A")
    monkeypatch.setattr(_tune, "_TUNED", {})
    assert _tune.load_cache(path, "GPU-A") == 2
    open(path, "w").write("{not json")
    assert _tune.load_cache(path, "GPU-A") == 0


def test_release_build_has_no_bounds_checks():
    # GBDX_BOUNDS=1 would select libgbdx_bounds.so (covered on the GPU)
    assert _lib.load().gbdx_bounds_checked() == (1 if _lib.bounds_requested() else 0)


def test_bounds_checked_abi_compiles():
    """The bounds-checked boundary (workspace area, record reset and report)
    compiles; the kernels' checks are compiled and run by the GPU test."""
    import subprocess
    from diffrax_gb300 import _build
    obj = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"gbdx_abi_bounds_{os.getpid()}.o")
    src = os.path.join(ROOT, "diffrax_gb300", "csrc", "gbdx_abi.cu")
    cmd = [_build.nvcc()] + _build.NVCC_FLAGS + ["-DGBDX_BOUNDS", "-I",
                                                 os.path.join(ROOT, "include"), "-c", src,
                                                 "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    os.unlink(obj)


def test_max_steps_none_rules():
    # diffrax/_integrate.py:1283-1292, 1316-1319, _adjoint.py:283-292
    from diffrax_gb300._integrate import _max_steps, UNBOUNDED_STEPS
    assert _max_steps(None, dfx.SaveAt(t1=True), False) == UNBOUNDED_STEPS
    assert _max_steps(17, dfx.SaveAt(steps=2), True) == 17
    with pytest.raises(ValueError, match="steps=n"):
        _max_steps(None, dfx.SaveAt(steps=1), False)
    with pytest.raises(ValueError, match="dense=True"):
        _max_steps(None, dfx.SaveAt(dense=True), False)
    with pytest.raises(NotImplementedError, match="finite max_steps"):
        _max_steps(None, dfx.SaveAt(t1=True), True)
    # the C ABI takes INT32_MAX for an unbounded forward solve only
    assert _lib.Problem(_fields(max_steps=UNBOUNDED_STEPS)).n_save == 1
    with pytest.raises(ValueError, match="unbounded"):
        _lib.Problem(_fields(max_steps=UNBOUNDED_STEPS, save_steps=1))


def test_saveat_subs_surface():
    # _saveat.py:14-105: SubSaveAt leaves in a tree; not with t0/t1/ts/steps
    from diffrax_gb300._core import _tree_leaves, _tree_unflatten
    a, b = dfx.SubSaveAt(t1=True), dfx.SubSaveAt(ts=[0.5, 1.0], fn=lambda t, y, args: y)
    tree = {"end": a, "grid": [b]}
    assert _tree_leaves(tree) == [a, b]
    assert _tree_unflatten(tree, [1, 2]) == {"end": 1, "grid": [2]}
    s = dfx.SaveAt(subs=tree, dense=True)
    assert s.subs is tree and not s.state_only
    with pytest.raises(ValueError, match="Cannot pass both"):
        dfx.SaveAt(subs=tree, t1=True)
    with pytest.raises(ValueError, match="Empty saveat"):
        dfx.SubSaveAt()
    with pytest.raises(TypeError):
        dfx.SaveAt(subs=[a, 3])


def test_pid_step_ts_builds_the_clip_controller():
    # pid.py:88-97: PIDController(..., step_ts=, jump_ts=) is the clip wrapper
    c = dfx.PIDController(rtol=1e-3, atol=1e-6, step_ts=[0.5, 1.0], jump_ts=[0.75])
    assert isinstance(c, dfx.ClipStepSizeController)
    assert isinstance(c.controller, dfx.PIDController) and c.controller.rtol == 1e-3
    assert isinstance(dfx.PIDController(rtol=1e-3, atol=1e-6, step_ts=None), dfx.PIDController)


def test_host_device_pointer_rejects_unmapped_memory():
    # zero-copy host I/O takes only page-locked memory the GPU maps: null
    # arguments are invalid, and pageable host memory (or, without a GPU,
    # any memory) is reported as unmapped rather than passed on
    lib = _lib.load()
    out = ctypes.c_void_p()
    assert lib.gbdx_host_device_pointer(None, ctypes.byref(out)) == -1
    buf = ctypes.create_string_buffer(64)
    assert lib.gbdx_host_device_pointer(ctypes.addressof(buf), None) == -1
    assert lib.gbdx_host_device_pointer(ctypes.addressof(buf), ctypes.byref(out)) == -1
    assert out.value is None
    assert _lib.host_device_pointer(ctypes.addressof(buf)) is None
