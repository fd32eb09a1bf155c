"""Pins of the FP64 oracle against the reference's own known-answer tests.

Each test restates a reference test (cited) with the oracle in place of
Diffrax.  The DETEST pin reads the problem definitions from the reference's
test file at run time (it is skipped where the reference tree is absent).
"""
import ast
import math
import os

import numpy as np
import pytest
import scipy.integrate
import scipy.linalg
import scipy.stats

import oracle as O
from conftest import tree_allclose

SOLVERS = [O.EULER, O.HEUN, O.DOPRI5, O.TSIT5, O.DOPRI8]
ORDERS = {O.EULER: 1, O.HEUN: 2, O.DOPRI5: 5, O.TSIT5: 5, O.DOPRI8: 8}


def _decay(**kw):
    # y' = -0.5 y, t in [0.1, 1.1], y0 = 2.1, Dopri5, PID(1e-8, 1e-8), dt0=None
    # (test/test_saveat_solution.py:24-40)
    d = O.make_desc(solver=O.DOPRI5, controller=O.PID, field=O.LINEAR, dim=1, rtol=1e-8,
                    atol=1e-8, **kw)
    return d


def test_saveat_t1_decay():
    # test/test_saveat_solution.py:62-87
    r = O.solve(_decay(save_t1=1), 0.1, 1.1, None, [[2.1]], params=[[-0.5]])
    assert r["ts"][0, 0] == 1.1
    assert tree_allclose(r["ys"][0, 0], 2.1 * math.exp(-0.5))
    assert r["stats"][0, 0] > 0 and r["result"][0] == 0


def test_saveat_t0_decay():
    # test/test_saveat_solution.py:43-60
    r = O.solve(_decay(save_t0=1, save_t1=0), 0.1, 1.1, None, [[2.1]], params=[[-0.5]])
    assert r["ts"].shape == (1, 1) and r["ts"][0, 0] == 0.1 and r["ys"][0, 0, 0] == 2.1


def test_saveat_ts_decay():
    # test/test_saveat_solution.py:96-113
    r = O.solve(_decay(n_ts=2, save_t1=0), 0.1, 1.1, None, [[2.1]], params=[[-0.5]],
                ts=[0.5, 0.8])
    assert r["ts"][0, 0] == 0.5 and r["ts"][0, 1] == 0.8
    assert tree_allclose(r["ys"][0, 0], 2.1 * math.exp(-0.2))
    assert tree_allclose(r["ys"][0, 1], 2.1 * math.exp(-0.35))


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("ctrl", ["constant", "pid", "pi"])
def test_basic_decay(solver, ctrl):
    # y' = -y on [0, 1], dt0 = 0.01 (test/test_integrate.py:48-141)
    if ctrl != "constant" and solver == O.EULER:
        return
    kw = dict(controller=O.CONSTANT) if ctrl == "constant" else dict(
        controller=O.PID, rtol=1e-5, atol=1e-8)
    if ctrl == "pi":
        kw.update(pcoeff=0.3, icoeff=0.3)
    d = O.make_desc(solver=solver, field=O.LINEAR, dim=1, **kw)
    y0 = np.array([[0.7], [-1.3], [2.0]])
    r = O.solve(d, 0.0, 1.0, 0.01, y0, params=[[-1.0]])
    assert tree_allclose(r["ys"][:, 0], y0 * math.exp(-1), rtol=1e-2, atol=1e-2)


@pytest.mark.parametrize("solver", SOLVERS)
def test_ode_order(solver):
    # Linear ODE against expm, fitted order (test/test_integrate.py:144-190).
    rng = np.random.default_rng(5678)
    A = rng.standard_normal((10, 10)) * 0.5
    y0 = rng.standard_normal(10)
    true = scipy.linalg.expm(4.0 * A) @ y0
    d = O.make_desc(solver=solver, controller=O.CONSTANT, field=O.LINEAR, dim=10,
                    max_steps=1 << 20)
    exps, errs = [], []
    for e in [0, -1, -2, -3, -4, -6, -8, -12]:
        r = O.solve(d, 0.0, 4.0, 2.0 ** e, y0[None], params=A)
        err = np.sum(np.abs(r["ys"][0, -1] - true))
        if err < 2 ** -28:
            break
        exps.append(e)
        errs.append(np.log2(err))
    order = scipy.stats.linregress(exps, errs).slope
    assert -0.9 < order - ORDERS[solver] < 0.9


def test_backwards_in_time():
    # t1 < t0 integrates backwards (_integrate.py:1157-1176): y' = -0.5 y from
    # t=1.1 to t=0.1 multiplies by exp(0.5).
    d = _decay(n_ts=2, save_t1=1)
    r = O.solve(d, 1.1, 0.1, None, [[2.1]], params=[[-0.5]], ts=[0.8, 0.5])
    assert tree_allclose(r["ys"][0, 0], 2.1 * math.exp(0.15))
    assert tree_allclose(r["ys"][0, 1], 2.1 * math.exp(0.3))
    assert tree_allclose(r["ys"][0, 2], 2.1 * math.exp(0.5))
    assert r["ts"][0, 0] == 0.8 and r["ts"][0, 2] == 0.1


def test_t0_equals_t1():
    # _integrate.py:823-845: ts are filled with y0, t1 saves y0.
    d = _decay(n_ts=2, save_t1=1)
    r = O.solve(d, 0.3, 0.3, None, [[2.1]], params=[[-0.5]], ts=[0.3, 0.3])
    assert np.all(r["ys"] == 2.1) and r["stats"][0, 0] == 0 and r["result"][0] == 0


def test_max_steps_reached():
    # _integrate.py:883: unfinished solves report max_steps_reached; the t1 save
    # takes the next free slot and later slots stay +inf.
    d = O.make_desc(solver=O.TSIT5, controller=O.CONSTANT, field=O.LINEAR, dim=1, n_ts=3,
                    save_t1=1, max_steps=5)
    r = O.solve(d, 0.0, 1.0, 0.1, [[1.0]], params=[[-1.0]], ts=[0.2, 0.7, 0.9])
    assert r["result"][0] == 1 and r["stats"][0, 0] == 5
    assert np.isfinite(r["ys"][0, 0, 0]) and r["ts"][0, 1] == 0.5
    assert np.all(np.isinf(r["ys"][0, 2:])) and np.all(np.isinf(r["ts"][0, 2:]))


def test_constant_grid():
    # constant.py:48-57, 84-90: N = ceil((t1 - t0) / nextafter(dt0)) steps,
    # t_n = t0 + (t1 - t0) n / N, the last one exactly t1.
    d = O.make_desc(solver=O.EULER, controller=O.CONSTANT, field=O.LINEAR, dim=1)
    r = O.solve(d, 0.0, 1.0, 0.1, [[1.0]], params=[[0.0]])
    assert r["stats"][0, 0] == 10
    r = O.solve(d, 0.0, 1.0, 0.3, [[1.0]], params=[[0.0]])
    assert r["stats"][0, 0] == 4


def test_dtmax_dtmin():
    d = O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.LINEAR, dim=1, rtol=1e-3,
                    atol=1e-6, dtmax=0.05)
    r = O.solve(d, 0.0, 1.0, None, [[1.0]], params=[[-1.0]])
    assert r["stats"][0, 1] >= 20
    d = O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.LINEAR, dim=1, rtol=1e-12,
                    atol=1e-12, dtmin=0.1)
    r = O.solve(d, 0.0, 1.0, 0.1, [[1.0]], params=[[-1.0]])
    assert r["stats"][0, 1] <= 11 and r["result"][0] == 0
    d = O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.LINEAR, dim=1, rtol=1e-12,
                    atol=1e-12, dtmin=0.1, force_dtmin=0)
    r = O.solve(d, 0.0, 1.0, 0.1, [[1.0]], params=[[-1.0]], )
    assert r["result"][0] == 2


# --- local interpolants (test/test_local_interpolation.py:8-60) -------------

def test_hermite_interpolant_exact_on_cubics():
    # A cubic solution is reproduced exactly by Heun's Hermite interpolant when
    # y1 and the endpoint slopes are exact.  With y' = 3 t^2 integrated by Heun
    # the stage slopes are exact and y1 is the trapezoid value, so interpolate
    # y = t^3 on one step and compare with the cubic Hermite formula.
    d = O.make_desc(solver=O.HEUN, controller=O.CONSTANT, field=O.CALLBACK, dim=1, n_ts=3)
    ts = [2.2, 2.6, 3.5]
    r = O.solve(d, 2.0, 3.9, 1.9, [[8.0]], ts=ts, callback=lambda t, y: np.array([3 * t * t]))
    h = 1.9
    y0, y1 = 8.0, 8.0 + 0.5 * h * (3 * 4.0 + 3 * 3.9 ** 2)
    k0, k1 = 3 * 4.0 * h, 3 * 3.9 ** 2 * h
    for i, t in enumerate(ts):
        th = (t - 2.0) / h
        a = k0 + k1 + 2 * y0 - 2 * y1
        b = -2 * k0 - k1 - 3 * y0 + 3 * y1
        assert np.isclose(r["ys"][0, i, 0], ((a * th + b) * th + k0) * th + y0, rtol=1e-13)


@pytest.mark.parametrize("solver", [O.DOPRI5, O.TSIT5])
def test_high_order_interpolants(solver):
    # Dense output of the 5th-order methods is accurate to ~tolerance.
    d = O.make_desc(solver=solver, controller=O.PID, field=O.LINEAR, dim=1, rtol=1e-10,
                    atol=1e-10, n_ts=50, save_t1=0)
    ts = np.linspace(0.0, 3.0, 50)
    r = O.solve(d, 0.0, 3.0, None, [[1.3]], params=[[-0.7]], ts=ts)
    assert np.allclose(r["ys"][0, :, 0], 1.3 * np.exp(-0.7 * ts), rtol=1e-7, atol=1e-9)


# --- DETEST against scipy DOP853 (test/test_detest.py:390-469) --------------

# The reference tree: DIFFRAX_REFERENCE_DIR, else a checkout beside this
# repository.  The test is skipped where neither exists.
REF_DIR = os.environ.get("DIFFRAX_REFERENCE_DIR",
                         os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
                             os.path.abspath(__file__)))), "reference"))
REF_DETEST = os.path.join(REF_DIR, "test", "test_detest.py")


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        arr = self.arr

        class _Set:
            def set(self, v):
                out = np.array(arr, dtype=float).view(_AtArray)
                out[idx] = v
                return out
        return _Set()


class _AtArray(np.ndarray):
    @property
    def at(self):
        return _At(self)


class _JnpShim:
    def __getattr__(self, name):
        fn = getattr(np, name)
        if callable(fn):
            def wrapped(*a, **k):
                out = fn(*a, **k)
                return out.view(_AtArray) if isinstance(out, np.ndarray) else out
            return wrapped
        return fn


class _JaxShim:
    class numpy_rank_promotion:
        def __init__(self, *_):
            pass

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False


def _flatten(tree):
    if isinstance(tree, (tuple, list)):
        parts = [_flatten(x) for x in tree]
        leaves = np.concatenate([p[0] for p in parts]) if parts else np.zeros(0)

        def unflat(v, parts=parts, typ=type(tree)):
            out, i = [], 0
            for (lv, uf) in parts:
                out.append(uf(v[i:i + lv.size]))
                i += lv.size
            return typ(out)
        return leaves, unflat
    a = np.asarray(tree, dtype=float)
    shape = a.shape
    return a.reshape(-1), (lambda v, shape=shape: np.asarray(v).reshape(shape))


def _detest_problems():
    src = open(REF_DETEST).read()
    tree = ast.parse(src)
    ns = {"jnp": _JnpShim(), "jax": _JaxShim(), "math": math, "np": np}
    names = []
    def is_problem(n):
        return n[:2] in ("_a", "_b", "_c", "_d", "_e") and n[2:].isdigit()
    for node in tree.body:
        keep = False
        if isinstance(node, ast.FunctionDef):
            keep = is_problem(node.name) or node.name == "_make_d"
            if is_problem(node.name):
                names.append(node.name)
        elif isinstance(node, ast.Assign) and len(node.targets) == 1 and \
                isinstance(node.targets[0], ast.Name) and is_problem(node.targets[0].id):
            keep = True
            names.append(node.targets[0].id)
        if keep:
            exec(compile(ast.Module(body=[node], type_ignores=[]), REF_DETEST, "exec"), ns)
    return ns, names


@pytest.mark.skipif(not os.path.exists(REF_DETEST), reason="reference tree absent")
@pytest.mark.parametrize("solver", [O.HEUN, O.DOPRI5, O.TSIT5, O.DOPRI8])
def test_detest_against_scipy(solver):
    ns, names = _detest_problems()
    assert len(names) == 25
    checked = 0
    for name in names:
        higher = name[1] != "a"
        if higher and ORDERS[solver] < 4:
            continue
        diffeq, init = ns[name]()
        y0, unflat = _flatten(init)
        if y0.size > 64:
            continue

        def fn(t, y, diffeq=diffeq, unflat=unflat):
            return _flatten(diffeq(t, unflat(y), None))[0]
        tol = 1e-6 if ORDERS[solver] < 4 else 1e-8
        d = O.make_desc(solver=solver, controller=O.PID, field=O.CALLBACK, dim=y0.size,
                        rtol=tol, atol=tol, max_steps=16 ** 4)
        r = O.solve(d, 0.0, 20.0, None, y0[None], callback=fn)
        ref = scipy.integrate.solve_ivp(fn, (0, 20), y0, method="DOP853", rtol=1e-8,
                                        atol=1e-8, t_eval=[20]).y[:, 0]
        t2 = 1e-3 if ORDERS[solver] < 4 else 4e-5
        assert r["result"][0] == 0, name
        assert tree_allclose(r["ys"][0, 0], ref, rtol=t2, atol=t2), name
        checked += 1
    assert checked >= 5


# --- gradients: oracle VJP against central finite differences ---------------
# (test/test_adjoint.py:33-215 checks adjoints against finite differences.)

def _fd_check(desc, t0, t1, dt0, y0, args=None, params=None, ts=None, eps=1e-6, tol=1e-5):
    rng = np.random.default_rng(0)
    n_save = desc.save_t0 + desc.n_ts + desc.save_t1
    gys = rng.standard_normal((y0.shape[0], n_save, desc.dim))

    def loss(y0_, args_, params_):
        r = O.solve(desc, t0, t1, dt0, y0_, args=args_, params=params_, ts=ts)
        return float(np.sum(r["ys"] * gys))
    g = O.grad_recursive(desc, t0, t1, dt0, y0, gys, args=args, params=params, ts=ts)
    # y0
    for i in range(y0.shape[1]):
        e = np.zeros_like(y0)
        e[:, i] = eps
        fd = (loss(y0 + e, args, params) - loss(y0 - e, args, params)) / (2 * eps)
        assert np.isclose(g["grad_y0"][:, i].sum(), fd, rtol=tol, atol=tol)
    if args is not None:
        a = np.asarray(args, dtype=float)
        for i in range(a.shape[-1]):
            e = np.zeros_like(a)
            e[..., i] = eps
            fd = (loss(y0, a + e, params) - loss(y0, a - e, params)) / (2 * eps)
            assert np.isclose(g["grad_args"][:, i].sum(), fd, rtol=tol, atol=tol)
    if params is not None:
        p = np.asarray(params, dtype=float).reshape(-1)
        idx = rng.choice(p.size, size=min(8, p.size), replace=False)
        for j in idx:
            e = np.zeros_like(p)
            e[j] = eps
            fd = (loss(y0, args, p + e) - loss(y0, args, p - e)) / (2 * eps)
            assert np.isclose(g["grad_params"][j], fd, rtol=tol, atol=tol)
    return g


@pytest.mark.parametrize("solver", [O.EULER, O.HEUN, O.DOPRI5, O.TSIT5])
def test_grad_lotka_volterra_constant_steps(solver):
    # With a fixed grid the discrete map is smooth: FD and VJP agree tightly.
    d = O.make_desc(solver=solver, controller=O.CONSTANT, field=O.LOTKA_VOLTERRA, dim=2,
                    n_ts=5, save_t1=1, n_args=4)
    y0 = np.array([[10.0, 5.0], [7.0, 12.0]])
    _fd_check(d, 0.0, 10.0, 0.05, y0, args=np.array([0.1, 0.02, 0.4, 0.02]),
              ts=np.linspace(0, 10, 5), tol=1e-6)


@pytest.mark.parametrize("solver", [O.HEUN, O.DOPRI5, O.TSIT5])
def test_grad_lotka_volterra_pid(solver):
    # Under PID the controller is stop-gradient (pid.py:374, 499-501, 529-530);
    # FD also sees dt's dependence on the state, which shrinks with the
    # tolerance, so compare at a tight tolerance.
    tol = 1e-10 if solver != O.HEUN else 1e-7
    d = O.make_desc(solver=solver, controller=O.PID, field=O.LOTKA_VOLTERRA, dim=2,
                    rtol=tol, atol=tol, n_ts=5, save_t1=1, n_args=4, max_steps=100000)
    y0 = np.array([[10.0, 5.0], [7.0, 12.0]])
    _fd_check(d, 0.0, 10.0, 0.1, y0, args=np.array([0.1, 0.02, 0.4, 0.02]),
              ts=np.linspace(0, 10, 5), tol=1e-5 if solver != O.HEUN else 1e-3)


def test_grad_van_der_pol_per_trajectory_args():
    d = O.make_desc(solver=O.DOPRI5, controller=O.PID, field=O.VAN_DER_POL, dim=2, rtol=1e-10,
                    atol=1e-12, pcoeff=0.3, icoeff=0.4, save_t1=1, n_args=1)
    y0 = np.array([[1.0, -0.5], [0.3, 1.5]])
    _fd_check(d, 0.0, 5.0, None, y0, args=np.array([[1.3], [0.4]]), tol=1e-5)


def test_grad_mlp():
    rng = np.random.default_rng(3)
    widths = [4, 8, 8, 4]
    P = []
    for i in range(3):
        P.append(rng.standard_normal((widths[i + 1], widths[i])) / np.sqrt(widths[i]))
        P.append(rng.standard_normal(widths[i + 1]) * 0.1)
    params = np.concatenate([p.reshape(-1) for p in P])
    d = O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.MLP, dim=4, rtol=1e-10,
                    atol=1e-10, save_t1=1, mlp_depth=3, mlp_widths=widths)
    y0 = rng.standard_normal((3, 4))
    _fd_check(d, 0.0, 1.0, None, y0, params=params, tol=1e-5)


def test_grad_sde_heun_tanh_diffusion():
    rng = np.random.default_rng(4)
    widths = [3, 6, 3]
    P = []
    for i in range(2):
        P.append(rng.standard_normal((widths[i + 1], widths[i])) / np.sqrt(widths[i]))
        P.append(np.zeros(widths[i + 1]))
    P.append(rng.standard_normal((3, 3)) / np.sqrt(3))
    P.append(rng.standard_normal(3) * 0.1)
    params = np.concatenate([p.reshape(-1) for p in P])
    d = O.make_desc(solver=O.HEUN, controller=O.CONSTANT, field=O.MLP, dim=3, save_t1=1,
                    mlp_depth=2, mlp_widths=widths, diffusion=O.DIFF_TANH_DIAG,
                    vbt_t0=0.0, vbt_t1=1.0, vbt_tol=1e-3, seed=99)
    y0 = rng.standard_normal((2, 3))
    _fd_check(d, 0.0, 1.0, 0.01, y0, params=params, tol=1e-5)


# --- BacksolveAdjoint (test/test_adjoint.py:33-215) ---------------------------

_BS_A = np.array([[0.1, -1.0], [1.0, -0.1]])  # _VectorField with args (0.1, -1), (1, -0.1)


def _linear_exact_grads(A, y0, t0, saved_ts, G):
    """dL/dy0 and dL/dA of L = sum_k <G_k, y(t_k)> for y' = A y, exactly:
    exp(A^T tau) G_k and the Frechet derivative of the matrix exponential."""
    gy = np.zeros(A.shape[0])
    gA = np.zeros_like(A)
    for tk, g in zip(saved_ts, G):
        tau = tk - t0
        gy += scipy.linalg.expm(A.T * tau) @ g
        if tau > 0:
            gA += scipy.linalg.expm_frechet(A.T * tau, tau * np.outer(g, y0),
                                            compute_expm=False)
    return gy, gA


@pytest.mark.parametrize("save_t0", [1, 0])
@pytest.mark.parametrize("save_t1", [1, 0])
@pytest.mark.parametrize("ts", [None, [0.3], [2.0], [9.5], [1.0, 7.0], [0.3, 7.0, 9.5]])
def test_backsolve_against_recursive_and_exact(save_t0, save_t1, ts):
    # test/test_adjoint.py:139-163: on y' = A y over [0.3, 9.5], Tsit5 with
    # PID(1e-8, 1e-8) and dt0=None, BacksolveAdjoint agrees with the
    # discretise-then-optimise gradient at atol 1e-5 for every SaveAt.
    if not save_t0 and not save_t1 and ts is None:
        pytest.skip("empty SaveAt")
    d = O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.LINEAR, dim=2, rtol=1e-8,
                    atol=1e-8, save_t0=save_t0, save_t1=save_t1,
                    n_ts=0 if ts is None else len(ts))
    y0 = np.array([[0.9, 5.4]])
    fwd = O.solve(d, 0.3, 9.5, None, y0, params=_BS_A, ts=ts)
    G = np.ones_like(fwd["ys"])
    rec = O.grad_recursive(d, 0.3, 9.5, None, y0, G, params=_BS_A, ts=ts)
    bs = O.backsolve(d, 0.3, 9.5, None, fwd["ts"], fwd["ys"], G, params=_BS_A)
    assert bs["result"][0] == 0
    assert tree_allclose(bs["grad_y0"], rec["grad_y0"], atol=1e-5)
    assert tree_allclose(bs["grad_params"], rec["grad_params"], atol=1e-5)
    gy, gA = _linear_exact_grads(_BS_A, y0[0], 0.3, fwd["ts"][0], G[0])
    assert tree_allclose(bs["grad_y0"][0], gy, atol=1e-5)
    assert tree_allclose(bs["grad_params"].reshape(2, 2), gA, atol=1e-5)


@pytest.mark.parametrize("solver", ["TSIT5", "DOPRI5"])
def test_backsolve_steps_equal_a_forward_solve_of_the_adjoint_system(solver):
    # Under adjoint_rms_seminorm the error norm covers (y, a) only, and for
    # y' = A y the (y, a) part of AdjointTerm.vf (_term.py:886-910) is the
    # linear field z' = blockdiag(A, -A^T) z.  One backward segment (SaveAt(t1))
    # must therefore take exactly the steps of a forward solve of that system
    # from t1 to t0 with the same controller and dt0 -- including the retries
    # after rejected steps, whose first stage is f at the unchanged state
    # (the solver state of a rejected step is kept, _integrate.py:424).
    kw = dict(solver=getattr(O, solver), controller=O.PID, rtol=1e-8, atol=1e-8, save_t1=1)
    d = O.make_desc(field=O.LINEAR, dim=2, norm=O.NORM_ADJOINT_SEMI, **kw)
    y0 = np.array([[0.9, 5.4]])
    fwd = O.solve(d, 0.3, 9.5, 3.0, y0, params=_BS_A)
    G = np.array([[[0.7, -1.3]]])
    bs = O.backsolve(d, 0.3, 9.5, 3.0, fwd["ts"], fwd["ys"], G, params=_BS_A)
    M = np.zeros((4, 4))
    M[:2, :2] = _BS_A
    M[2:, 2:] = -_BS_A.T
    d4 = O.make_desc(field=O.LINEAR, dim=4, **kw)
    z0 = np.concatenate([fwd["ys"][0, -1], G[0, -1]])[None]
    aug = O.solve(d4, 9.5, 0.3, -3.0, z0, params=M)
    assert bs["result"][0] == 0 and aug["result"][0] == 0
    assert bs["stats"][0, 2] > 0  # the large dt0 forces rejections
    assert np.array_equal(bs["stats"], aug["stats"])
    assert np.allclose(bs["grad_y0"][0], aug["ys"][0, -1, 2:], rtol=1e-12, atol=0)


def test_backsolve_seminorm():
    # adjoint_rms_seminorm (_misc.py:85-116) drops a_args and a_theta from the
    # error norm: fewer steps, same gradient to the tolerance.
    kw = dict(solver=O.TSIT5, controller=O.PID, field=O.LINEAR, dim=2, rtol=1e-8, atol=1e-8,
              n_ts=2, save_t1=1)
    d = O.make_desc(**kw)
    ds = O.make_desc(norm=O.NORM_ADJOINT_SEMI, **kw)
    y0 = np.array([[0.9, 5.4]])
    ts = [1.0, 7.0]
    fwd = O.solve(d, 0.3, 9.5, None, y0, params=_BS_A, ts=ts)
    G = np.ones_like(fwd["ys"])
    full = O.backsolve(d, 0.3, 9.5, None, fwd["ts"], fwd["ys"], G, params=_BS_A)
    semi = O.backsolve(ds, 0.3, 9.5, None, fwd["ts"], fwd["ys"], G, params=_BS_A)
    assert semi["stats"][0, 0] != full["stats"][0, 0]
    gy, gA = _linear_exact_grads(_BS_A, y0[0], 0.3, fwd["ts"][0], G[0])
    assert tree_allclose(semi["grad_y0"][0], gy, atol=1e-5)
    assert tree_allclose(semi["grad_params"].reshape(2, 2), gA, rtol=1e-4, atol=1e-5)


def test_backsolve_mlp_converges_to_recursive():
    # Optimise-then-discretise and discretise-then-optimise gradients agree as
    # the tolerance shrinks (both converge to the continuous gradient).
    rng = np.random.default_rng(5)
    widths = [4, 8, 8, 4]
    P = []
    for i in range(3):
        P.append(rng.standard_normal((widths[i + 1], widths[i])) / np.sqrt(widths[i]))
        P.append(rng.standard_normal(widths[i + 1]) * 0.1)
    params = np.concatenate([p.reshape(-1) for p in P])
    y0 = rng.standard_normal((3, 4))
    ts = np.linspace(0.0, 1.0, 5)
    errs = []
    for tol in (1e-5, 1e-8):
        d = O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.MLP, dim=4, rtol=tol,
                        atol=tol, n_ts=5, mlp_depth=3, mlp_widths=widths)
        fwd = O.solve(d, 0.0, 1.0, None, y0, params=params, ts=ts)
        G = rng.standard_normal(fwd["ys"].shape)
        rec = O.grad_recursive(d, 0.0, 1.0, None, y0, G, params=params, ts=ts)
        bs = O.backsolve(d, 0.0, 1.0, None, fwd["ts"], fwd["ys"], G, params=params)
        scale = max(np.abs(rec["grad_params"]).max(), np.abs(rec["grad_y0"]).max())
        errs.append(max(np.abs(bs["grad_params"] - rec["grad_params"]).max(),
                        np.abs(bs["grad_y0"] - rec["grad_y0"]).max()) / scale)
    assert errs[1] < 1e-6 and errs[1] < errs[0] / 10


def test_backsolve_constant_steps_converge():
    # ConstantStepSize: the backward reuses the forward's controller; its
    # carried state extends the first segment's grid (constant.py:59-104).
    # Halving dt0 shrinks the Heun gradient error ~4x.  (With a zero-length
    # first segment, e.g. SaveAt(ts=[..., t1], t1=True), that grid has zero
    # steps and the reference's constant controller produces NaN times.)
    y0 = np.array([[0.9, 5.4]])
    ts = [1.0, 2.5, 4.0]
    errs = []
    for dt0 in (0.02, 0.01):
        d = O.make_desc(solver=O.HEUN, controller=O.CONSTANT, field=O.LINEAR, dim=2, n_ts=3,
                        save_t1=0)
        fwd = O.solve(d, 0.3, 4.0, dt0, y0, params=_BS_A, ts=ts)
        G = np.ones_like(fwd["ys"])
        bs = O.backsolve(d, 0.3, 4.0, dt0, fwd["ts"], fwd["ys"], G, params=_BS_A)
        gy, gA = _linear_exact_grads(_BS_A, y0[0], 0.3, fwd["ts"][0], G[0])
        errs.append(np.abs(bs["grad_params"].reshape(2, 2) - gA).max())
    assert 3.0 < errs[0] / errs[1] < 5.0


# --- virtual Brownian tree statistics (test/test_brownian.py:117-494) --------

def test_vbt_increment_distribution():
    d = O.make_desc(dim=4, vbt_t0=0.0, vbt_t1=1.0, vbt_tol=1e-3, seed=7)
    n = 4000
    traj = np.arange(n, dtype=np.uint32)
    ta = np.full(n, 0.23)
    tb = np.full(n, 0.61)
    w = O.vbt_increments(d, traj, ta, tb)
    z = (w / np.sqrt(0.61 - 0.23)).reshape(-1)
    assert scipy.stats.kstest(z, "norm").pvalue > 1e-3
    # Chen's relation is exact and disjoint increments are uncorrelated.
    w1 = O.vbt_increments(d, traj, ta, np.full(n, 0.4))
    w2 = O.vbt_increments(d, traj, np.full(n, 0.4), tb)
    assert np.allclose(w1 + w2, w, atol=1e-12)
    assert abs(np.corrcoef(w1.reshape(-1), w2.reshape(-1))[0, 1]) < 0.05


def test_vbt_conditional_bridge():
    # W(s) given W(0)=0 and W(1) has mean s W(1) and variance s (1 - s).
    d = O.make_desc(dim=1, vbt_t0=0.0, vbt_t1=1.0, vbt_tol=2 ** -12, seed=3)
    n = 20000
    traj = np.arange(n, dtype=np.uint32)
    w1 = O.vbt_increments(d, traj, np.zeros(n), np.ones(n))[:, 0]
    s = 0.37
    ws = O.vbt_increments(d, traj, np.zeros(n), np.full(n, s))[:, 0]
    resid = (ws - s * w1) / np.sqrt(s * (1 - s))
    assert scipy.stats.kstest(resid, "norm").pvalue > 1e-3
    assert abs(np.corrcoef(resid, w1)[0, 1]) < 0.03


# --- the tree with space-time Levy area (test/test_brownian.py) ------------

def test_levy_tree_statistics():
    # test/test_brownian.py:120-175: over [0, 5] with tol 2^-5, W ~ N(0, 5),
    # H ~ N(0, 5/12), and W and H uncorrelated.
    d = O.make_desc(dim=1, vbt_t0=0.0, vbt_t1=5.0, vbt_tol=2 ** -5, seed=5678)
    n = 200000
    traj = np.arange(n, dtype=np.uint32)
    w, h = O.vbt_levy_increments(d, traj, np.zeros(n), np.full(n, 5.0))
    w, h = w[:, 0], h[:, 0]
    assert scipy.stats.kstest(h, scipy.stats.norm(0, math.sqrt(5 / 12)).cdf).pvalue > 0.1
    assert scipy.stats.kstest(w, scipy.stats.norm(0, math.sqrt(5)).cdf).pvalue > 0.1
    assert abs(np.mean(h * w)) < 0.01


def _true_cond_stats_wh(w_s, h_s, w_u, h_u, s, r, u):
    # Law of (W_r, H_r) given (W_s, H_s, W_u, H_u), H = H_{0,.}: Foster's
    # bridge as the reference's test writes it (test/test_brownian.py:183-211).
    su, sr, ru = u - s, r - s, u - r
    sr3, ru3, su2 = sr ** 3, ru ** 3, su ** 2
    sr_ru_half = math.sqrt(sr * ru)
    dd = math.sqrt(sr3 + ru3)
    a = sr3 * sr_ru_half / (2 * su * dd)
    b = ru3 * sr_ru_half / (2 * su * dd)
    c = sr ** 1.5 * ru ** 1.5 / (math.sqrt(12) * dd)
    h_su = (u * h_u - s * h_s - u / 2 * w_s + s / 2 * w_u) / su
    w_mean = w_s + (sr / su) * (w_u - w_s) + (6 * sr * ru / su2) * h_su
    w_std = 2 * (a + b) / su
    h_mean = (s / r) * h_s + (sr3 / (r * su2)) * h_su + 0.5 * w_s - s / (2 * r) * w_mean
    h_std = math.sqrt((c / r) ** 2 + ((a * u + s * b) / (r * su)) ** 2)
    return w_mean, w_std, h_mean, h_std


def test_levy_tree_conditional_statistics():
    # test/test_brownian.py:276-490 (SpaceTimeLevyArea, use_levy=True):
    # evaluate(t0, t_i) on many paths at sorted times at least 2^-8 apart; the
    # middle of each consecutive triple, normalised by its conditional law
    # given the outer two, is N(0, 1) (KS at 0.1 with a Bonferroni correction).
    t0, t1 = 0.0, 8.7
    d = O.make_desc(dim=1, vbt_t0=t0, vbt_t1=t1, vbt_tol=2 ** -10, seed=5680)
    rng = np.random.default_rng(5680)
    ts = np.sort(rng.uniform(t0 + 0.1, t1 - 0.1, 40))
    keep = [ts[0]]
    for t in ts[1:]:
        if t >= keep[-1] + 2 ** -8:
            keep.append(t)
    ts = np.array(keep)
    n = 20000
    traj = np.arange(n, dtype=np.uint32)
    vals = [O.vbt_levy_increments(d, traj, np.full(n, t0), np.full(n, t)) for t in ts]
    pw1, pw2, ph = [], [], []
    for i in range(1, len(ts) - 1):
        s, r, u = ts[i - 1] - t0, ts[i] - t0, ts[i + 1] - t0
        (w_s, h_s), (w_r, h_r), (w_u, h_u) = [(v[0][:, 0], v[1][:, 0]) for v in vals[i - 1:i + 2]]
        w_mean1 = w_s + (w_u - w_s) * (r - s) / (u - s)
        w_std1 = math.sqrt((u - r) * (r - s) / (u - s))
        pw1.append(scipy.stats.kstest((w_r - w_mean1) / w_std1, "norm").pvalue)
        w_mean, w_std, h_mean, h_std = _true_cond_stats_wh(w_s, h_s, w_u, h_u, s, r, u)
        pw2.append(scipy.stats.kstest((w_r - w_mean) / w_std, "norm").pvalue)
        ph.append(scipy.stats.kstest((h_r - h_mean) / h_std, "norm").pvalue)
    m = len(pw1)
    assert m >= 10
    assert min(pw1) > 0.1 / m and min(pw2) > 0.1 / m and min(ph) > 0.1 / m


def test_levy_tree_reverse_time():
    # test/test_brownian.py:679-695: increments over reversed intervals are
    # the negated forward ones (W); H of [b, a] by Chen's relation equals H
    # of [a, b].
    d = O.make_desc(dim=1, vbt_t0=0.0, vbt_t1=5.0, vbt_tol=2 ** -5, seed=5678)
    rng = np.random.default_rng(1)
    ts = rng.uniform(0, 5, 100)
    traj = np.zeros(99, dtype=np.uint32)
    wf, hf = O.vbt_levy_increments(d, traj, ts[:-1], ts[1:])
    wb, hb = O.vbt_levy_increments(d, traj, ts[1:], ts[:-1])
    assert np.allclose(wf, -wb, atol=1e-13)
    assert np.allclose(hf, hb, atol=1e-9)


def _nonlinear_additive_sde(solver, level, n=100, t0=0.3, t1=5.3):
    # An additive-noise SDE in the spirit of the reference's get_time_sde
    # (test/helpers.py:452-491): a bounded nonlinear drift with cubic damping
    # and a constant diffusion, on a Levy area tree with tol 2^-14; steps of
    # (t1 - t0) / 2^level land on every SaveAt time of the coarsest level.
    d = O.make_desc(solver=solver, controller=O.CONSTANT, field=O.CALLBACK, dim=2, n_ts=3,
                    save_t1=0, diffusion=O.DIFF_OU, vbt_t0=t0, vbt_t1=t1, vbt_tol=2 ** -14,
                    seed=5678, levy_area=1, n_args=3)

    def drift(t, y):
        return (0.5 * np.sin(3 * y[::-1]) - 0.5 * y ** 3) / ((y * y).sum() + 1.0)

    y0 = np.tile([0.7, -0.4], (n, 1))
    r = O.solve(d, t0, t1, (t1 - t0) / 2 ** level, y0, args=[0.0, 0.0, 1.0],
                ts=np.linspace(t0, t1, 3), callback=drift)
    assert (r["result"] == 0).all()
    return r["ys"], r["stats"][:, 0].mean()


def _path_l2_dist(a, b):
    # test/helpers.py:97-116: sqrt(mean over paths of sup over the saves of
    # the squared distance)
    return math.sqrt(np.mean(np.max(((a - b) ** 2).sum(-1), axis=1)))


@pytest.mark.parametrize("solver, theoretical", [(O.SHARK, 1.5), (O.SRA1, 1.5), (O.SEA, 1.0)])
def test_additive_srk_strong_order(solver, theoretical):
    # test/test_sde1.py:16-91 (ShARK, SRA1 and SEA on additive noise, orders
    # 1.5, 1.5, 1.0): levels 1..7 against the solver itself at level 9, order
    # by a log-log fit, within 0.4 of the theoretical order.
    ref, _ = _nonlinear_additive_sde(solver, 9)
    errs, steps = [], []
    for level in range(1, 8):
        ys, n = _nonlinear_additive_sde(solver, level)
        errs.append(_path_l2_dist(ys, ref))
        steps.append(n)
    order = np.polyfit(np.log(1 / np.array(steps)), np.log(errs), 1)[0]
    assert -0.4 < order - theoretical < 0.4, order


def test_additive_srk_limit_is_heuns_limit():
    # test/test_sde1.py:118-190: the SRKs and Heun (all Stratonovich; the
    # noise is additive) converge to the same solution on the same tree:
    # Heun's distance to ShARK at a fine level shrinks as Heun refines, and
    # SRA1 and SEA at fine levels are as close to ShARK as Heun is.
    ref, _ = _nonlinear_additive_sde(O.SHARK, 9)
    e = [_path_l2_dist(_nonlinear_additive_sde(O.HEUN, lv)[0], ref) for lv in (7, 9, 11)]
    assert e[0] > 2.5 * e[1] > 6 * e[2], e
    assert e[2] < 2e-3, e
    assert _path_l2_dist(_nonlinear_additive_sde(O.SRA1, 9)[0], ref) < 2e-3
    assert _path_l2_dist(_nonlinear_additive_sde(O.SEA, 11)[0], ref) < 2e-3


@pytest.mark.parametrize("solver, levy", [(O.HEUN, 0), (O.SHARK, 1)])
def test_sde_extended_outputs_agree(solver, levy):
    # On one Brownian path and a constant-step grid: SaveAt(steps=1) saves the
    # step ends, SaveAt(ts=grid) interpolates to the same points, and the dense
    # output evaluated there gives them again (_integrate.py:456-540).
    kw = dict(solver=solver, controller=O.CONSTANT, field=O.ORNSTEIN_UHLENBECK, dim=2,
              diffusion=O.DIFF_OU, vbt_t0=0.0, vbt_t1=1.0, vbt_tol=1e-3, seed=23,
              levy_area=levy, n_args=3, max_steps=20, save_t1=0)
    rng = np.random.default_rng(5)
    y0 = rng.uniform(-1, 1, (16, 2))
    args = [1.5, 0.5, 0.6]
    grid = np.linspace(0.05, 1.0, 20)
    a = O.solve(O.make_desc(save_steps=1, **kw), 0.0, 1.0, 0.05, y0, args=args)
    b = O.solve(O.make_desc(n_ts=20, **kw), 0.0, 1.0, 0.05, y0, args=args, ts=grid)
    assert np.allclose(a["ts"], grid[None, :], rtol=0, atol=1e-15)
    assert np.allclose(a["ys"], b["ys"], rtol=1e-12, atol=1e-12)
    d = O.make_desc(save_dense=1, save_t1=1, **{k: v for k, v in kw.items() if k != "save_t1"})
    c = O.solve(d, 0.0, 1.0, 0.05, y0, args=args)
    q = O.dense_evaluate(d, 0.0, 1.0, y0, c, grid)
    assert np.allclose(q, a["ys"], rtol=1e-12, atol=1e-12)


def test_srk_needs_levy_area():
    # srk.py:374-379: a tree without the space-time Levy area is rejected;
    # SEA has no error estimate for adaptive steps (pid.py:437-447).
    for solver in (O.SHARK, O.SRA1, O.SEA):
        d = O.make_desc(solver=solver, controller=O.CONSTANT, field=O.ORNSTEIN_UHLENBECK,
                        dim=2, diffusion=O.DIFF_OU, levy_area=0, n_args=3)
        with pytest.raises(ValueError):
            O.solve(d, 0.0, 1.0, 0.1, np.zeros((1, 2)), args=[1.0, 0.0, 1.0])
    d = O.make_desc(solver=O.SEA, controller=O.PID, field=O.ORNSTEIN_UHLENBECK, dim=2,
                    diffusion=O.DIFF_OU, levy_area=1, n_args=3)
    with pytest.raises(ValueError):
        O.solve(d, 0.0, 1.0, 0.1, np.zeros((1, 2)), args=[1.0, 0.0, 1.0])


# ---------------------------------------------------------------------------
# SaveAt(steps=n) and SaveAt(dense=True)
# ---------------------------------------------------------------------------

def test_saveat_steps_decay():
    # test/test_saveat_solution.py:116-180: shapes (max_steps // n, plus a t1
    # slot only when max_steps % n != 0) and the analytic values at the saved ts
    for steps, t1, n in ((1, 0, 4096), (2, 0, 2048), (2, 1, 2048), (3, 1, 1366)):
        d = _decay(save_steps=steps, save_t1=t1)
        assert O.n_saves(d) == n
        r = O.solve(d, 0.1, 1.1, None, [[2.1]], params=[[-0.5]])
        assert r["ys"].shape == (1, n, 1) and r["result"][0] == 0
        ts = r["ts"][0]
        fin = np.isfinite(ts)
        assert fin.sum() >= 1 and np.all(np.isinf(ts[~fin])) and np.all(ts[~fin] > 0)
        assert np.all(np.diff(ts[fin]) > 0)
        np.testing.assert_allclose(r["ys"][0, fin, 0], 2.1 * np.exp(-0.5 * (ts[fin] - 0.1)),
                                   rtol=1e-5, atol=1e-8)
        assert np.all(np.isinf(r["ys"][0, ~fin, 0]))
        nacc = r["stats"][0, 1]
        assert fin.sum() == nacc // steps + (t1 and nacc % steps != 0)
        assert ts[fin][-1] == 1.1 or (steps > 1 and nacc % steps != 0 and not t1)


@pytest.mark.parametrize("with_7", [True, False])
def test_saveat_steps_skip(with_7):
    # test/test_saveat_solution.py:198-247: Euler on the unit grid 0..7 (or
    # 0..6); the reference's StepTo(ts) grid is ConstantStepSize(dt0=1) here
    t1 = 7.0 if with_7 else 6.0
    cases = [((2, 0, 0), [2, 4, 6], [2, 4, 6]),
             ((2, 1, 0), [2, 4, 6, 7], [2, 4, 6]),
             ((2, 1, 1), [0, 2, 4, 6, 7], [0, 2, 4, 6]),
             ((3, 0, 0), [3, 6], [3, 6]),
             ((3, 1, 0), [3, 6, 7], [3, 6]),
             ((3, 1, 1), [0, 3, 6, 7], [0, 3, 6])]
    for (steps, st1, st0), want7, want6 in cases:
        d = O.make_desc(solver=O.EULER, controller=O.CONSTANT, field=O.LINEAR, dim=1,
                        save_steps=steps, save_t1=st1, save_t0=st0, max_steps=10)
        r = O.solve(d, 0.0, t1, 1.0, [[1.0]], params=[[-0.5]])
        ts = r["ts"][0]
        assert list(ts[np.isfinite(ts)]) == (want7 if with_7 else want6)


def test_saveat_steps_vs_ts():
    # test/test_saveat_solution.py:250-279: steps=2 with t0 saves the same
    # points as ts=[0, 2, 4, 6] on the unit grid
    d = O.make_desc(solver=O.EULER, controller=O.CONSTANT, field=O.LINEAR, dim=1,
                    save_steps=2, save_t0=1, save_t1=0, max_steps=6)
    r = O.solve(d, 0.0, 6.0, 1.0, [[1.0]], params=[[-0.5]])
    d2 = O.make_desc(solver=O.EULER, controller=O.CONSTANT, field=O.LINEAR, dim=1,
                     n_ts=4, save_t1=0, max_steps=6)
    r2 = O.solve(d2, 0.0, 6.0, 1.0, [[1.0]], params=[[-0.5]], ts=[0.0, 2.0, 4.0, 6.0])
    assert np.array_equal(r["ts"], r2["ts"]) and np.array_equal(r["ys"], r2["ys"])


def test_saveat_t0_eq_t1_steps():
    # test/test_saveat_solution.py:323-368 (the steps=1 sub): y0 at t0 and the
    # three ts, then max_steps infs
    d = O.make_desc(solver=O.DOPRI5, controller=O.CONSTANT, field=O.LINEAR, dim=1,
                    save_t0=1, n_ts=3, save_t1=0, save_steps=1, max_steps=256)
    r = O.solve(d, 1.0, 1.0, 0.1, [[2.0]], params=[[1.0]], ts=[1.0, 1.0, 1.0])
    assert r["ys"].shape == (1, 4 + 256, 1)
    assert np.all(r["ys"][0, :4, 0] == 2.0) and np.all(np.isinf(r["ys"][0, 4:, 0]))


def test_dense_decay():
    # test/test_saveat_solution.py:182-195: evaluate(0.2), evaluate(0.8),
    # evaluate(0.2, 0.8) as the difference, derivative(0.2)
    d = _decay(save_dense=1, save_t1=1)
    r = O.solve(d, 0.1, 1.1, None, [[2.1]], params=[[-0.5]])
    assert r["dense_n"][0] == r["stats"][0, 1] + 1
    assert r["dense_ts"][0, 0] == 0.1 and r["dense_ts"][0, r["dense_n"][0] - 1] == 1.1
    assert np.all(np.isinf(r["dense_ts"][0, r["dense_n"][0]:]))
    v = O.dense_evaluate(d, 0.1, 1.1, [[2.1]], r, [0.2, 0.8])
    assert tree_allclose(v[0, 0, 0], 2.1 * math.exp(-0.05))
    assert tree_allclose(v[0, 1, 0], 2.1 * math.exp(-0.35))
    g = O.dense_evaluate(d, 0.1, 1.1, [[2.1]], r, [0.2], order=1)
    assert tree_allclose(g[0, 0, 0], -0.5 * 2.1 * math.exp(-0.05))
    # outside [t0, t1]: NaN (_global_interpolation.py:367-378)
    o = O.dense_evaluate(d, 0.1, 1.1, [[2.1]], r, [0.0, 1.2])
    assert np.all(np.isnan(o))


def test_dense_trivial():
    # test/test_saveat_solution.py:431-447: t0 == t1 evaluates to y0 at t0
    d = _decay(save_dense=1)
    r = O.solve(d, 2.0, 2.0, None, [[2.1]], params=[[-0.5]])
    assert r["dense_n"][0] == 1
    v = O.dense_evaluate(d, 2.0, 2.0, [[2.1]], r, [2.0, 2.5])
    assert v[0, 0, 0] == 2.1 and np.isnan(v[0, 1, 0])


@pytest.mark.parametrize("solver", SOLVERS)
def test_dense_matches_saveat_ts_and_derivative(solver):
    # The dense interpolant at the ts equals SaveAt(ts) (both evaluate the
    # step's local interpolation, _integrate.py:456-487 and
    # _global_interpolation.py:339-353); the derivative matches the vector
    # field to the interpolant's accuracy, and a central difference of the
    # interpolant, left and right limits, and reverse time
    A = np.array([[-0.3, 1.0], [-1.0, -0.3]])
    ctrl = (dict(controller=O.CONSTANT) if solver == O.EULER else
            dict(rtol=1e-6, atol=1e-8) if solver == O.HEUN else dict(rtol=1e-8, atol=1e-10))
    dt0 = 0.01 if solver == O.EULER else None
    for t0, t1 in ((0.0, 3.0), (3.0, 0.0)):
        ts = np.linspace(t0, t1, 9)[1:-1]
        d = O.make_desc(solver=solver, field=O.LINEAR, dim=2, save_dense=1, save_t1=0,
                        n_ts=len(ts), **ctrl)
        r = O.solve(d, t0, t1, None if dt0 is None else math.copysign(dt0, t1 - t0),
                    [[1.0, 0.5]], params=A, ts=ts)
        assert r["result"][0] == 0
        v = O.dense_evaluate(d, t0, t1, [[1.0, 0.5]], r, ts)
        np.testing.assert_allclose(v[0], r["ys"][0], rtol=1e-13, atol=1e-14)
        # derivative away from the step boundaries (Euler's interpolant has a
        # kink at each one)
        tq = ts + math.copysign(0.0031, t1 - t0)
        g = O.dense_evaluate(d, t0, t1, [[1.0, 0.5]], r, tq, order=1)
        h = 1e-6
        fd = (O.dense_evaluate(d, t0, t1, [[1.0, 0.5]], r, tq + h) -
              O.dense_evaluate(d, t0, t1, [[1.0, 0.5]], r, tq - h)) / (2 * h)
        np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-7)
        vq = O.dense_evaluate(d, t0, t1, [[1.0, 0.5]], r, tq)
        tol = 0.05 if solver == O.EULER else 1e-4
        np.testing.assert_allclose(g[0], vq[0] @ A.T, rtol=tol, atol=tol * 1e-1)
        # at a step boundary the left and right limits use the two neighbouring steps
        kb = r["dense_ts"][0, 3] * (1 if t1 > t0 else -1)
        lv = O.dense_evaluate(d, t0, t1, [[1.0, 0.5]], r, [kb], left=True)
        rv = O.dense_evaluate(d, t0, t1, [[1.0, 0.5]], r, [kb], left=False)
        np.testing.assert_allclose(lv, rv, rtol=1e-12, atol=1e-13)


# ---------------------------------------------------------------------------
# ClipStepSizeController(step_ts, jump_ts) (clip.py)
# ---------------------------------------------------------------------------

def test_clip_find_idx_with_hint():
    # test/test_adaptive_stepsize_controller.py:284-292: the first index
    # strictly greater than t, whatever the hint
    ts = np.arange(5.0)
    for hint in (0, 2, 3, 5):
        assert O.clip_find(ts, 2.5, hint) == 3
        assert O.clip_find(ts, 2.0, hint) == 3
        assert O.clip_find(ts, 1.9, hint) == 2
    # backwards in time the array is sort(-ts) = [-4, ..., 0]
    assert O.clip_find(ts, -2.5, 0, direction=-1) == 2


def test_clip_adapt_known_answers():
    # clip.py:330-389 on one wrapper with jump_ts=[3, 13], step_ts=[23]
    # (the inner wrapper of test/test_adaptive_stepsize_controller.py:255-281)
    pb = lambda x: np.nextafter(x, -np.inf)  # noqa: E731
    na = lambda x: np.nextafter(x, np.inf)  # noqa: E731
    t0, t1, mj, idx = O.clip_adapt([23.0], [3.0, 13.0], 1.0, 11.0)
    assert (t0, t1, mj) == (1.0, pb(3.0), False)
    # a step that ended just before the jump restarts after it (two ulps on)
    t0, t1, mj, idx = O.clip_adapt([23.0], [3.0, 13.0], t1, t1 + 10.0, idx)
    assert t0 == na(3.0) and mj and t1 == min(pb(3.0) + 10.0, pb(13.0))
    # and a step that ended exactly on the jump restarts one ulp on
    t0, t1, mj, idx = O.clip_adapt([23.0], [3.0, 13.0], 13.0, 14.0, idx)
    assert t0 == na(13.0) and mj and t1 == 14.0
    t0, t1, mj, idx = O.clip_adapt([23.0], [3.0, 13.0], 20.0, 30.0, idx)
    assert (t0, t1, mj) == (20.0, 23.0, False)
    # step_ts: a step that ended on a step time clips to the next one
    t0, t1, mj, idx = O.clip_adapt([2.0, 13.0], None, 2.0, 40.0)
    assert (t0, t1, mj) == (2.0, 13.0, False)
    # never an empty interval after a bump (clip.py:354-372)
    t0, t1, mj, idx = O.clip_adapt(None, [0.98], pb(0.98), pb(0.98))
    assert t0 == na(0.98) and t1 == na(t0) and mj


def _clip_desc(**kw):
    return O.make_desc(**dict(dict(solver=O.DOPRI5, controller=O.PID, rtol=1e-4, atol=1e-6,
                                   save_steps=1, save_t1=0), **kw))


@pytest.mark.parametrize("backwards", [False, True])
def test_clip_step_ts(backwards):
    # test/test_adaptive_stepsize_controller.py:18-41: y' = -0.2 y, Dopri5,
    # PID(1e-4, 1e-6), step_ts=[3, 4], SaveAt(steps=True): 3 and 4 are steps
    t0, t1 = (5.0, 0.0) if backwards else (0.0, 5.0)
    d = _clip_desc(field=O.LINEAR, dim=1)
    r = O.solve(d, t0, t1, None, [[1.0]], params=[[-0.2]], step_ts=[3, 4])
    assert r["result"][0] == 0
    assert 3.0 in r["ts"][0] and 4.0 in r["ts"][0]
    r0 = O.solve(_clip_desc(field=O.LINEAR, dim=1), t0, t1, None, [[1.0]], params=[[-0.2]])
    assert 3.0 not in r0["ts"][0]


def _forced(t, y):
    # test/test_adaptive_stepsize_controller.py:47-51: a damped oscillator
    # whose forcing flips sign at t = 7.5
    x, v = y
    force = 10.0 if t < 7.5 else -10.0
    return np.array([v, -4 * np.pi ** 2 * x - 4 * np.pi * 0.05 * v + force])


@pytest.mark.parametrize("backwards", [False, True])
def test_clip_jump_ts(backwards):
    # test/test_adaptive_stepsize_controller.py:44-88
    t0, t1 = (15.0, 0.0) if backwards else (0.0, 15.0)

    def run(**kw):
        d = _clip_desc(field=O.CALLBACK, dim=2)
        return O.solve(d, t0, t1, None, [[1.5, 0.0]], callback=_forced, **kw)

    no_jump, jump = run(), run(jump_ts=[7.5])
    assert no_jump["stats"][0, 0] > jump["stats"][0, 0]
    assert jump["result"][0] == 0
    assert run(jump_ts=[7.5], step_ts=[7.5])["result"][0] == 0
    r = run(jump_ts=[7.5], step_ts=[3.5, 8])
    assert r["result"][0] == 0
    assert 3.5 in r["ts"][0] and 8.0 in r["ts"][0]
    # the solve steps to just before the jump and restarts just after it
    ts = np.abs(r["ts"][0][np.isfinite(r["ts"][0])])
    if backwards:
        assert np.nextafter(7.5, np.inf) in ts and np.nextafter(7.5, -np.inf) not in ts
    else:
        assert np.nextafter(7.5, -np.inf) in ts and 7.5 not in ts


def test_clip_jump_at_t1():
    # test/test_adaptive_stepsize_controller.py:322-343 (here in FP64 time):
    # a jump at t1 still ends the solve exactly at t1
    d = O.make_desc(solver=O.HEUN, controller=O.PID, rtol=1e-6, atol=1e-6, field=O.LINEAR,
                    dim=1, n_ts=1, save_t1=0, max_steps=1 << 16)
    r = O.solve(d, 0.0, 1e3, 0.01, [[1.0]], params=[[-1.0]], ts=[1e3], jump_ts=[1e3])
    assert r["result"][0] == 0 and r["ts"][0, 0] == 1e3


def test_clip_t0_just_before_jump():
    # test/test_adaptive_stepsize_controller.py:346-371 (without its event): a
    # solve starting at prevbefore(jump) takes a zero-length first step, then
    # restarts past the jump and finishes
    d = O.make_desc(solver=O.HEUN, controller=O.PID, rtol=1e-6, atol=1e-6, field=O.LINEAR,
                    dim=4, save_t1=1, max_steps=100)
    r = O.solve(d, np.nextafter(0.98, -np.inf), 1.2, None, np.zeros((1, 4)),
                params=np.zeros((4, 4)), jump_ts=[0.98])
    assert r["result"][0] == 0 and r["ts"][0, 0] == 1.2


# ---------------------------------------------------------------------------
# Events (_event.py, _integrate.py:542-633, 686-877), restating
# test/test_event.py with the registered conditions: a linear form
# w.y + wt t + c (real-valued, or "> 0" as a boolean) and steady_state_event.
# ---------------------------------------------------------------------------

def _event_desc(conds, root=False, dim=1, **kw):
    """conds: list of (kind, coef[6], direction)."""
    base = dict(solver=O.TSIT5, controller=O.CONSTANT, dim=dim, save_t1=1,
                n_event=len(conds), event_root=int(root), ev_kind=[c[0] for c in conds],
                ev_coef=sum([list(c[1]) for c in conds], []), ev_dir=[c[2] for c in conds],
                newton_rtol=1e-5, newton_atol=1e-5)
    base.update(kw)
    return O.make_desc(**base)


def _lin(w=(0, 0, 0, 0), wt=0.0, c=0.0, kind=O.EV_LINEAR, direction=O.EV_EITHER):
    return (kind, list(w) + [0.0] * (4 - len(w)) + [wt, c], direction)


def _const_field(v):
    return lambda t, y: np.asarray(v, dtype=np.float64)


def test_event_steady_state():
    # test/test_event.py:106-121: tolerances from the PID controller
    d = _event_desc([(O.EV_STEADY, [1e-3, 1e-6, 0, 0, 0, 0], 0)], controller=O.PID,
                    rtol=1e-3, atol=1e-6, field=O.LINEAR)
    r = O.solve(d, 0.0, np.inf, 1.0, [[1.0]], params=[[-1.0]])
    assert r["event_index"][0] == 0 and r["result"][0] == 3
    assert abs(r["ys"][0, 0, 0]) < 1e-5


def test_event_no_step():
    # test/test_event.py:124-143: a boolean condition true at t0 ends the
    # solve before its first step
    d = _event_desc([_lin(w=(0, -1), kind=O.EV_LINEAR_BOOL)], dim=2, field=O.CALLBACK)
    r = O.solve(d, 0.0, 10.0, 1.0, [[1.0, -0.1]], callback=_const_field([1.0, 1.0]))
    assert r["stats"][0, 0] == 0 and r["event_index"][0] == 0
    assert np.array_equal(r["ys"][0, -1], [1.0, -0.1]) and r["ts"][0, -1] == 0.0


def test_event_continuous_terminate():
    # test/test_event.py:146-178: t > 10 as a boolean ends with y > 10; t - 10
    # as a real condition ends at t >= 10 (no root finder)
    d = _event_desc([_lin(wt=1.0, c=-10.0, kind=O.EV_LINEAR_BOOL)], field=O.LINEAR)
    r = O.solve(d, 0.0, np.inf, 1.0, [[1.0]], params=[[1.0]])
    assert r["ys"][0, 0, 0] > 10 and r["result"][0] == 3
    d = _event_desc([_lin(wt=1.0, c=-10.0)], field=O.LINEAR)
    r = O.solve(d, 0.0, np.inf, 1.0, [[1.0]], params=[[1.0]])
    assert r["ts"][0, 0] >= 10


def test_event_time_and_value():
    # test/test_event.py:181-216: with Newton(1e-5, 1e-5) the event time of
    # y = e^t crossing e is 1 (rtol 1e-4), and y' = 1 from -10 stops at y = 0
    d = _event_desc([_lin(w=(1,), c=-math.e)], root=True, field=O.LINEAR)
    r = O.solve(d, 0.0, np.inf, 1.0, [[1.0]], params=[[1.0]])
    assert tree_allclose(r["ts"][0, 0], 1.0, rtol=1e-4)
    d = _event_desc([_lin(w=(1,))], root=True, field=O.CALLBACK)
    r = O.solve(d, 0.0, np.inf, 1.0, [[-10.0]], callback=_const_field([1.0]))
    assert tree_allclose(r["ys"][0, 0, 0], 0.0, rtol=1e-5, atol=1e-8)
    assert tree_allclose(r["ts"][0, 0], 10.0, rtol=1e-5)


def test_event_none_and_two_conditions():
    # test/test_event.py:219-262
    d = _event_desc([_lin(w=(1,))], root=True, field=O.CALLBACK)
    r = O.solve(d, 0.0, 5.0, 1.0, [[-10.0]], callback=_const_field([1.0]))
    assert r["event_index"][0] == -1 and r["result"][0] == 0
    assert tree_allclose(r["ts"][0, 0], 5.0)
    d = _event_desc([_lin(wt=1.0, c=-10.0), _lin(w=(1,), c=5.0)], root=True, field=O.CALLBACK)
    r = O.solve(d, 0.0, np.inf, 1.0, [[-10.0]], callback=_const_field([1.0]))
    assert r["event_index"][0] == 1
    assert tree_allclose(r["ts"][0, 0], 5.0, rtol=1e-5)


def test_event_directions():
    # _integrate.py:585-597: up-crossings only, down-crossings only
    for direction, fires in ((O.EV_UP, True), (O.EV_DOWN, False), (O.EV_EITHER, True)):
        d = _event_desc([_lin(w=(1,), direction=direction)], root=True, field=O.CALLBACK)
        r = O.solve(d, 0.0, 20.0, 1.0, [[-10.0]], callback=_const_field([1.0]))
        assert (r["event_index"][0] == 0) == fires


@pytest.mark.parametrize("steps", (1, 2, 3, 4, 5))
def test_event_save_all_steps(steps):
    # test/test_event.py:566-612: y' = (1, 1), event x = thr, every step saved;
    # the save after the event time is replaced by the event's (t, y)
    thr = steps - 0.5
    for t0_save, t1_save, n in ((0, 0, steps), (0, 1, steps), (1, 1, steps + 1)):
        d = _event_desc([_lin(w=(1, 0), c=-thr)], root=True, dim=2, field=O.CALLBACK,
                        save_steps=1, save_t0=t0_save, save_t1=t1_save, max_steps=4096)
        r = O.solve(d, 0.0, 10.0, 1.0, [[0.0, -thr]], callback=_const_field([1.0, 1.0]))
        ts, ys = r["ts"][0], r["ys"][0]
        assert np.isfinite(ts).sum() == n and np.isfinite(ys[:, 0]).sum() == n
        assert tree_allclose(ts[n - 1], thr, atol=1e-5)
        assert tree_allclose(ys[n - 1], [thr, 0.0], atol=1e-5)


@pytest.mark.parametrize("steps", (1, 2, 3, 4, 5))
def test_event_save_ts(steps):
    # test/test_event.py:615-666: ts saves after the event time are deleted;
    # with t1 (or steps) the last save is the event's
    thr = steps - 0.5
    ts_save = [0.5, 3.5, 5.5]
    cases = [(dict(), False), (dict(save_t1=1), True), (dict(save_t0=1), False),
             (dict(save_steps=1), True)]
    for extra, save_final in cases:
        kw = dict(save_t1=0, save_t0=0, n_ts=3, max_steps=4096)
        kw.update(extra)
        d = _event_desc([_lin(w=(1, 0), c=-thr)], root=True, dim=2, field=O.CALLBACK, **kw)
        r = O.solve(d, 0.0, 10.0, 1.0, [[0.0, -thr]], ts=ts_save,
                    callback=_const_field([1.0, 1.0]))
        ts, ys = r["ts"][0], r["ys"][0]
        fin = np.isfinite(ts)
        if save_final:
            assert tree_allclose(ts[fin][-1], thr, atol=1e-5)
            assert tree_allclose(ys[fin][-1], [thr, 0.0], atol=1e-5)
        else:
            assert np.all(ts[fin] <= thr)


def test_event_constant_step_infinite_t1():
    # constant.py:48-55, 94-97: with t1 = inf the grid keeps adding dt0; the
    # condition t - 3 changes sign (to 0) on reaching t = 3
    d = _event_desc([_lin(wt=1.0, c=-3.0)], field=O.CALLBACK, save_steps=1, save_t1=0)
    r = O.solve(d, 0.0, np.inf, 0.5, [[0.0]], callback=_const_field([1.0]))
    ts = r["ts"][0]
    assert list(ts[np.isfinite(ts)]) == [0.5, 1.0, 1.5, 2.0, 2.5, 3.0]


# ---------------------------------------------------------------------------
# Resuming a solve (diffeqsolve's solver_state / controller_state / made_jump,
# _integrate.py:1252-1271, 1309, 1489-1500): split = whole.
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("solver", [O.DOPRI5, O.TSIT5, O.HEUN])
def test_resume_pid_split_reproduces_the_whole_solve(solver):
    # A PID solve stopped after k attempted steps (max_steps) and resumed from
    # its records, with dt0 = the whole solve's next step size, takes the
    # whole solve's remaining steps bit for bit: the controller's history and
    # the FSAL value carry over (FSAL solvers skip the first evaluation).  The
    # split is taken where attempts k and k + 1 are both accepted, so that the
    # next step size is the whole solve's next step.
    tol = 1e-4 if solver == O.HEUN else 1e-6  # a second-order method at a looser tolerance

    def desc(max_steps):
        return O.make_desc(solver=solver, controller=O.PID, field=O.VAN_DER_POL, dim=2,
                           rtol=tol, atol=tol * 1e-2, n_args=1, save_steps=1,
                           max_steps=max_steps)
    y0 = np.array([[1.2, -0.3]])
    mu = [1.5]
    whole = O.solve(desc(4096), 0.0, 3.0, 0.05, y0, args=mu, want_state=True)
    n = int(whole["stats"][0, 1])
    assert whole["result"][0] == 0
    acc = [int(O.solve(desc(k), 0.0, 3.0, 0.05, y0, args=mu)["stats"][0, 1])
           for k in range(1, 41)]
    k = next(k for k in range(10, 40) if acc[k - 1] == acc[k - 2] + 1 and acc[k] == acc[k - 1] + 1)
    leg1 = O.solve(desc(k), 0.0, 3.0, 0.05, y0, args=mu, want_state=True)
    st = leg1["state"]
    assert st[0, 4] == 1 and st[0, 5] == (0 if solver != O.HEUN else 1)  # FSAL value or none
    ka = int(leg1["stats"][0, 1])
    tk = whole["ts"][0, ka - 1]
    assert leg1["ts"][0, ka - 1] == tk
    leg2 = O.solve(desc(4096), tk, 3.0, whole["ts"][0, ka] - tk, leg1["ys"][:, ka - 1], args=mu,
                   state_in=st, want_state=True)
    m = n - ka
    assert leg2["stats"][0, 1] == m
    assert np.array_equal(leg2["ts"][0, :m], whole["ts"][0, ka:n])
    assert np.array_equal(leg2["ys"][0, :m], whole["ys"][0, ka:n])
    # the final records of the whole and of the resumed leg agree
    assert np.array_equal(leg2["state"], whole["state"])


def test_resume_constant_grid_and_fresh_state_defaults():
    # ConstantStepSize: steps_completed starts at 1 and the grid is
    # t0 + (t1 - t0) n / N (constant.py:30-104); a leg resumed with the grid
    # state ends on the whole solve's t1 value.  A record without a
    # controller state ([4] = 0) or with first_step set changes nothing.
    d = O.make_desc(solver=O.TSIT5, controller=O.CONSTANT, field=O.LOTKA_VOLTERRA, dim=2,
                    n_args=4, save_steps=1, max_steps=4096)
    args = [[0.1, 0.02, 0.4, 0.02]]
    y0 = np.array([[10.0, 5.0]])
    whole = O.solve(d, 0.0, 20.0, 0.1, y0, args=args, want_state=True)
    assert whole["state"][0, 0] == 201 and whole["state"][0, 1] == 200
    d1 = O.make_desc(solver=O.TSIT5, controller=O.CONSTANT, field=O.LOTKA_VOLTERRA, dim=2,
                     n_args=4, save_steps=1, max_steps=70)
    leg1 = O.solve(d1, 0.0, 20.0, 0.1, y0, args=args, want_state=True)
    assert leg1["state"][0, 0] == 71
    leg2 = O.solve(d, leg1["ts"][0, 69], 20.0, 0.1, leg1["ys"][:, 69], args=args,
                   state_in=leg1["state"], want_state=True)
    assert leg2["stats"][0, 0] == 130 and leg2["state"][0, 0] == 201
    assert tree_allclose(leg2["ys"][0, 129], whole["ys"][0, 199], rtol=1e-12, atol=1e-12)
    blank = np.zeros_like(leg1["state"])
    blank[:, 5] = 1.0  # no controller state, first_step
    fresh = O.solve(d, 0.0, 20.0, 0.1, y0, args=args, state_in=blank)
    assert np.array_equal(fresh["ys"], whole["ys"])
