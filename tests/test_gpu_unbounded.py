"""max_steps=None (diffrax/_integrate.py:1283-1292, 1316-1319): an unbounded
solve gives the same results as a bounded one that its trajectories do not
reach, on the trajectory kernels, the MLP integrator and under
BacksolveAdjoint."""
import numpy as np
import pytest
import torch

import diffrax_gb300 as dfx

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", ["fused", "plain"])
def test_unbounded_matches_bounded_van_der_pol(kernel):
    dev = torch.device("cuda")
    rng = np.random.default_rng(41)
    y0 = torch.tensor(rng.uniform(-2, 2, (2048, 2)), dtype=torch.float32, device=dev)
    mu = torch.tensor(rng.uniform(0.5, 3.0, (2048, 1)), dtype=torch.float32, device=dev)
    t1 = torch.tensor(rng.uniform(5.0, 20.0, 2048), dtype=torch.float64, device=dev)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9)
    sols = [dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Dopri5(), 0.0, t1, None, y0, mu,
                            saveat=dfx.SaveAt(ts=[1.0, 2.0], t1=True), stepsize_controller=pid,
                            max_steps=m, kernel=kernel) for m in (None, 100000)]
    assert torch.equal(sols[0].ys, sols[1].ys)
    assert torch.equal(sols[0].stats["num_steps"], sols[1].stats["num_steps"])
    assert sols[0].stats["max_steps"] is None


def test_unbounded_mlp_and_backsolve():
    dev = torch.device("cuda")
    rng = np.random.default_rng(42)
    W = [torch.tensor(rng.standard_normal((o, i)) / np.sqrt(i), dtype=torch.float32,
                      device=dev, requires_grad=True) for i, o in ((64, 128), (128, 128), (128, 64))]
    b = [torch.zeros(o, device=dev, requires_grad=True) for o in (128, 128, 64)]
    y0 = torch.tensor(rng.standard_normal((256, 64)), dtype=torch.float32, device=dev)
    pid = dfx.PIDController(rtol=1e-5, atol=1e-7)
    out = []
    for m in (None, 5000):
        sol = dfx.diffeqsolve(dfx.ODETerm(dfx.MLPField(W, b)), dfx.Tsit5(), 0.0, 1.0, None, y0,
                              saveat=dfx.SaveAt(ts=[0.5, 1.0]), stepsize_controller=pid,
                              adjoint=dfx.BacksolveAdjoint(), max_steps=m)
        g = torch.autograd.grad(sol.ys.square().mean(), W[1])[0]
        out.append((sol.ys.detach(), g))
    assert torch.equal(out[0][0], out[1][0])
    assert torch.allclose(out[0][1], out[1][1], rtol=1e-5, atol=1e-8)
    with pytest.raises(NotImplementedError, match="finite max_steps"):
        dfx.diffeqsolve(dfx.ODETerm(dfx.MLPField(W, b)), dfx.Tsit5(), 0.0, 1.0, None, y0,
                        stepsize_controller=pid, max_steps=None)


def test_saveat_fn_maps_the_saves():
    # SaveAt(fn=...) (_saveat.py:20-43): here fn(t, y, args) = t * y[..., :1]
    dev = torch.device("cuda")
    rng = np.random.default_rng(43)
    y0 = torch.tensor(rng.uniform(-2, 2, (512, 2)), dtype=torch.float32, device=dev)
    mu = torch.ones((1,), dtype=torch.float32, device=dev)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9)
    ts = [0.5, 1.0, 2.0]
    plain = dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Tsit5(), 0.0, 2.0, None, y0, mu,
                            saveat=dfx.SaveAt(ts=ts), stepsize_controller=pid)
    fn = lambda t, y, args: t[..., None].to(y.dtype) * y[..., :1] * args[0]  # noqa: E731
    mapped = dfx.diffeqsolve(dfx.ODETerm(dfx.VanDerPol()), dfx.Tsit5(), 0.0, 2.0, None, y0, mu,
                             saveat=dfx.SaveAt(ts=ts, fn=fn), stepsize_controller=pid)
    assert mapped.ys.shape == (512, 3, 1)
    assert torch.equal(mapped.ys, fn(plain.ts, plain.ys, mu))


def test_saveat_subs_tree_of_solves():
    # SaveAt(subs={...}): each SubSaveAt's saves, as separate SaveAt solves give them
    dev = torch.device("cuda")
    rng = np.random.default_rng(44)
    y0 = torch.tensor(rng.uniform(-2, 2, (256, 2)), dtype=torch.float32, device=dev)
    mu = torch.ones((1,), dtype=torch.float32, device=dev)
    pid = dfx.PIDController(rtol=1e-6, atol=1e-9)
    term = dfx.ODETerm(dfx.VanDerPol())
    subs = {"t1": dfx.SubSaveAt(t1=True), "grid": [dfx.SubSaveAt(ts=[0.5, 1.5], t0=True),
                                                   dfx.SubSaveAt(steps=2)]}
    sol = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, 2.0, None, y0, mu,
                          saveat=dfx.SaveAt(subs=subs), stepsize_controller=pid)
    for got, sa in ((sol.ys["t1"], dfx.SaveAt(t1=True)),
                    (sol.ys["grid"][0], dfx.SaveAt(ts=[0.5, 1.5], t0=True)),
                    (sol.ys["grid"][1], dfx.SaveAt(steps=2))):
        want = dfx.diffeqsolve(term, dfx.Dopri5(), 0.0, 2.0, None, y0, mu, saveat=sa,
                               stepsize_controller=pid)
        assert torch.equal(got, want.ys)
