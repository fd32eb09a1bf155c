"""The multi-rank path on CPU (gloo, world size 2): a batch of trajectories
sharded across ranks, each rank's gradient of the global loss, and the one
collective -- the sum of dL/dtheta -- against the single-process gradient.

The per-rank gradients come from the FP64 oracle (the GPU kernels cannot run
on a CPU machine); what is under test is the sharding and the reduction."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle as O
from diffrax_gb300 import distributed as gdist

WIDTHS = [4, 8, 8, 4]
B = 13  # uneven shards: 7 + 6


def _problem():
    rng = np.random.default_rng(0)
    Ws = [rng.standard_normal((WIDTHS[i + 1], WIDTHS[i])) / np.sqrt(WIDTHS[i])
          for i in range(3)]
    bs = [rng.standard_normal(WIDTHS[i + 1]) * 0.1 for i in range(3)]
    params = np.concatenate([np.concatenate([W.reshape(-1), b]) for W, b in zip(Ws, bs)])
    y0 = rng.standard_normal((B, WIDTHS[0]))
    d = O.make_desc(solver=O.TSIT5, controller=O.PID, field=O.MLP, dim=WIDTHS[0], rtol=1e-6,
                    atol=1e-8, save_t1=1, mlp_depth=3, mlp_widths=WIDTHS)
    return d, params, y0


def _grads(y0):
    """The oracle's dL/dy0 and dL/dtheta of L = sum over the global batch of
    mean(y(1)^2) restricted to the rows y0."""
    d, params, _ = _problem()
    fwd = O.solve(d, 0.0, 1.0, None, y0, params=params)
    G = 2.0 * fwd["ys"] / (B * WIDTHS[0])
    r = O.grad_recursive(d, 0.0, 1.0, None, y0, G, params=params)
    return r["grad_y0"], r["grad_params"]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _, _, y0 = _problem()
        a, b = gdist.shard_bounds(B, rank, world)
        gy0, gp = _grads(y0[a:b])
        gp_t = torch.tensor(gp)
        gdist.all_reduce_gradients([gp_t])
        out[rank] = (a, b, gy0, gp_t.numpy())
    finally:
        dist.destroy_process_group()


def test_shard_bounds_cover_the_batch():
    for batch in (0, 1, 7, 13, 65536):
        for world in (1, 2, 3, 8):
            spans = [gdist.shard_bounds(batch, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == batch
            assert all(spans[r][1] == spans[r + 1][0] for r in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        gdist.shard_bounds(4, 2, 2)


def test_two_rank_gradient_sum_equals_the_single_process_gradient():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    _, _, y0 = _problem()
    gy0_ref, gp_ref = _grads(y0)
    # dL/dtheta: the reduced sum on both ranks equals the whole-batch gradient
    for r in range(2):
        np.testing.assert_allclose(out[r][3], gp_ref, rtol=1e-12, atol=1e-15)
    # dL/dy0: each rank's shard, stitched back, is the whole-batch gradient
    stitched = np.concatenate([out[r][2] for r in range(2)])
    np.testing.assert_allclose(stitched, gy0_ref, rtol=1e-12, atol=1e-15)
    assert [out[r][:2] for r in range(2)] == [(0, 7), (7, 13)]


def test_all_reduce_is_a_no_op_without_a_process_group():
    g = torch.arange(4.0)
    gdist.all_reduce_gradients([g, None])
    assert torch.equal(g, torch.arange(4.0))
