"""Inverse rendering across ranks: view sharding, the one gradient all-reduce
per iteration and identical Adam steps on every rank, run as two gloo ranks
on the CPU with stand-in views (a linear image model with its exact
gradient in place of the renderer), plus bench.py's multi-rank plumbing
(barrier, max over ranks)."""
import os
import socket
import tempfile

import numpy as np
import pytest

from lucent_gb300.inverse import Adam, InverseRendering, views_of_rank

MATERIALS, ENV_H, ENV_W, PIXELS, VIEWS, STEPS = 4, 8, 16, 96, 7, 5


class LinearView:
    """image = A @ [theta | env] + b, an exact-gradient stand-in for a rendered view."""

    def __init__(self, v, n_params):
        rng = np.random.default_rng(1000 + v)
        self.A = rng.uniform(-1, 1, (PIXELS * 3, n_params)).astype(np.float32) / 8
        self.b = rng.uniform(0, 1, PIXELS * 3).astype(np.float32)
        self.target = rng.uniform(0, 1, PIXELS * 3).astype(np.float32)

    def loss_and_grad(self, theta, env):
        x = np.concatenate([theta.reshape(-1), env.reshape(-1)]).astype(np.float32)
        diff = self.A @ x + self.b - self.target
        g = (2.0 * diff) @ self.A
        n = theta.size
        return float(np.square(diff, dtype=np.float64).sum()), g[:n].reshape(theta.shape), g[n:].reshape(env.shape)


def start_params():
    rng = np.random.default_rng(7)
    return rng.uniform(0, 1, (MATERIALS, 6)), rng.uniform(0, 2, (ENV_H, ENV_W, 3))


def run(rank, world, reduce=None):
    theta, env = start_params()
    n_params = theta.size + env.size
    views = [LinearView(v, n_params) for v in views_of_rank(VIEWS, rank, world)]
    opt = InverseRendering(views, theta, env, reduce=reduce)
    for _ in range(STEPS):
        opt.step()
    return opt


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    from lucent_gb300.inverse import TorchAllReduce
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        red = TorchAllReduce()
        opt = run(rank, world, red)
        np.savez(os.path.join(out, "rank%d.npz" % rank), theta=opt.theta, env=opt.env,
                 history=np.array(opt.history), calls=red.calls, size=opt.size)
        import bench
        bench._pg = dist
        bench.barrier(world)
        np.save(os.path.join(out, "max%d.npy" % rank), bench.max_over_ranks(10.0 + rank, world))
    finally:
        dist.destroy_process_group()


@pytest.fixture(scope="module")
def two_ranks():
    import torch.multiprocessing as mp
    with tempfile.TemporaryDirectory() as out:
        mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
        res = [dict(np.load(os.path.join(out, "rank%d.npz" % r))) for r in range(2)]
        res_max = [float(np.load(os.path.join(out, "max%d.npy" % r))) for r in range(2)]
    return res, res_max


def test_views_of_rank_cover_every_view_once():
    for world in (1, 2, 3, 8, 9):
        got = sorted(v for r in range(world) for v in views_of_rank(VIEWS, r, world))
        assert got == list(range(VIEWS))
    with pytest.raises(ValueError):
        views_of_rank(VIEWS, 2, 2)


def test_adam_matches_closed_form_first_step():
    # The first bias-corrected Adam step moves each coordinate by lr * sign(g).
    opt = Adam(3, 0.1)
    x = opt.step(np.zeros(3), np.array([2.0, -0.5, 1e-3]))
    np.testing.assert_allclose(x, [-0.1, 0.1, -0.1], rtol=1e-4)


def test_loss_decreases_on_one_rank():
    opt = run(0, 1)
    assert all(b < a for a, b in zip(opt.history, opt.history[1:]))
    assert opt.history[-1] < 0.8 * opt.history[0]
    assert 0 <= opt.theta.min() and opt.theta.max() <= 1 and opt.env.min() >= 0


def test_two_ranks_agree_with_each_other_and_with_one(two_ranks):
    res, _ = two_ranks
    one = run(0, 1)
    for r in res:
        assert int(r["calls"]) == STEPS  # one all-reduce per iteration
        assert int(r["size"]) == MATERIALS * 6 + ENV_H * ENV_W * 3 + 1
        np.testing.assert_array_equal(r["theta"], res[0]["theta"])
        np.testing.assert_array_equal(r["env"], res[0]["env"])
        np.testing.assert_array_equal(r["history"], res[0]["history"])
    # binary64 sums of these binary32 gradients are exact, so the split does not show in the
    # parameters; the losses are binary64 values themselves and may differ in the last bits
    np.testing.assert_array_equal(res[0]["theta"], one.theta)
    np.testing.assert_array_equal(res[0]["env"], one.env)
    np.testing.assert_allclose(res[0]["history"], one.history, rtol=1e-14)


def test_bench_max_over_ranks(two_ranks):
    _, mx = two_ranks
    assert mx == [11.0, 11.0]
