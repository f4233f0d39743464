"""Inverse rendering over many views and GPUs: one gradient all-reduce per iteration.

The optimised parameters are the adjoint's (base colour, roughness, metallic
and clearcoat of every material, and the environment map's texels); the loss
is the L2 image loss summed over the views. Views are independent units:
view v belongs to rank v % world. Each rank renders its own views forward,
runs the path-replay backward of each against the L2 loss, and adds its
views' gradients into one flat binary64 vector

    [material_count * 6 material gradients | env texels * 3 | loss]

(32 * 6 + 256 * 128 * 3 + 1 = 98,497 values for 32 materials and a
256x128 map). One all-reduce (sum) of that vector per iteration gives every
rank the whole gradient; every rank then applies the same Adam step to the
same parameters, so the parameters stay identical on all ranks without a
broadcast.

The partial sums are binary64 sums of binary32 gradients, so the reduced
gradient does not depend on how the views are split across ranks whenever
the terms' exponents span fewer than 29 bits (binary64 then adds them
exactly); otherwise it differs in the last binary64 bits, far below the
binary32 gradients' own precision.

The rendering stays in the CUDA kernels (`adjoint.forward` / `adjoint.backward`
over the C ABI); this module is host logic: sharding, the reduction and the
optimiser. A view is anything with `loss_and_grad(theta, env)`, which lets
the sharding and the reduction be tested on the CPU with stand-in views.
"""
import time

import numpy as np

from . import adjoint as AD


def views_of_rank(n_views, rank, world):
    """The views rank `rank` of `world` renders: v % world == rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    return list(range(rank, n_views, world))


class RendererView:
    """One camera view of an inverse problem: a renderer holding the scene
    from that camera, the target image and the sample count and seed of the
    forward render and its replay."""

    def __init__(self, renderer, target, spp, seed):
        self.renderer, self.target, self.spp, self.seed = renderer, np.asarray(target, np.float32), spp, seed
        self.timing = {"upload": 0.0, "forward": 0.0, "backward": 0.0}

    def loss_and_grad(self, theta, env):
        """(L2 loss, [materials, 6] gradient, [env_h, env_w, 3] gradient or None)."""
        r = self.renderer
        t0 = time.perf_counter()
        AD.set_materials(r, AD.set_params(r.packed.materials, theta))
        if env is not None:
            AD.set_env(r, env)
        t1 = time.perf_counter()
        img = AD.forward(r, self.spp, self.seed)
        t2 = time.perf_counter()
        diff = img - self.target
        dm, de = AD.backward(r, self.spp, self.seed, 2.0 * diff, env_grad=env is not None)
        t3 = time.perf_counter()
        self.timing["upload"] += t1 - t0
        self.timing["forward"] += t2 - t1
        self.timing["backward"] += t3 - t2
        return float(np.square(diff, dtype=np.float64).sum()), dm, de


class Adam:
    """Adam (Kingma and Ba, 2015) with bias correction, in binary64, on one flat vector."""

    def __init__(self, size, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.lr = np.broadcast_to(np.asarray(lr, np.float64), (size,)).copy()
        self.b1, self.b2, self.eps = beta1, beta2, eps
        self.m = np.zeros(size)
        self.v = np.zeros(size)
        self.t = 0

    def step(self, x, g):
        self.t += 1
        self.m = self.b1 * self.m + (1 - self.b1) * g
        self.v = self.b2 * self.v + (1 - self.b2) * g * g
        mh = self.m / (1 - self.b1 ** self.t)
        vh = self.v / (1 - self.b2 ** self.t)
        return x - self.lr * mh / (np.sqrt(vh) + self.eps)


class TorchAllReduce:
    """Sum over the ranks of a torch.distributed process group (gloo on host
    memory, NCCL through a device copy). Counts its calls."""

    def __init__(self, group=None, device=None):
        import torch.distributed as dist
        self.dist, self.group, self.device = dist, group, device
        self.calls = 0

    def __call__(self, vec):
        import torch
        t = torch.from_numpy(np.ascontiguousarray(vec, np.float64))
        if self.device is not None:
            t = t.to(self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        self.calls += 1
        return t.cpu().numpy()


class InverseRendering:
    """Gradient descent on materials and environment over `views` (this rank's
    share, `views_of_rank`), with `reduce` summing the flat gradient vector
    over the ranks (None: one rank). `theta` is [materials, 6] in [0, 1];
    `env` is [env_h, env_w, 3] (texels kept >= 0) or None to leave the
    environment fixed. The step sizes are multiplied by `decay` after every
    iteration."""

    def __init__(self, views, theta, env=None, reduce=None, lr_materials=0.02, lr_env=0.05, decay=1.0):
        self.views = list(views)
        self.theta = np.asarray(theta, np.float64).copy()
        self.env = None if env is None else np.asarray(env, np.float64).copy()
        self.reduce = reduce
        self.n_theta = self.theta.size
        self.n_env = 0 if self.env is None else self.env.size
        lr = np.concatenate([np.full(self.n_theta, lr_materials), np.full(self.n_env, lr_env)])
        self.opt = Adam(self.n_theta + self.n_env, lr)
        self.decay = decay
        self.history = []
        self.timing = {"reduce": 0.0, "update": 0.0}

    @property
    def size(self):
        """Length of the reduced vector: gradients plus the loss."""
        return self.n_theta + self.n_env + 1

    def partial(self):
        """This rank's sum over its views of [material grads | env grads | loss] (binary64)."""
        acc = np.zeros(self.size)
        theta = self.theta.astype(np.float32)
        env = None if self.env is None else self.env.astype(np.float32)
        for v in self.views:
            loss, dm, de = v.loss_and_grad(theta, env)
            acc[:self.n_theta] += np.asarray(dm, np.float64).reshape(-1)
            if self.n_env:
                acc[self.n_theta:-1] += np.asarray(de, np.float64).reshape(-1)
            acc[-1] += loss
        return acc

    def apply(self, total):
        """One Adam step from the reduced vector; returns the summed loss."""
        t0 = time.perf_counter()
        x = np.concatenate([self.theta.reshape(-1), self.env.reshape(-1) if self.n_env else np.zeros(0)])
        x = self.opt.step(x, total[:-1])
        self.opt.lr *= self.decay
        self.theta = np.clip(x[:self.n_theta], 0.0, 1.0).reshape(self.theta.shape)
        if self.n_env:
            self.env = np.maximum(x[self.n_theta:], 0.0).reshape(self.env.shape)
        self.timing["update"] += time.perf_counter() - t0
        self.history.append(float(total[-1]))
        return float(total[-1])

    def step(self):
        """One iteration: forward + backward of this rank's views, one
        all-reduce, one Adam step. Returns the loss over all views (before
        the step)."""
        acc = self.partial()
        t0 = time.perf_counter()
        total = acc if self.reduce is None else self.reduce(acc)
        self.timing["reduce"] += time.perf_counter() - t0
        return self.apply(total)
