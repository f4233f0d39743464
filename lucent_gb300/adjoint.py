"""Differentiable rendering over the C ABI (path replay backpropagation).

The parameters are, per material, base colour (r, g, b), roughness,
metallic and clearcoat, plus the environment map's texels. `forward` renders
`spp` samples from a seed with given parameters; `backward` returns the
gradient of sum_px dl[px] . image[px] (lucent_renderer_backward). Sampling is
held fixed in the derivative (directions, pdfs, MIS, lobe and roulette
choices), as in path replay backpropagation.

`RenderFunction` wraps the pair as a torch.autograd.Function, so a host can
optimise with any torch optimiser; the rendering itself never leaves the
CUDA kernels.
"""
import ctypes as C

import numpy as np

from . import _native as N
from .renderer import Renderer

# Offsets of the optimised parameters inside a packed material (40 floats,
# packMaterials, material.ts:132-149): albedo.rgb, roughness, metallic, clearcoat.
PARAMS = ("r", "g", "b", "roughness", "metallic", "clearcoat")
PARAM_OFFSETS = np.array([0, 1, 2, 4, 3, 21])
PARAM_RANGES = np.array([[0.0, 1.0]] * 3 + [[0.0, 1.0], [0.0, 1.0], [0.0, 1.0]])


def _f(a):
    return N.ptr(a, C.c_float) if a is not None else None


def get_params(packed):
    """[material_count, 6] parameters of a packed material array."""
    m = np.asarray(packed, np.float32).reshape(-1, 40)
    return m[:, PARAM_OFFSETS].copy()


def set_params(packed, theta):
    """Packed materials with the 6 parameters of every material replaced."""
    m = np.array(packed, np.float32).reshape(-1, 40)
    m[:, PARAM_OFFSETS] = np.clip(np.asarray(theta, np.float32), PARAM_RANGES[:, 0], PARAM_RANGES[:, 1])
    return m.reshape(-1)


def set_materials(r: Renderer, packed):
    p = np.ascontiguousarray(packed, np.float32).reshape(-1)
    N.check(N.lib().lucent_renderer_set_materials(r.handle, _f(p), p.size // 40))
    r.packed.materials = p


def set_env(r: Renderer, rgb):
    """Replaces the environment map's texels (same size); its sampler is
    rebuilt on the GPU (lucent_renderer_set_env), not on the host."""
    env = r.scene.env.map
    env.data = np.ascontiguousarray(rgb, np.float32).reshape(-1)
    N.check(N.lib().lucent_renderer_set_env(r.handle, _f(env.data), env.width, env.height, None))


def forward(r: Renderer, spp, seed, theta=None, env=None):
    """Renders `spp` samples from sample seed `seed`; returns the [H, W, 3] mean radiance."""
    if theta is not None:
        set_materials(r, set_params(r.packed.materials, theta))
    if env is not None:
        set_env(r, env)
    r.reset()
    r.set_seed(seed)
    r.trace_samples(spp)
    return r.read()[0][..., :3].copy()


def backward(r: Renderer, spp, seed, dl, env_grad=True):
    """Gradient of sum_px dl[px] . forward(...)[px]: ([material_count, 6], [env_h, env_w, 3] or None)."""
    h, w = r.height, r.width
    d = np.zeros((h, w, 4), np.float32)
    d[..., :3] = np.asarray(dl, np.float32).reshape(h, w, 3)
    n = r.packed.material_count
    dm = np.zeros(n * 6, np.float32)
    env = r.scene.env.map
    de = np.zeros(env.width * env.height * 3, np.float32) if env_grad else None
    N.check(N.lib().lucent_renderer_backward(r.handle, spp, seed, _f(d), _f(dm), _f(de), None))
    return dm.reshape(n, 6), (de.reshape(env.height, env.width, 3) if de is not None else None)


def _torch_function():
    import torch

    class RenderFunction(torch.autograd.Function):
        """image = RenderFunction.apply(theta, env, renderer, spp, seed): theta [materials, 6],
        env [H, W, 3] (float32 tensors), image [height, width, 3]."""

        @staticmethod
        def forward(ctx, theta, env, renderer, spp, seed):
            img = forward(renderer, spp, seed, theta.detach().cpu().numpy(), env.detach().cpu().numpy())
            ctx.renderer, ctx.spp, ctx.seed = renderer, spp, seed
            return torch.from_numpy(img).to(theta.device)

        @staticmethod
        def backward(ctx, grad):
            dm, de = backward(ctx.renderer, ctx.spp, ctx.seed, grad.detach().cpu().numpy())
            return torch.from_numpy(dm).to(grad.device), torch.from_numpy(de).to(grad.device), None, None, None

    return RenderFunction


def __getattr__(name):
    if name == "RenderFunction":
        return _torch_function()
    raise AttributeError(name)
