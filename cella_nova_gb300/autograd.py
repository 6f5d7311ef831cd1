"""torch.autograd over the hand-written adjoint kernels.

``unroll(world, seed, mu, sigma, weights, h, T, every)`` runs T DiffusionLenia
steps on the GPU (cg_unroll, checkpoints every ``every`` steps) and its
backward runs the adjoint kernels (cg_unroll_backward, each segment recomputed
from its checkpoint), returning gradients for the seed, mu, sigma, the growth
weights and the spatial kernels h (K, n, n).  Gradients for any kernel
parametrisation follow from h by ordinary torch autograd, e.g. through
:class:`RingKernelBuilder`.

``unroll_rings(world, specs, seed, mu, sigma, weights, rings, T, every)`` does
the same for Lenia ring kernels given by their ring weights: the kernels are
built on the GPU (cg_build_ring_kernels) and the ring-weight gradients come
from cg_ring_weight_grad, so no step of the loop runs torch compute.

This is the differentiable form of train/diff_lenia_org.py's
``DiffusionLenia.step`` (the reference differentiates it with torch
autograd); :class:`DiffusionLeniaGPU` mirrors that model's parameters.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _abi
from ._abi import check, fptr, uptr


def _p(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


class LeniaWorld:
    """A GPU world bound to torch's current CUDA stream (all work of the
    world and of torch then stays ordered)."""

    def __init__(self, n: int, C: int, c0, c1, temp: float = 1.0, device=None):
        self.lib = _abi.load()
        self.device = torch.device(device or "cuda")
        self.n, self.C = int(n), int(C)
        self.c0 = np.ascontiguousarray(c0, dtype=np.uint32)
        self.c1 = np.ascontiguousarray(c1, dtype=np.uint32)
        self.K = len(self.c0)
        self.temp = float(temp)
        with torch.cuda.device(self.device):
            # bind to torch's current stream; its default stream is the legacy
            # stream, handle 0, which the C ABI would read as "own stream",
            # so pass cudaStreamLegacy (1) instead
            stream = torch.cuda.current_stream(self.device).cuda_stream or 1
            one = np.ones(self.K, np.float32)
            h = ctypes.c_void_p()
            check(self.lib.cg_create(self.n, self.C, self.K, uptr(self.c0), uptr(self.c1),
                                     fptr(one * 0.1), fptr(one * 0.05), fptr(one),
                                     ctypes.c_float(self.temp), ctypes.c_void_p(stream),
                                     ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            check(self.lib.cg_destroy(self.h))
            self.h = None

    def autotune(self, reps: int = 5):
        """Pick the fastest variant of every phase (cg_autotune); the adjoint
        kernels follow the forward phases' CTA shapes.  Returns the variants."""
        ms = np.zeros(4 * _abi.MAX_VARIANTS, dtype=np.float64)
        chosen = (ctypes.c_int * 4)()
        check(self.lib.cg_autotune(self.h, int(reps), ms.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   chosen))
        return list(chosen)

    def set_variants(self, v):
        arr = (ctypes.c_int * 4)(*[int(x) for x in v])
        check(self.lib.cg_set_variants(self.h, arr))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_rings(self, specs, rings: torch.Tensor, params: torch.Tensor):
        """Device-side parameters: params = [mu | sigma | weights] (3K f32) and
        ring weights rings (K, 8) f32, both on the world's stream; the kernel
        spectra are built on the GPU."""
        p = params.data_ptr()
        K = self.K
        check(self.lib.cg_set_params_device(self.h, ctypes.c_void_p(p), ctypes.c_void_p(p + 4 * K),
                                            ctypes.c_void_p(p + 8 * K)))
        check(self.lib.cg_build_ring_kernels(self.h, ctypes.cast(specs, ctypes.c_void_p),
                                             _p(rings)))

    def load(self, mu, sigma, weights, h: torch.Tensor):
        """Growth parameters (host arrays) and the spatial kernels h (K, n, n)
        f32 on the device, whose spectra the library takes with its own
        FFTs (cg_set_kernels_spatial_device)."""
        mu = np.ascontiguousarray(mu, np.float32)
        sg = np.ascontiguousarray(sigma, np.float32)
        w = np.ascontiguousarray(weights, np.float32)
        check(self.lib.cg_set_params(self.h, fptr(mu), fptr(sg), fptr(w),
                                     ctypes.c_float(self.temp)))
        check(self.lib.cg_set_kernels_spatial_device(self.h, _p(h)))


class _Unroll(torch.autograd.Function):
    @staticmethod
    def forward(ctx, world, T, every, seed, mu, sigma, weights, h):
        lib = world.lib
        hk = h.detach().float().contiguous()
        host = [t.detach().float().cpu().numpy() for t in (mu, sigma, weights)]
        world.load(*host, hk)
        x0 = seed.detach().float().contiguous()
        nck = (T - 1) // every + 1
        ckpt = torch.empty((nck,) + tuple(x0.shape), dtype=torch.float32, device=x0.device)
        xT = torch.empty_like(x0)
        check(lib.cg_unroll(world.h, _p(x0), int(T), int(every), _p(ckpt), _p(xT)))
        ctx.world, ctx.T, ctx.every = world, int(T), int(every)
        ctx.dtypes = (seed.dtype, mu.dtype, sigma.dtype, weights.dtype, h.dtype)
        ctx.host, ctx.h = host, hk
        ctx.save_for_backward(ckpt)
        return xT

    @staticmethod
    def backward(ctx, gT):
        world = ctx.world
        lib = world.lib
        (ckpt,) = ctx.saved_tensors
        world.load(*ctx.host, ctx.h)   # another unroll may have run since
        gT = gT.contiguous().float()
        g0 = torch.empty_like(gT)
        gtmp = torch.empty_like(gT)
        seg = torch.empty((ctx.every,) + tuple(gT.shape), dtype=torch.float32, device=gT.device)
        K, n = world.K, world.n
        pgrad = torch.zeros(3 * K, dtype=torch.float64, device=gT.device)
        kgrad = torch.zeros((K, n // 2, n, 2), dtype=torch.float32, device=gT.device)
        check(lib.cg_unroll_backward(world.h, _p(ckpt), ctx.T, ctx.every, _p(gT), _p(g0),
                                     _p(pgrad), _p(kgrad), _p(seg), _p(gtmp)))
        hbar = torch.empty((K, n, n), dtype=torch.float32, device=gT.device)
        check(lib.cg_kernel_grad_spatial(world.h, _p(kgrad), _p(hbar)))
        ds, dm, dsg, dw, dh = ctx.dtypes
        return (None, None, None, g0.to(ds), pgrad[:K].to(dm), pgrad[K:2 * K].to(dsg),
                pgrad[2 * K:].to(dw), hbar.to(dh))


def unroll(world: LeniaWorld, seed, mu, sigma, weights, h, T: int, every: int = 8):
    """x_T after T steps, differentiable in every tensor argument."""
    return _Unroll.apply(world, T, every, seed, mu, sigma, weights, h)


class _UnrollRings(torch.autograd.Function):
    @staticmethod
    def forward(ctx, world, T, every, specs, seed, mu, sigma, weights, rings):
        lib = world.lib
        params = torch.cat([mu.detach(), sigma.detach(), weights.detach()]).float().contiguous()
        rw = rings.detach().float().contiguous()
        world.load_rings(specs, rw, params)
        x0 = seed.detach().float().contiguous()
        nck = (T - 1) // every + 1
        ckpt = torch.empty((nck,) + tuple(x0.shape), dtype=torch.float32, device=x0.device)
        xT = torch.empty_like(x0)
        check(lib.cg_unroll(world.h, _p(x0), int(T), int(every), _p(ckpt), _p(xT)))
        ctx.world, ctx.T, ctx.every, ctx.specs = world, int(T), int(every), specs
        ctx.dtypes = (seed.dtype, mu.dtype, sigma.dtype, weights.dtype, rings.dtype)
        ctx.save_for_backward(ckpt, params, rw)
        return xT

    @staticmethod
    def backward(ctx, gT):
        world = ctx.world
        lib = world.lib
        ckpt, params, rw = ctx.saved_tensors
        world.load_rings(ctx.specs, rw, params)   # another unroll may have run since
        gT = gT.contiguous().float()
        g0 = torch.empty_like(gT)
        gtmp = torch.empty_like(gT)
        seg = torch.empty((ctx.every,) + tuple(gT.shape), dtype=torch.float32, device=gT.device)
        K, n = world.K, world.n
        pgrad = torch.zeros(3 * K, dtype=torch.float64, device=gT.device)
        kgrad = torch.zeros((K, n // 2, n, 2), dtype=torch.float32, device=gT.device)
        check(lib.cg_unroll_backward(world.h, _p(ckpt), ctx.T, ctx.every, _p(gT), _p(g0),
                                     _p(pgrad), _p(kgrad), _p(seg), _p(gtmp)))
        hbar = torch.empty((K, n, n), dtype=torch.float32, device=gT.device)
        check(lib.cg_kernel_grad_spatial(world.h, _p(kgrad), _p(hbar)))
        grings = torch.zeros_like(rw)
        check(lib.cg_ring_weight_grad(world.h, ctypes.cast(ctx.specs, ctypes.c_void_p), _p(rw),
                                      _p(hbar), _p(grings)))
        ds, dm, dsg, dw, dr = ctx.dtypes
        return (None, None, None, None, g0.to(ds), pgrad[:K].to(dm), pgrad[K:2 * K].to(dsg),
                pgrad[2 * K:].to(dw), grings.to(dr))


def unroll_rings(world: LeniaWorld, specs, seed, mu, sigma, weights, rings, T: int,
                 every: int = 8):
    """x_T after T steps with Lenia ring kernels built on the GPU from their
    ring weights rings (K, 8); differentiable in seed, mu, sigma, weights and
    rings.  specs: the kernels' cg_ring_spec array (ring_spec_array)."""
    return _UnrollRings.apply(world, T, every, specs, seed, mu, sigma, weights, rings)


class RingKernelBuilder(torch.nn.Module):
    """Lenia ring kernels h_k = sum_l b_kl S_kl / sum(...) (the construction of
    cella_nova_gb300/creature.py) as differentiable torch ops; the shells
    S_kl are fixed buffers."""

    def __init__(self, n, radii, ring_counts, device=None, dtype=torch.float64):
        super().__init__()
        from .creature import ring_shells
        self.counts = [int(c) for c in ring_counts]
        shells = [torch.from_numpy(ring_shells(n, float(R), c)) for R, c in zip(radii, self.counts)]
        for k, s in enumerate(shells):
            self.register_buffer(f"shells{k}", s.to(device=device, dtype=dtype))

    def forward(self, ring_weights):
        out = []
        for k, b in enumerate(ring_weights):
            S = getattr(self, f"shells{k}")
            hk = torch.tensordot(b.to(S.dtype), S, dims=1)
            out.append(hk / hk.sum())
        return torch.stack(out)


class DiffusionLeniaGPU(torch.nn.Module):
    """Differentiable DiffusionLenia with the GPU step: the parameters of
    train/diff_lenia_org.py's model (seed state, mu, sigma, growth weights;
    here per kernel in the orchestrator's c0/c1 order) plus the ring weights
    of each kernel."""

    def __init__(self, creature, device="cuda", autotune=True):
        super().__init__()
        cr = creature
        self.world = LeniaWorld(cr.n, cr.C, cr.c0, cr.c1, cr.temp, device)
        if autotune:
            self.world.autotune()
        f32 = dict(dtype=torch.float32, device=device)
        self.seed = torch.nn.Parameter(torch.tensor(cr.seed, **f32))
        self.mu = torch.nn.Parameter(torch.tensor(np.asarray(cr.mu), **f32))
        self.sigma = torch.nn.Parameter(torch.tensor(np.asarray(cr.sigma), **f32))
        self.weights = torch.nn.Parameter(torch.tensor(np.asarray(cr.weights), **f32))
        self.ring_weights = torch.nn.ParameterList(
            [torch.nn.Parameter(torch.tensor(np.asarray(b, np.float64), device=device))
             for b in cr.ring_weights])
        self.builder = RingKernelBuilder(cr.n, cr.ring_radius, [len(b) for b in cr.ring_weights],
                                         device=device)
        from .orchestrator import creature_ring_specs, ring_spec_array
        self.specs = ring_spec_array(creature_ring_specs(cr)[0])

    def kernels(self):
        """The spatial kernels (K, n, n) as differentiable torch ops (float64)."""
        return self.builder(list(self.ring_weights))

    def rings(self):
        """Ring weights padded to (K, 8), differentiable."""
        return torch.stack([torch.nn.functional.pad(b, (0, _abi.MAX_RINGS - b.numel()))
                            for b in self.ring_weights])

    def forward(self, T: int, every: int = 8):
        """x_T; the kernels are built on the GPU from the ring weights."""
        return unroll_rings(self.world, self.specs, self.seed, self.mu, self.sigma, self.weights,
                            self.rings(), T, every)
