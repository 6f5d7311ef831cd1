"""Batched gradient search: many candidate creatures optimised together.

Each iteration, for every candidate:
- build its ring kernels on the GPU from the current ring weights
  (cg_build_ring_kernels);
- fold mu/sigma/weights on the device (cg_set_params_device);
- unroll T steps with checkpoints (cg_unroll);
- take the loss MSE(x_T, target) and its gradient (cg_mse_grad);
- run the adjoint back to the seed, mu, sigma, weights and spectra
  (cg_unroll_backward), then bring the spectral gradient to space
  (cg_kernel_grad_spatial);
- from it, get the ring-weight gradients (cg_ring_weight_grad);
- take one Adam step on every parameter group (cg_adam_step).

That is the loop of the reference's training scripts (train/, torch autograd
plus torch.optim.Adam over a DiffusionLenia) with every kernel our own. The
first iteration runs eagerly; it allocates the library's scratch. The whole
iteration of all candidates is then captured once as a CUDA graph, Adam
included, and replayed. Candidates are spread over a few streams. Inside the
graph they run concurrently, since one 1024^2 world fills only part of the
GPU in its row phases.

torch provides the device memory, the streams and the graph capture; it runs
no compute here.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _abi
from ._abi import check, fptr, uptr
from .orchestrator import creature_ring_specs, ring_spec_array


def _v(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


@dataclass
class AdamConfig:
    lr_seed: float = 1e-3
    lr_params: float = 1e-3      # mu, sigma, growth weights
    lr_rings: float = 1e-2       # ring weights
    beta1: float = 0.9
    beta2: float = 0.999
    eps: float = 1e-8


class _Candidate:
    """Device state of one candidate: its world, parameters, Adam moments and
    the buffers of one forward/backward iteration."""

    def __init__(self, lib, cr, target, T, every, stream: torch.cuda.Stream):
        self.cr, self.stream = cr, stream
        n, C, K = cr.n, cr.C, cr.K
        dev = torch.device("cuda", torch.cuda.current_device())
        f32 = dict(dtype=torch.float32, device=dev)
        one = np.ones(K, np.float32)
        h = ctypes.c_void_p()
        c0 = np.ascontiguousarray(cr.c0, np.uint32)
        c1 = np.ascontiguousarray(cr.c1, np.uint32)
        check(lib.cg_create(n, C, K, uptr(c0), uptr(c1), fptr(one * 0.1), fptr(one * 0.05),
                            fptr(one), ctypes.c_float(cr.temp), ctypes.c_void_p(stream.cuda_stream),
                            ctypes.byref(h)))
        self.h = h
        specs, w = creature_ring_specs(cr)
        self.specs = ring_spec_array(specs)
        # parameters
        self.seed = torch.tensor(np.asarray(cr.seed, np.float32), **f32)
        self.params = torch.tensor(np.concatenate([cr.mu, cr.sigma, cr.weights]).astype(np.float32),
                                   **f32)                   # [mu | sigma | weights], 3K
        self.rings = torch.tensor(w, **f32)                 # (K, 8)
        self.target = torch.tensor(np.asarray(target, np.float32), **f32)
        # Adam moments
        self.m = [torch.zeros_like(p) for p in (self.seed, self.params, self.rings)]
        self.v = [torch.zeros_like(p) for p in (self.seed, self.params, self.rings)]
        # iteration buffers
        nck = (T - 1) // every + 1
        self.ckpt = torch.empty((nck, C, n, n), **f32)
        self.xT = torch.empty((C, n, n), **f32)
        self.gT = torch.empty((C, n, n), **f32)
        self.g0 = torch.empty((C, n, n), **f32)
        self.gtmp = torch.empty((C, n, n), **f32)
        self.seg = torch.empty((every, C, n, n), **f32)
        self.pgrad = torch.zeros(3 * K, dtype=torch.float64, device=dev)
        self.kgrad = torch.zeros((K, n // 2, n, 2), **f32)
        self.hbar = torch.empty((K, n, n), **f32)
        self.ring_grad = torch.zeros((K, _abi.MAX_RINGS), **f32)
        self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        self.scratch = torch.zeros(_abi.REDUCE_BLOCKS, dtype=torch.float64, device=dev)

    def close(self, lib):
        if self.h:
            check(lib.cg_destroy(self.h))
            self.h = None

    def autotune(self, lib, reps: int = 5):
        ms = np.zeros(4 * _abi.MAX_VARIANTS, dtype=np.float64)
        chosen = (ctypes.c_int * 4)()
        check(lib.cg_autotune(self.h, int(reps), ms.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              chosen))
        return list(chosen)

    def set_variants(self, lib, v):
        check(lib.cg_set_variants(self.h, (ctypes.c_int * 4)(*v)))


class GradientSearch:
    """Candidates (creatures of :func:`cella_nova_gb300.creature.make_creature`)
    optimised towards their targets with Adam, one CUDA graph per iteration."""

    def __init__(self, creatures, targets, T: int = 128, every: int = 16,
                 adam: AdamConfig | None = None, n_streams: int = 4, autotune: bool = True):
        self.lib = _abi.load()
        self.T, self.every = int(T), int(every)
        self.adam = adam or AdamConfig()
        self.streams = [torch.cuda.Stream() for _ in range(max(1, min(n_streams, len(creatures))))]
        self.cands = [_Candidate(self.lib, cr, tg, self.T, self.every,
                                 self.streams[i % len(self.streams)])
                      for i, (cr, tg) in enumerate(zip(creatures, targets))]
        self.step = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.graph = None
        self.iterations = 0
        if autotune:   # one tuning per grid side, shared by its candidates
            chosen = {}
            for c in self.cands:
                if c.cr.n not in chosen:
                    chosen[c.cr.n] = c.autotune(self.lib)
                else:
                    c.set_variants(self.lib, chosen[c.cr.n])

    def close(self):
        for c in self.cands:
            c.close(self.lib)
        self.cands = []
        self.graph = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- one iteration -----------------------------------------------------
    def _candidate_work(self, c: _Candidate):
        lib, a = self.lib, self.adam
        K = c.cr.K
        st = ctypes.c_void_p(c.stream.cuda_stream)
        check(lib.cg_build_ring_kernels(c.h, ctypes.cast(c.specs, ctypes.c_void_p), _v(c.rings)))
        p = c.params.data_ptr()
        check(lib.cg_set_params_device(c.h, ctypes.c_void_p(p), ctypes.c_void_p(p + 4 * K),
                                       ctypes.c_void_p(p + 8 * K)))
        check(lib.cg_unroll(c.h, _v(c.seed), self.T, self.every, _v(c.ckpt), _v(c.xT)))
        check(lib.cg_mse_grad(_v(c.xT), _v(c.target), c.xT.numel(), _v(c.gT), _v(c.loss),
                              _v(c.scratch), st))
        check(lib.cg_zero_grads(c.h, _v(c.pgrad), _v(c.kgrad)))
        check(lib.cg_unroll_backward(c.h, _v(c.ckpt), self.T, self.every, _v(c.gT), _v(c.g0),
                                     _v(c.pgrad), _v(c.kgrad), _v(c.seg), _v(c.gtmp)))
        check(lib.cg_kernel_grad_spatial(c.h, _v(c.kgrad), _v(c.hbar)))
        check(lib.cg_ring_weight_grad(c.h, ctypes.cast(c.specs, ctypes.c_void_p), _v(c.rings),
                                      _v(c.hbar), _v(c.ring_grad)))
        groups = [(c.seed, c.g0, None, a.lr_seed), (c.params, None, c.pgrad, a.lr_params),
                  (c.rings, c.ring_grad, None, a.lr_rings)]
        for (param, g32, g64, lr), m, v in zip(groups, c.m, c.v):
            check(lib.cg_adam_step(_v(param), _v(g32) if g32 is not None else None,
                                   _v(g64) if g64 is not None else None, _v(m), _v(v),
                                   param.numel(), ctypes.c_float(lr), ctypes.c_float(a.beta1),
                                   ctypes.c_float(a.beta2), ctypes.c_float(a.eps), _v(self.step),
                                   st))

    def _iteration(self):
        main = torch.cuda.current_stream()
        fork = torch.cuda.Event()
        fork.record(main)
        for s in self.streams:
            s.wait_event(fork)
        for c in self.cands:
            self._candidate_work(c)
        for s in self.streams:
            e = torch.cuda.Event()
            e.record(s)
            main.wait_event(e)
        check(self.lib.cg_count_step(_v(self.step), ctypes.c_void_p(main.cuda_stream or 1)))

    def run(self, iterations: int):
        """iterations Adam steps of every candidate (the first one eager, the
        rest graph replays)."""
        for _ in range(int(iterations)):
            if self.graph is None and self.iterations >= 1:
                self._capture()
            if self.graph is None:
                self._iteration()
            else:
                self.graph.replay()
            self.iterations += 1

    def run_eager(self, iterations: int):
        """The same iterations without the graph (for comparison)."""
        for _ in range(int(iterations)):
            self._iteration()
            self.iterations += 1

    def _capture(self):
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream()
        with torch.cuda.graph(g, stream=cap):
            self._iteration()
        torch.cuda.synchronize()
        self.graph = g

    # -- results -----------------------------------------------------------
    def losses(self) -> np.ndarray:
        """Loss of each candidate at the start of its last iteration."""
        torch.cuda.synchronize()
        return np.array([float(c.loss.item()) for c in self.cands])

    def parameters(self, i: int) -> dict:
        c = self.cands[i]
        K = c.cr.K
        torch.cuda.synchronize()
        p = c.params.cpu().numpy()
        return {"seed": c.seed.cpu().numpy(), "mu": p[:K], "sigma": p[K:2 * K],
                "weights": p[2 * K:], "ring_weights": c.rings.cpu().numpy()}

    def gradients(self, i: int) -> dict:
        """Gradients of candidate i's last iteration, with the state it
        started from (the seed before that iteration's Adam step) and its
        final state."""
        c = self.cands[i]
        K = c.cr.K
        torch.cuda.synchronize()
        g = c.pgrad.cpu().numpy()
        return {"loss": float(c.loss.item()), "seed": c.g0.cpu().numpy(), "mu": g[:K],
                "sigma": g[K:2 * K], "weights": g[2 * K:],
                "ring_weights": c.ring_grad.cpu().numpy(), "final": c.xT.cpu().numpy(),
                "initial": c.ckpt[0].cpu().numpy()}
