"""TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.

Differentiable FP64 restatement of the DiffusionLenia step for gradient
checks.  It is torch (CPU, float64) with autograd, run only by tests/ as the
checker of the GPU adjoint.  It follows train/diff_lenia_org.py:27-53 (step,
compute_affinity) and train/lenia_org.py:93-136 (growth, get_fftconv) in the
orchestrator's kernel order (kernel k reads c0[k], feeds c1[k]); the spatial
ring kernels follow cella_nova_gb300/creature.py so that gradients reach the
ring weights.

It is pinned by tests/test_grad_oracle.py against (a) gradients of the
reference's own PyTorch model (tests/golden/grad_*.npz, made by
tests/golden/make_golden.py) and (b) FP64 central finite differences of the C
oracle (oracle/lenia_oracle.c).
"""
from __future__ import annotations

import numpy as np
import torch

from cella_nova_gb300.creature import ring_shells

DT = torch.float64


def box3(a):
    """Toroidal 3x3 sum over the last two axes (example.rs:275-286)."""
    s = torch.zeros_like(a)
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            s = s + torch.roll(a, (di, dj), dims=(-2, -1))
    return s


def step(x, kspec, c0, c1, mu, sigma, w, temp):
    """One step; x (C,n,n), kspec (K,n,n) complex128 full spectra."""
    C = x.shape[0]
    S = torch.fft.fft2(x)
    wsum = [torch.zeros_like(x[0]) for _ in range(C)]
    for k in range(kspec.shape[0]):
        u = torch.real(torch.fft.ifft2(S[int(c0[k])] * kspec[k]))
        g = 2.0 * torch.exp(-((u - mu[k]) ** 2) / (2.0 * sigma[k] ** 2)) - 1.0
        wsum[int(c1[k])] = wsum[int(c1[k])] + w[k] * g
    A = torch.exp(temp * torch.stack(wsum))
    Z = box3(A)
    return A * box3(x / Z)


class RingKernels:
    """Spatial ring kernels h_k = sum_l b_kl S_kl / sum(...) and their
    spectra, differentiable in the ring weights b."""

    def __init__(self, n, radii, ring_weights):
        self.n = n
        self.shells = [torch.from_numpy(ring_shells(n, float(R), len(b))) for R, b in
                       zip(radii, ring_weights)]

    def spectra(self, bs):
        out = []
        for S, b in zip(self.shells, bs):
            h = torch.tensordot(b, S, dims=1)
            h = h / h.sum()
            out.append(torch.fft.fft2(h.to(torch.complex128)))
        return torch.stack(out)


def unroll_loss(seed, kspec, c0, c1, mu, sigma, w, temp, T, target):
    x = seed
    for _ in range(T):
        x = step(x, kspec, c0, c1, mu, sigma, w, temp)
    return torch.mean((x - target) ** 2), x


def gradients(cr, T, target, *, kspec=None, ring=True):
    """d loss / d (seed, mu, sigma, w, ring weights) for MSE(x_T, target).

    kspec: override spectra (complex); otherwise built from the creature's
    ring parameters (then ring-weight gradients are returned)."""
    seed = torch.tensor(cr.seed, dtype=DT, requires_grad=True)
    mu = torch.tensor(np.asarray(cr.mu, np.float64), requires_grad=True)
    sg = torch.tensor(np.asarray(cr.sigma, np.float64), requires_grad=True)
    w = torch.tensor(np.asarray(cr.weights, np.float64), requires_grad=True)
    bs = [torch.tensor(np.asarray(b, np.float64), requires_grad=True) for b in cr.ring_weights]
    if kspec is None:
        rk = RingKernels(cr.n, cr.ring_radius, cr.ring_weights)
        ks = rk.spectra(bs)
    else:
        ks = torch.tensor(np.asarray(kspec), dtype=torch.complex128)
        ring = False
    tgt = torch.tensor(np.asarray(target), dtype=DT)
    loss, xT = unroll_loss(seed, ks, cr.c0, cr.c1, mu, sg, w, float(cr.temp), T, tgt)
    wrt = [seed, mu, sg, w] + (bs if ring else [])
    g = torch.autograd.grad(loss, wrt)
    out = {"loss": float(loss.detach()), "seed": g[0].numpy(), "mu": g[1].numpy(),
           "sigma": g[2].numpy(), "weights": g[3].numpy(), "final": xT.detach().numpy()}
    if ring:
        out["ring_weights"] = [gi.numpy() for gi in g[4:]]
    return out


def shifted_target(seed, dy=8, dx=16):
    """The seed translated by (+dx, +dy) pixels (x = columns, y = rows)."""
    return np.roll(np.asarray(seed), (dy, dx), axis=(-2, -1))
