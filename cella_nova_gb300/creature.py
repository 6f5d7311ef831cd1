"""Seeded synthetic creatures written in the reference's two file formats.

The reference's 66 shipped creatures (``seed/*.json`` + ``kernels/*.bin``) are
not available, so workloads are generated here with numpy ``default_rng``.
The on-disk formats are the ones ml-rs/config.rs reads and
train/generate_kernel_json.py writes:

* ``seed/{name}.json`` (generate_kernel_json.py:195-215, config.rs:14-25):
  ``seed_size``, ``num_channels``, ``num_kernels``, ``seed_channels`` (C lists
  of n*n f64, row-major), ``c0``, ``c1``, ``growth_mu``, ``growth_sigma``,
  ``growth_weights``.  JSON ``c1`` is the *input* channel and JSON ``c0`` the
  output channel; config.rs:40 swaps them into the orchestrator's order.
  Extra keys (``temp``, ``ring_radius``, ``ring_weights``) are ignored by
  the reference's loader (serde skips unknown fields) and carry what this
  generator drew.
* ``kernels/{name}_{n}.bin`` (generate_kernel_json.py:182-192,
  config.rs:49-80): K blocks of n*n complex64 little-endian (re, im), the
  FFT of the origin-centred spatial kernel.

Kernel construction (a Lenia ring kernel): r = |x| / R_k with the distance
measured on the torus from the origin; B rings with weights b; inside ring
l = floor(r*B) the shell is exp(4 - 1/(t(1-t))), t = frac(r*B), zero for
r >= 1; the kernel is normalised to sum 1 and transformed in float64.
"""
from __future__ import annotations

import json
import struct
import os
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Creature:
    """One DiffusionLenia instance in the orchestrator's (post-swap) order.

    ``c0[k]`` is the channel kernel k reads, ``c1[k]`` the channel its growth
    feeds (ml-rs/orchestrator/mod.rs:52-54).
    """
    n: int
    C: int
    K: int
    seed: np.ndarray            # (C, n, n) float64
    kspec: np.ndarray           # (K, n, n) complex64
    c0: np.ndarray              # (K,) uint32, input channel
    c1: np.ndarray              # (K,) uint32, output channel
    mu: np.ndarray              # (K,) float32
    sigma: np.ndarray           # (K,) float32
    weights: np.ndarray         # (K,) float32
    temp: float = 1.0
    ring_radius: np.ndarray = field(default_factory=lambda: np.zeros(0))
    ring_weights: list = field(default_factory=list)


def torus_radius(n: int) -> np.ndarray:
    """Distance of every grid point from the origin on an n x n torus."""
    d = (np.arange(n) + n // 2) % n - n // 2
    return np.sqrt(d[:, None].astype(np.float64) ** 2 + d[None, :].astype(np.float64) ** 2)


def ring_shells(n: int, R: float, B: int) -> np.ndarray:
    """(B, n, n) float64: ring l's shell exp(4 - 1/(t(1-t))) on its annulus."""
    r = torus_radius(n) / R
    rb = r * B
    idx = np.floor(rb).astype(np.int64)
    t = rb - idx
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        core = np.where((t > 0) & (t < 1), np.exp(4.0 - 1.0 / (t * (1.0 - t))), 0.0)
    core = np.where(r < 1.0, core, 0.0)
    out = np.zeros((B, n, n))
    for l in range(B):
        out[l] = np.where(idx == l, core, 0.0)
    return out


def ring_kernel(n: int, R: float, b) -> np.ndarray:
    """Spatial ring kernel (n, n) float64, origin-centred, summing to 1."""
    b = np.asarray(b, dtype=np.float64)
    k = np.tensordot(b, ring_shells(n, R, len(b)), axes=1)
    s = k.sum()
    return k / s if s > 0 else k


def _kernel_spectrum_torch(n: int, R: float, b, device) -> np.ndarray:
    """ring_kernel + fft2 in float64 with torch on `device` (same math)."""
    import torch
    d = (torch.arange(n, device=device, dtype=torch.float64) + n // 2) % n - n // 2
    r = torch.sqrt(d[:, None] ** 2 + d[None, :] ** 2) / R
    B = len(b)
    rb = r * B
    idx = torch.floor(rb)
    t = rb - idx
    inside = (t > 0) & (t < 1) & (r < 1.0)
    tt = torch.where(inside, t, torch.full_like(t, 0.5))
    core = torch.where(inside, torch.exp(4.0 - 1.0 / (tt * (1.0 - tt))), torch.zeros_like(t))
    bw = torch.tensor(list(b) + [0.0], dtype=torch.float64, device=device)
    k = core * bw[idx.clamp(0, B).long()]
    s = k.sum()
    if float(s) > 0:
        k = k / s
    return torch.fft.fft2(k).to(torch.complex64).cpu().numpy()


def all_pairs(C: int):
    """Kernels over every (input, output) pair, in the orchestrator's order.

    JSON order of the reference config generator is c0=k%C, c1=k//C
    (generate_kernel_json.py:72-73); after config.rs:40's swap the input
    channel is k//C and the output channel k%C.
    """
    k = np.arange(C * C)
    return (k // C).astype(np.uint32), (k % C).astype(np.uint32)


def make_creature(n: int, C: int = 3, *, seed: int = 0, K: int | None = None,
                  c0=None, c1=None, radius=None, temp: float = 1.0,
                  seed_box: int = 256, mu_range=(0.05, 0.3),
                  sigma_range=(0.01, 0.08), device=None) -> Creature:
    """Draw a creature from ``default_rng(seed)``.

    radius: (lo, hi) for R_k; default scales (12, 30) px at 1024^2 with n.
    seed_box: side of the central square seeded with U[0,1] (clipped to n/2).
    device: if given (a torch device), the kernel spectra are computed there
    with torch in float64 instead of numpy (same draws, same math).
    """
    rng = np.random.default_rng(seed)
    if c0 is None or c1 is None:
        c0, c1 = all_pairs(C)
    c0 = np.asarray(c0, dtype=np.uint32)
    c1 = np.asarray(c1, dtype=np.uint32)
    K = len(c0) if K is None else K
    if radius is None:
        radius = (12.0 * n / 1024.0, 30.0 * n / 1024.0)
    lo, hi = radius
    lo = max(lo, 2.0)
    hi = max(hi, lo + 1.0)
    hi = min(hi, n / 2 - 1)
    R = rng.uniform(lo, hi, size=K)
    rings = []
    kspec = np.empty((K, n, n), dtype=np.complex64)
    for k in range(K):
        B = int(rng.integers(1, 4))
        b = rng.uniform(0.0, 1.0, size=B)
        b[rng.integers(0, B)] = max(b.max(), 0.25)   # never an all-zero kernel
        rings.append(b.tolist())
        if device is not None:
            kspec[k] = _kernel_spectrum_torch(n, R[k], b, device)
        else:
            kspec[k] = np.fft.fft2(ring_kernel(n, R[k], b)).astype(np.complex64)
    mu = rng.uniform(*mu_range, size=K).astype(np.float32)
    sigma = rng.uniform(*sigma_range, size=K).astype(np.float32)
    w = rng.uniform(0.0, 1.0, size=K)
    for c in range(C):
        sel = c1 == c
        s = w[sel].sum()
        if s > 0:
            w[sel] /= s
    box = min(seed_box, n // 2)
    st = np.zeros((C, n, n))
    o = (n - box) // 2
    st[:, o:o + box, o:o + box] = rng.uniform(0.0, 1.0, size=(C, box, box))
    return Creature(n=n, C=C, K=K, seed=st, kspec=kspec, c0=c0, c1=c1, mu=mu,
                    sigma=sigma, weights=w.astype(np.float32), temp=float(temp),
                    ring_radius=R, ring_weights=rings)


def write_kernels_bin(path: str, kspec: np.ndarray) -> None:
    """K x n x n complex64 little-endian, interleaved (re, im)."""
    a = np.empty(kspec.shape + (2,), dtype="<f4")
    a[..., 0] = kspec.real
    a[..., 1] = kspec.imag
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    a.tofile(path)


def write_seed_json(path: str, cr: Creature) -> None:
    """Seed JSON in the reference's field order and c0/c1 orientation."""
    data = {
        "seed_size": cr.n,
        "num_channels": cr.C,
        "num_kernels": cr.K,
        "seed_channels": [cr.seed[c].ravel().tolist() for c in range(cr.C)],
        # JSON c0 is the output channel, JSON c1 the input (config.rs:35-40)
        "c0": [int(x) for x in cr.c1],
        "c1": [int(x) for x in cr.c0],
        "growth_mu": [float(x) for x in cr.mu],
        "growth_sigma": [float(x) for x in cr.sigma],
        "growth_weights": [float(x) for x in cr.weights],
        "temp": cr.temp,
        "ring_radius": [float(x) for x in cr.ring_radius],
        "ring_weights": cr.ring_weights,
    }
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as f:
        json.dump(data, f)


def write_seed_bin(path: str, cr: Creature) -> None:
    """The binary twin of the seed JSON (magic CNSEED01; layout in
    include/cella_gpu.h): the JSON's fields, c0/c1 in the JSON's order."""
    K = cr.K
    parts = [b"CNSEED01", struct.pack("<IIIf", cr.n, cr.C, K, float(cr.temp)),
             np.asarray(cr.c1, dtype="<u4").tobytes(),    # JSON c0 (output)
             np.asarray(cr.c0, dtype="<u4").tobytes(),    # JSON c1 (input)
             np.asarray(cr.mu, dtype="<f4").tobytes(),
             np.asarray(cr.sigma, dtype="<f4").tobytes(),
             np.asarray(cr.weights, dtype="<f4").tobytes()]
    head = b"".join(parts)
    head += b"\0" * (-len(head) % 8)
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "wb") as f:
        f.write(head)
        f.write(np.ascontiguousarray(cr.seed, dtype="<f8").tobytes())


def write_creature(root: str, name: str, cr: Creature) -> tuple[str, str]:
    """Write ``{root}/seed/{name}.json`` and ``{root}/kernels/{name}_{n}.bin``."""
    js = os.path.join(root, "seed", f"{name}.json")
    kb = os.path.join(root, "kernels", f"{name}_{cr.n}.bin")
    write_seed_json(js, cr)
    write_kernels_bin(kb, cr.kspec)
    return js, kb
