"""TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.

Python side of the CPU oracle for the DiffusionLenia step of
anima-zetta/cella-nova.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only as the
checker; the product path never calls it.

Contents
--------
* ``build()`` / ``lib()``: compile and load ``liblenia_oracle.so`` (the C
  restatement of ml-rs/example.rs:164-303, FP64 and FP32 builds).
* ``step_c(...)``: one step through the C oracle (FP64 by default).
* ``step_np(...)``: numpy float64 twin of the same step (ml-rs/example.rs:
  164-303 with numpy's FFT in place of example.rs:42-126), used to cross-check
  the C build and as a fast oracle for larger grids.
* ``load_config_np`` / ``load_kernels_np``: restatement of
  ml-rs/config.rs:32-125 (JSON seed format with the c0/c1 swap, .bin kernel
  spectra with the spectral zero-padding resample).
* ``gauss_ring_kernels_np``: restatement of the reference's kernel generator
  (train/generate_kernel_json.py:106-146, ml-rs/example.rs:338-407).
* ``render_np`` / ``rgb24_np``: restatement of render_main
  (ml-rs/shaders/compute_1024.wgsl:428-443) and of download_render's byte
  conversion (ml-rs/orchestrator/mod.rs:322-329).

The oracle is pinned by tests/test_oracle.py against golden vectors that the
reference's own PyTorch model (train/diff_lenia_org.py) produced
(tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "liblenia_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile liblenia_oracle.so with plain gcc (oracle/Makefile)."""
    src = [os.path.join(_HERE, f) for f in ("lenia_oracle.c", "oracle_impl.h")]
    if force or not os.path.exists(_SO) or any(
            os.path.getmtime(s) > os.path.getmtime(_SO) for s in src):
        subprocess.run(["make", "-s", "-C", _HERE, "liblenia_oracle.so"], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        for suf, ct in (("_f64", ctypes.c_double), ("_f32", ctypes.c_float)):
            fn = getattr(L, "orc_step" + suf)
            P = ctypes.POINTER(ct)
            U = ctypes.POINTER(ctypes.c_uint32)
            fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, U, U, P,
                           P, P, ct, ctypes.c_int, ctypes.c_int, P, P]
            fn.restype = ctypes.c_int
            m = getattr(L, "orc_mass" + suf)
            m.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.POINTER(ctypes.c_double)]
            m.restype = None
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def step_c(state, kspec, c0, c1, mu, sigma, weight, temp, *, dtype=np.float64,
           faithful=False, nthreads=1, want_u=False, want_aff=False):
    """One step through the C oracle.

    state: (C, n, n) real; kspec: (K, n, n) complex full spectra.
    Returns (new_state, u or None, aff or None) in ``dtype``.
    """
    L = lib()
    C, n, _ = state.shape
    K = kspec.shape[0]
    ct = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    fn = L.orc_step_f64 if dtype == np.float64 else L.orc_step_f32
    st = np.ascontiguousarray(state, dtype=dtype).copy()
    ks = np.empty((K, n, n, 2), dtype=dtype)
    ks[..., 0] = kspec.real
    ks[..., 1] = kspec.imag
    c0a = np.ascontiguousarray(c0, dtype=np.uint32)
    c1a = np.ascontiguousarray(c1, dtype=np.uint32)
    mua = np.ascontiguousarray(mu, dtype=dtype)
    sga = np.ascontiguousarray(sigma, dtype=dtype)
    wa = np.ascontiguousarray(weight, dtype=dtype)
    u = np.empty((K, n, n), dtype=dtype) if want_u else None
    aff = np.empty((C, n, n), dtype=dtype) if want_aff else None
    null = ctypes.POINTER(ct)()
    rc = fn(n, C, K, _ptr(st, ct), _ptr(ks, ct), _ptr(c0a, ctypes.c_uint32),
            _ptr(c1a, ctypes.c_uint32), _ptr(mua, ct), _ptr(sga, ct), _ptr(wa, ct),
            ct(temp), int(faithful), int(nthreads),
            _ptr(u, ct) if u is not None else null,
            _ptr(aff, ct) if aff is not None else null)
    if rc != 0:
        raise MemoryError("oracle step failed")
    return st, u, aff


def mass_c(state, dtype=np.float64):
    L = lib()
    C, n, _ = state.shape
    ct = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    fn = L.orc_mass_f64 if dtype == np.float64 else L.orc_mass_f32
    st = np.ascontiguousarray(state, dtype=dtype)
    out = np.empty(C, dtype=np.float64)
    fn(n, C, _ptr(st, ct), _ptr(out, ctypes.c_double))
    return out


def box3(a):
    """Toroidal 3x3 box sum over the last two axes (example.rs:275-286)."""
    s = np.zeros_like(a)
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            s += np.roll(a, (di, dj), axis=(-2, -1))
    return s


def step_np(state, kspec, c0, c1, mu, sigma, weight, temp, *, want_u=False,
            want_aff=False):
    """numpy float64 twin of the step (example.rs:164-303).

    u_k = Re(ifft2(fft2(state[c0[k]]) * kspec[k])); growth per example.rs:
    244-255; A = exp(temp * wsum); diffusion per example.rs:272-303.
    """
    state = np.asarray(state, dtype=np.float64)
    C, n, _ = state.shape
    K = kspec.shape[0]
    S = np.fft.fft2(state)
    u = np.empty((K, n, n))
    for k in range(K):
        u[k] = np.real(np.fft.ifft2(S[c0[k]] * kspec[k]))
    wsum = np.zeros((C, n, n))
    for k in range(K):
        d = u[k] - mu[k]
        g = 2.0 * np.exp(-0.5 * d * d / (sigma[k] * sigma[k])) - 1.0
        wsum[c1[k]] += g * weight[k]
    A = np.exp(temp * wsum)
    Z = box3(A)
    new = A * box3(state / Z)
    return new, (u if want_u else None), (A if want_aff else None)


# ---------------------------------------------------------------------------
# File formats (restating ml-rs/config.rs:32-125)
# ---------------------------------------------------------------------------

def load_config_np(path):
    """seed/{name}.json -> dict with API-order c0 (input) / c1 (output).

    config.rs:40 swaps the JSON c0 and c1 fields on load.
    """
    with open(path) as f:
        cfg = json.load(f)
    n = int(cfg["seed_size"])
    C = int(cfg["num_channels"])
    K = int(cfg["num_kernels"])
    seed = np.asarray(cfg["seed_channels"], dtype=np.float64).reshape(C, n, n)
    return {
        "n": n, "C": C, "K": K, "seed": seed,
        "c0": np.asarray(cfg["c1"], dtype=np.uint32),
        "c1": np.asarray(cfg["c0"], dtype=np.uint32),
        "mu": np.asarray(cfg["growth_mu"], dtype=np.float32),
        "sigma": np.asarray(cfg["growth_sigma"], dtype=np.float32),
        "weights": np.asarray(cfg["growth_weights"], dtype=np.float32),
    }


def load_kernels_np(path, K, target):
    """kernels/{name}_{size}.bin -> (K, target, target) complex64.

    config.rs:61-65: the source size is sqrt(file_size / K / 8).  Same size:
    read as is (config.rs:74-80).  Other size: centre with an fftshift,
    zero-pad to the target, shift back (config.rs:81-116).
    """
    raw = np.fromfile(path, dtype="<f4")
    kb = raw.size * 4 // K
    src = int(np.sqrt(kb / 8))
    data = raw[: K * src * src * 2].reshape(K, src, src, 2)
    spec = (data[..., 0] + 1j * data[..., 1]).astype(np.complex64)
    if src == target:
        return spec
    out = np.zeros((K, target, target), dtype=np.complex64)
    hs, hd = src // 2, target // 2
    pad = (target - src) // 2
    for k in range(K):
        centered = np.roll(spec[k], (hs, hs), axis=(0, 1))
        big = np.zeros((target, target), dtype=np.complex64)
        big[pad:pad + src, pad:pad + src] = centered
        out[k] = np.roll(big, (hd, hd), axis=(0, 1))
    return out


def render_np(state):
    """Packed 0x00RRGGBB words (n, n) uint32 from channels 0, 1, 2 of an f32
    state: level = u32(sqrt(clamp(1.5 c, 0, 1)) * 255), all in float32
    (compute_1024.wgsl:428-443).  Channels the state lacks give 0; a NaN
    clamps to 0 (fmax/fmin semantics)."""
    st = np.asarray(state, dtype=np.float32)

    def level(c):
        v = np.fmin(np.fmax(c * np.float32(1.5), np.float32(0.0)), np.float32(1.0))
        return (np.sqrt(v) * np.float32(255.0)).astype(np.uint32)

    out = level(st[0]) << np.uint32(16)
    if st.shape[0] > 1:
        out |= level(st[1]) << np.uint32(8)
    if st.shape[0] > 2:
        out |= level(st[2])
    return out


def rgb24_np(packed):
    """download_render's conversion (mod.rs:322-329): (n, n) words -> (n, n, 3)
    bytes R, G, B."""
    p = np.asarray(packed, dtype=np.uint32)
    return np.stack([(p >> 16) & 255, (p >> 8) & 255, p & 255], axis=-1).astype(np.uint8)


def gauss_ring_kernels_np(size, global_r, radii, widths):
    """(K, size, size) complex128 spectra of the reference's Gaussian ring
    kernels (train/generate_kernel_json.py:106-146): per kernel, distance
    from the grid centre size//2 scaled by global_r * radius, a sigmoid gate
    sigmoid(-(d-1)*10) (sigmoid(x) = (tanh(x/2)+1)/2, :102-103) times
    exp(-(d-1/2)^2 / (2 width^2)), normalised to sum 1, ifftshift-ed to put
    the centre at [0, 0], then fft2.  Float64 throughout (the generator
    builds float32 values; the spectra differ from it at the 1e-7 level)."""
    mid = size // 2
    i = np.arange(size, dtype=np.float64) - mid
    dist = np.sqrt(i[:, None] ** 2 + i[None, :] ** 2)
    out = []
    for radius, width in zip(radii, widths):
        d = dist / (global_r * radius)
        sig = 0.5 * (np.tanh(-(d - 1.0) * 10.0 / 2.0) + 1.0)
        val = sig * np.exp(-((d - 0.5) ** 2) / (2.0 * width * width))
        total = val.sum()
        if total > 0:
            val = val / total
        out.append(np.fft.fft2(np.fft.ifftshift(val)))
    return np.stack(out)

