"""ctypes binding of include/cella_gpu.h (libcella_gpu.so, built in-tree).

This is the same C ABI a Rust host binds with `extern "C"` declarations;
Python uses it for tests, the benchmark and the torch autograd wrapper.  There is no fallback:
if the library cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

# variants per phase in the autotuner's tables (CG_MAX_VARIANTS)
MAX_VARIANTS = 5
_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libcella_gpu.so")

CG_OK = 0
STATUS = {
    -1: "CG_ERR_ARG", -2: "CG_ERR_OOM", -3: "CG_ERR_CUDA", -4: "CG_ERR_TIMEOUT",
    -5: "CG_ERR_IO", -6: "CG_ERR_FORMAT", -7: "CG_ERR_UNSUPPORTED",
}


class CellaError(RuntimeError):
    """A libcella_gpu call returned a negative status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code


class cg_config(ctypes.Structure):
    _fields_ = [
        ("seed_size", ctypes.c_int), ("num_channels", ctypes.c_int),
        ("num_kernels", ctypes.c_int),
        ("seed_channels", ctypes.POINTER(ctypes.c_double)),
        ("c0", ctypes.POINTER(ctypes.c_uint32)), ("c1", ctypes.POINTER(ctypes.c_uint32)),
        ("growth_mu", ctypes.POINTER(ctypes.c_float)),
        ("growth_sigma", ctypes.POINTER(ctypes.c_float)),
        ("growth_weights", ctypes.POINTER(ctypes.c_float)),
        ("temp", ctypes.c_float),
    ]


class cg_ring_spec(ctypes.Structure):
    _fields_ = [("family", ctypes.c_int), ("rings", ctypes.c_int), ("radius", ctypes.c_float),
                ("width", ctypes.c_float)]


RING_SHELL, RING_GAUSS, MAX_RINGS = 0, 1, 8
REDUCE_BLOCKS = 296   # CG_REDUCE_BLOCKS

_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_FP = ctypes.POINTER(ctypes.c_float)
_DP = ctypes.POINTER(ctypes.c_double)
_UP = ctypes.POINTER(ctypes.c_uint32)

# name: (argtypes, restype) — every function include/cella_gpu.h declares.
SIGNATURES = {
    "cg_last_error": ([], ctypes.c_char_p),
    "cg_version": ([], ctypes.c_char_p),
    "cg_create": ([_I, _I, _I, _UP, _UP, _FP, _FP, _FP, _F, _P, ctypes.POINTER(_P)], _I),
    "cg_destroy": ([_P], _I),
    "cg_set_kernel": ([_P, _I, _FP], _I),
    "cg_upload_channel": ([_P, _I, _DP], _I),
    "cg_set_kernel_device": ([_P, _I, _P], _I),
    "cg_set_kernels_spatial_device": ([_P, _P], _I),
    "cg_set_params": ([_P, _FP, _FP, _FP, _F], _I),
    "cg_set_params_device": ([_P, _P, _P, _P], _I),
    "cg_build_ring_kernels": ([_P, _P, _P], _I),
    "cg_mse_grad": ([_P, _P, ctypes.c_size_t, _P, _P, _P, _P], _I),
    "cg_adam_step": ([_P, _P, _P, _P, _P, ctypes.c_size_t, _F, _F, _F, _F, _P, _P], _I),
    "cg_count_step": ([_P, _P], _I),
    "cg_ring_weight_grad": ([_P, _P, _P, _P, _P], _I),
    "cg_iterate_and_render": ([_P], _I),
    "cg_render": ([_P], _I),
    "cg_download_render": ([_P, ctypes.POINTER(ctypes.c_uint8)], _I),
    "cg_download_render_packed": ([_P, _UP], _I),
    "cg_render_ptr": ([_P, ctypes.POINTER(_P)], _I),
    "cg_stream_frames": ([_P, _I, _I, _I], _I),
    "cg_check_bounded_wait": ([_P, _I], _I),
    "cg_step_host_async": ([_P, _DP, _FP, _I], _I),
    "cg_host_wait": ([_P], _I),
    "cg_step_from": ([_P, _P, _P], _I),
    "cg_step_backward": ([_P, _P, _P, _P, _P, _P], _I),
    "cg_kernel_grad_spatial": ([_P, _P, _P], _I),
    "cg_zero_grads": ([_P, _P, _P], _I),
    "cg_unroll": ([_P, _P, _I, _I, _P, _P], _I),
    "cg_unroll_backward": ([_P, _P, _I, _I, _P, _P, _P, _P, _P, _P], _I),
    "cg_upload_channel_f32": ([_P, _I, _FP], _I),
    "cg_iterate": ([_P], _I),
    "cg_step": ([_P, _I], _I),
    "cg_iterate_on": ([_P, _P], _I),
    "cg_download_channels": ([_P, _FP], _I),
    "cg_download_conv_real": ([_P, _FP], _I),
    "cg_download_affinity": ([_P, _FP], _I),
    "cg_timed_iterate": ([_P, _DP], _I),
    "cg_profile_kernels": ([_P, _I, _DP], _I),
    "cg_autotune": ([_P, _I, _DP, ctypes.POINTER(_I)], _I),
    "cg_set_variants": ([_P, ctypes.POINTER(_I)], _I),
    "cg_kernels_real": ([_P, ctypes.POINTER(_I)], _I),
    "cg_set_graph_layout": ([_P, _I], _I),
    "cg_get_graph_layout": ([_P, ctypes.POINTER(_I)], _I),
    "cg_get_variants": ([_P, ctypes.POINTER(_I)], _I),
    "cg_mass_f64": ([_P, _DP], _I),
    "cg_mass_f64_noalloc": ([_P, _I, _I, _P, _P], _I),
    "cg_channel_ptr": ([_P, ctypes.POINTER(_P)], _I),
    "cg_stream": ([_P, ctypes.POINTER(_P)], _I),
    "cg_synchronize": ([_P], _I),
    "cg_batch_create": ([_I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), _UP, _UP,
                         _FP, _FP, _FP, _FP, _P, ctypes.POINTER(_P)], _I),
    "cg_batch_destroy": ([_P], _I),
    "cg_batch_set_kernel": ([_P, _I, _I, _FP], _I),
    "cg_batch_upload_channel": ([_P, _I, _I, _DP], _I),
    "cg_batch_step": ([_P, _I], _I),
    "cg_batch_download_channels": ([_P, _I, _FP], _I),
    "cg_batch_mass_f64": ([_P, _I, _DP], _I),
    "cg_batch_synchronize": ([_P], _I),
    "cg_batch_profile": ([_P, _I, _DP], _I),
    "cg_batch_stream": ([_P, ctypes.POINTER(_P)], _I),
    "cg_batch_info": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "cg_batch_autotune": ([_P, _I, ctypes.POINTER(_I), _DP], _I),
    "cg_batch_set_variants": ([_P, _I, ctypes.POINTER(_I)], _I),
    "cg_batch_set_mode": ([_P, _I, _I], _I),
    "cg_batch_get_mode": ([_P, _I, ctypes.POINTER(_I)], _I),
    "cg_load_config_json": ([ctypes.c_char_p, ctypes.POINTER(cg_config)], _I),
    "cg_free_config": ([ctypes.POINTER(cg_config)], None),
    "cg_load_config_bin": ([ctypes.c_char_p, ctypes.POINTER(cg_config)], _I),
    "cg_save_config_bin": ([ctypes.c_char_p, ctypes.POINTER(cg_config)], _I),
    "cg_load_kernels_bin": ([ctypes.c_char_p, _I, _I, _FP], _I),
    "cg_kernels_bin_size": ([ctypes.c_char_p, _I, ctypes.POINTER(_I)], _I),
}

_lib = None


def load(path: str | None = None):
    """Load libcella_gpu.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (argt, rest) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argt
        fn.restype = rest
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != CG_OK:
        msg = load().cg_last_error().decode(errors="replace")
        raise CellaError(rc, msg)


def fptr(a):
    return a.ctypes.data_as(_FP)


def dptr(a):
    return a.ctypes.data_as(_DP)


def uptr(a):
    return a.ctypes.data_as(_UP)
