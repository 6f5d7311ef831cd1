"""The C ABI surface (CPU only: no call here launches device work)."""
import ctypes
import os
import re

import numpy as np
import pytest

from cella_nova_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(cg_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_builds_and_loads():
    lib = _abi.load()
    assert b"sm_103a" in lib.cg_version()


def test_every_declared_symbol_is_exported():
    lib = _abi.load()
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
        assert name in _abi.SIGNATURES, f"{name} has no ctypes signature"


def _create(n=64, C=3, K=9, c0=None, c1=None, mu=None, sigma=None, w=None, temp=1.0):
    lib = _abi.load()
    c0 = np.zeros(K, np.uint32) if c0 is None else np.asarray(c0, np.uint32)
    c1 = np.zeros(K, np.uint32) if c1 is None else np.asarray(c1, np.uint32)
    mu = np.full(K, 0.1, np.float32) if mu is None else np.asarray(mu, np.float32)
    sigma = np.full(K, 0.05, np.float32) if sigma is None else np.asarray(sigma, np.float32)
    w = np.full(K, 1.0, np.float32) if w is None else np.asarray(w, np.float32)
    h = ctypes.c_void_p()
    rc = lib.cg_create(n, C, K, _abi.uptr(c0), _abi.uptr(c1), _abi.fptr(mu), _abi.fptr(sigma),
                       _abi.fptr(w), ctypes.c_float(temp), None, ctypes.byref(h))
    return rc, lib.cg_last_error().decode()


@pytest.mark.parametrize("kw,code,msg", [
    (dict(n=100), -1, "power of two"),
    (dict(n=8), -7, "outside"),
    (dict(n=4096), -7, "outside"),
    (dict(C=0), -1, "channel count"),
    (dict(C=17, K=1), -1, "channel count"),
    (dict(K=0), -1, "kernel count"),
    (dict(K=65), -1, "kernel count"),
    (dict(C=2, K=2, c0=[0, 2]), -1, "maps channel"),
    (dict(C=2, K=2, c1=[3, 0]), -1, "maps channel"),
    (dict(K=1, sigma=[0.0]), -1, "zero-sigma"),
    (dict(K=1, mu=[float("nan")]), -1, "non-finite"),
    (dict(K=1, w=[float("inf")]), -1, "non-finite"),
    (dict(K=1, temp=float("nan")), -1, "temp"),
])
def test_create_rejects_bad_arguments(kw, code, msg):
    rc, err = _create(**kw)
    assert rc == code, err
    assert msg in err


def test_null_handles_are_rejected():
    lib = _abi.load()
    assert lib.cg_destroy(None) == -1
    assert lib.cg_step(None, 1) == -1
    assert lib.cg_iterate(None) == -1
    assert lib.cg_synchronize(None) == -1
    out = np.zeros(4)
    assert lib.cg_timed_iterate(None, _abi.dptr(out)) == -1
    assert "NULL" in lib.cg_last_error().decode()
