"""cg_mass_f64_noalloc: the FP64 mass sum for callers that cannot allocate.

Some callers cannot allocate device memory while they run: code inside a
memory budget that another component has already reserved, or a loop where
cudaMalloc's implicit device-wide synchronisation is not acceptable.  For
them the library offers one entry point that keeps its scratch in a fixed
device array instead of a cudaMalloc'd buffer.  This file checks it against
the allocating entry point (cg_mass_f64) on two calls in a row, so the second
call runs on the scratch the first one left behind.  It lives in a file of its
own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

from cella_nova_gb300 import GpuMaceLenia, _abi
from cella_nova_gb300.creature import make_creature

pytestmark = pytest.mark.gpu


def _noalloc(lib, dev_state, n, C, dev_out, stream):
    return lib.cg_mass_f64_noalloc(ctypes.c_void_p(dev_state), n, C, ctypes.c_void_p(dev_out),
                                   ctypes.c_void_p(stream))


def test_noalloc_mass_matches_allocating_entry_point():
    import torch
    cr = make_creature(256, 3, seed=31, radius=(10, 30), seed_box=128)
    with GpuMaceLenia.from_creature(cr) as sim:
        lib = sim._lib
        out = torch.full((cr.C,), -1.0, dtype=torch.float64, device="cuda")
        for call in range(2):
            sim.run_steps(5)              # a different state for each call
            ref = sim.mass_f64()          # allocating entry point (synchronises)
            rc = _noalloc(lib, sim.channel_ptr(), cr.n, cr.C, out.data_ptr(), sim.stream())
            _abi.check(rc)
            sim.synchronize()
            got = out.cpu().numpy()
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0,
                                       err_msg=f"call {call}")


def test_noalloc_mass_rejects_too_many_channels():
    import torch
    lib = _abi.load()
    x = torch.zeros((17, 16, 16), dtype=torch.float32, device="cuda")
    out = torch.zeros(17, dtype=torch.float64, device="cuda")
    rc = _noalloc(lib, x.data_ptr(), 16, 17, out.data_ptr(), 0)
    assert rc == -1
    assert "at most 16" in lib.cg_last_error().decode()


def test_noalloc_mass_leaves_free_device_memory_unchanged():
    """The property the entry point exists for, as far as the runtime shows
    it: after the first call on the device (which looks the scratch address
    up), further calls leave the device's free memory exactly as it was (no
    allocation outlives a call)."""
    import torch
    lib = _abi.load()
    x = torch.rand((4, 512, 512), dtype=torch.float32, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    _abi.check(_noalloc(lib, x.data_ptr(), 512, 4, out.data_ptr(), 0))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _abi.check(_noalloc(lib, x.data_ptr(), 512, 4, out.data_ptr(), 0))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    np.testing.assert_allclose(out.cpu().numpy(), x.double().sum(dim=(1, 2)).cpu().numpy(),
                               rtol=1e-12)
