"""cella_nova_gb300 — GB300-native (sm_103a) DiffusionLenia step.

Drop-in for the wgpu path behind ``GpuMaceLenia`` in anima-zetta/cella-nova
(ml-rs/orchestrator/mod.rs).  The product is ``libcella_gpu.so`` and its C
ABI (include/cella_gpu.h); this package is its Python binding:

* :class:`GpuMaceLenia`, :func:`load_config`, :func:`load_kernels`,
  :func:`setup_simulation` — the orchestrator and config.rs API;
  :func:`save_config_bin` writes the binary twin of the seed JSON.
* :class:`GpuMaceLeniaBatch` — many worlds stepped together.
* :mod:`cella_nova_gb300.autograd` — the differentiable unroll.
* :mod:`cella_nova_gb300.creature` — seeded synthetic creatures in the
  reference's file formats.
* :mod:`cella_nova_gb300.build` — builds the library in-tree.
"""
from ._abi import CellaError, load as load_library  # noqa: F401
from .orchestrator import (GpuMaceLenia, GpuMaceLeniaBatch, load_config, load_kernels,  # noqa: F401
                           save_config_bin, setup_simulation)

__all__ = ["CellaError", "GpuMaceLenia", "GpuMaceLeniaBatch", "load_config", "load_kernels",
           "save_config_bin", "setup_simulation", "load_library"]
