"""GpuMaceLenia — the reference orchestrator's API over the C ABI.

Mirrors ml-rs/orchestrator/mod.rs (method names, argument meaning and
order, panics turned into :class:`CellaError`) so that the reference's own
drivers (main.rs:88-140, profile.rs:32-108, save_pngs.rs:112-135) read the
same against this class.  Every method is one libcella_gpu call; the step
runs on the GPU as captured CUDA graphs.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import check, dptr, fptr, uptr


class GpuMaceLenia:
    """One DiffusionLenia world on the current CUDA device.

    ``GpuMaceLenia(shape, num_channels, num_kernels, c0, c1, mu, sigma,
    weights, temp)`` follows ``GpuMaceLenia::new`` (mod.rs:79-90):
    ``shape`` is ``(n, n)``, ``c0[k]`` the channel kernel k reads and
    ``c1[k]`` the channel its growth feeds.
    """

    def __init__(self, shape, num_channels, num_kernels, c0, c1, mu, sigma, weights,
                 temp=1.0, stream=None):
        shape = tuple(int(s) for s in shape)
        if len(shape) != 2:
            raise ValueError("DiffusionLenia requires 2D grids")          # mod.rs:94
        if shape[0] != shape[1]:
            raise ValueError("only square grids are supported")          # growth.rs:44
        self._lib = _abi.load()
        self.n = shape[0]
        self.shape = shape
        self.num_channels = int(num_channels)
        self.num_kernels = int(num_kernels)
        self.total_elements = self.n * self.n
        K = self.num_kernels
        self.c0 = np.ascontiguousarray(c0, dtype=np.uint32)
        self.c1 = np.ascontiguousarray(c1, dtype=np.uint32)
        self.mu = np.ascontiguousarray(mu, dtype=np.float32)
        self.sigma = np.ascontiguousarray(sigma, dtype=np.float32)
        self.weights = np.ascontiguousarray(weights, dtype=np.float32)
        self.temp = float(temp)
        for name in ("c0", "c1", "mu", "sigma", "weights"):
            if getattr(self, name).shape != (K,):
                raise ValueError(f"{name} must have num_kernels = {K} entries")
        h = ctypes.c_void_p()
        check(self._lib.cg_create(self.n, self.num_channels, K, uptr(self.c0), uptr(self.c1),
                                  fptr(self.mu), fptr(self.sigma), fptr(self.weights),
                                  ctypes.c_float(self.temp),
                                  ctypes.c_void_p(stream) if stream else None,
                                  ctypes.byref(h)))
        self._h = h

    # -- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            check(self._lib.cg_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- uploads (mod.rs:207-226) -----------------------------------------
    def set_kernel(self, kernel_fft, kernel_idx):
        """Kernel ``kernel_idx``'s full n x n complex spectrum (mod.rs:207)."""
        a = np.asarray(kernel_fft)
        if a.size != self.total_elements:
            raise ValueError(f"kernel spectrum has {a.size} values, expected "
                             f"{self.total_elements}")                     # mod.rs:208
        inter = np.empty((self.total_elements, 2), dtype=np.float32)
        flat = a.reshape(-1)
        if np.iscomplexobj(flat):
            inter[:, 0] = flat.real
            inter[:, 1] = flat.imag
        else:
            inter[:] = flat.reshape(-1, 2) if flat.size == 2 * self.total_elements else 0
        check(self._lib.cg_set_kernel(self._h, int(kernel_idx), fptr(inter)))

    def set_kernel_device(self, dev_ptr: int, kernel_idx):
        """Kernel ``kernel_idx``'s full spectrum from device memory (n*n
        interleaved f32 pairs), enqueued on the handle's stream."""
        check(self._lib.cg_set_kernel_device(self._h, int(kernel_idx), ctypes.c_void_p(dev_ptr)))

    def set_kernels_spatial_device(self, dev_ptr: int):
        """All K kernels from their spatial form: K*n*n f32 on the device
        (origin at [0][0]); the library takes the spectra with its own FFTs
        (cg_set_kernels_spatial_device)."""
        check(self._lib.cg_set_kernels_spatial_device(self._h, ctypes.c_void_p(dev_ptr)))

    def upload_channel(self, data, channel):
        """Channel ``channel`` from n*n f64 values (mod.rs:217-226)."""
        a = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
        if a.size != self.total_elements:
            raise ValueError(f"channel has {a.size} values, expected {self.total_elements}")
        check(self._lib.cg_upload_channel(self._h, int(channel), dptr(a)))

    def upload_channel_f32(self, data, channel):
        a = np.ascontiguousarray(data, dtype=np.float32).reshape(-1)
        if a.size != self.total_elements:
            raise ValueError(f"channel has {a.size} values, expected {self.total_elements}")
        check(self._lib.cg_upload_channel_f32(self._h, int(channel), fptr(a)))

    # -- stepping (mod.rs:229-233, 348-466) ------------------------------
    def iterate(self):
        check(self._lib.cg_iterate(self._h))

    def run_steps(self, n):
        check(self._lib.cg_step(self._h, int(n)))

    def iterate_on(self, stream):
        """iterate_with_encoder (mod.rs:435): enqueue on a caller stream."""
        check(self._lib.cg_iterate_on(self._h, ctypes.c_void_p(stream)))

    def set_params(self, mu, sigma, weights, temp=None):
        """Replace growth mu/sigma/weights (K each) and temp; takes effect for
        work enqueued afterwards."""
        t = self.temp if temp is None else float(temp)
        mu, sg, w = (np.ascontiguousarray(v, dtype=np.float32) for v in (mu, sigma, weights))
        check(self._lib.cg_set_params(self._h, fptr(mu), fptr(sg), fptr(w), ctypes.c_float(t)))
        self.temp = t

    def set_params_device(self, mu_ptr: int, sigma_ptr: int, weights_ptr: int):
        """The same from device arrays (K float32 each), folded on the device
        in stream order."""
        check(self._lib.cg_set_params_device(self._h, ctypes.c_void_p(mu_ptr),
                                             ctypes.c_void_p(sigma_ptr),
                                             ctypes.c_void_p(weights_ptr)))

    def build_ring_kernels(self, specs, ring_weights_ptr: int | None = None):
        """On-GPU kernel builder: specs is a list of K (family, rings, radius,
        width) tuples (family 0: Lenia shells, 1: the reference generator's
        Gaussian ring); ring_weights_ptr a device address of K * 8 float32
        ring weights, or None for all ones."""
        arr = ring_spec_array(specs)
        check(self._lib.cg_build_ring_kernels(self._h, ctypes.cast(arr, ctypes.c_void_p),
                                              ctypes.c_void_p(ring_weights_ptr or 0)))
        self._ring_specs = arr

    def ring_weight_grad(self, hbar_ptr: int, grad_ptr: int, ring_weights_ptr: int | None = None):
        """dL/d ring weights (K * 8 float32 at grad_ptr) of the last build,
        from dL/dh (K * n * n float32 at hbar_ptr)."""
        check(self._lib.cg_ring_weight_grad(self._h, ctypes.cast(self._ring_specs, ctypes.c_void_p),
                                            ctypes.c_void_p(ring_weights_ptr or 0),
                                            ctypes.c_void_p(hbar_ptr), ctypes.c_void_p(grad_ptr)))

    def iterate_and_render(self):
        """iterate_and_render (mod.rs:390): one step whose diffusion also
        writes the packed 0x00RRGGBB render buffer."""
        check(self._lib.cg_iterate_and_render(self._h))

    def render(self):
        """RenderPhase::run (render.rs:143): render the current state."""
        check(self._lib.cg_render(self._h))

    def download_render(self):
        """download_render (mod.rs:302): RGB24 bytes, shape (n, n, 3)."""
        out = np.empty(self.total_elements * 3, dtype=np.uint8)
        check(self._lib.cg_download_render(
            self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out.reshape(self.n, self.n, 3)

    def download_render_packed(self):
        """The packed render words, shape (n, n) uint32."""
        out = np.empty(self.total_elements, dtype=np.uint32)
        check(self._lib.cg_download_render_packed(self._h, uptr(out)))
        return out.reshape(self.n, self.n)

    def stream_frames(self, fd: int, nframes: int, steps_per_frame: int = 1):
        """Write nframes RGB24 frames (each after steps_per_frame steps) to the
        file descriptor fd, computing each frame while the previous one is
        written (main.rs:239-303's loop, to a file or a pipe)."""
        check(self._lib.cg_stream_frames(self._h, int(fd), int(nframes), int(steps_per_frame)))

    def step_host_async(self, host_in, host_out, nsteps: int = 1):
        """Upload all channels from host_in (C*n*n float64), run nsteps steps
        and download the state into host_out (C*n*n float32), pipelined with
        the calls before and after it; returns at once.  Both arrays must be
        page-locked (e.g. numpy views of torch pin_memory tensors) and stay
        untouched until host_wait()."""
        for a, dt in ((host_in, np.float64), (host_out, np.float32)):
            if a.dtype != dt or a.size != self.num_channels * self.total_elements \
                    or not a.flags["C_CONTIGUOUS"]:
                raise ValueError(f"expected a contiguous {np.dtype(dt).name} array of "
                                 f"{self.num_channels * self.total_elements} values")
        check(self._lib.cg_step_host_async(self._h, dptr(host_in), fptr(host_out), int(nsteps)))

    def host_wait(self):
        """Wait for every step_host_async enqueued so far."""
        check(self._lib.cg_host_wait(self._h))

    def check_bounded_wait(self, timeout_ms: int = 20):
        """Run the failure-path check: a kernel whose device-side wait can
        never complete gives up after timeout_ms and records the timeout.
        Raises CellaError(CG_ERR_TIMEOUT), as a step whose copy never landed
        would; the world is untouched and stays usable."""
        check(self._lib.cg_check_bounded_wait(self._h, int(timeout_ms)))

    def render_ptr(self) -> int:
        """Device address of the render buffer (n*n uint32)."""
        p = ctypes.c_void_p()
        check(self._lib.cg_render_ptr(self._h, ctypes.byref(p)))
        return p.value

    def timed_iterate(self):
        """[conv, growth, diffusion, copy] device ms for one step (mod.rs:469)."""
        ms = np.zeros(4, dtype=np.float64)
        check(self._lib.cg_timed_iterate(self._h, dptr(ms)))
        return ms

    def profile_kernels(self, nsteps):
        """Average device ms per kernel over nsteps steps: [row FFT, column
        convolution, inverse row FFT + growth, diffusion]."""
        ms = np.zeros(4, dtype=np.float64)
        check(self._lib.cg_profile_kernels(self._h, int(nsteps), dptr(ms)))
        return ms

    def autotune(self, reps=10):
        """Time every variant of every phase (CTA shapes and FFT plans), keep
        the fastest.  Returns (chosen[4], ms[4][5]); ms is -1 where a phase
        lacks a variant at this grid side."""
        ms = np.zeros(4 * _abi.MAX_VARIANTS, dtype=np.float64)
        ch = (ctypes.c_int * 4)()
        check(self._lib.cg_autotune(self._h, int(reps), dptr(ms), ch))
        return list(ch), ms.reshape(4, _abi.MAX_VARIANTS)

    def set_variants(self, v):
        arr = (ctypes.c_int * 4)(*[int(x) for x in v])
        check(self._lib.cg_set_variants(self._h, arr))

    def set_graph_layout(self, layout: int):
        """0: each channel on a forked stream; 1: one launch per phase over
        all channels (cg_set_graph_layout)."""
        check(self._lib.cg_set_graph_layout(self._h, int(layout)))

    def graph_layout(self) -> int:
        v = ctypes.c_int()
        check(self._lib.cg_get_graph_layout(self._h, ctypes.byref(v)))
        return v.value

    def kernels_real(self) -> bool:
        """Whether the column pass uses the real form of the kernel spectra
        (every kernel point-symmetric; see cg_set_kernel)."""
        v = ctypes.c_int()
        check(self._lib.cg_kernels_real(self._h, ctypes.byref(v)))
        return bool(v.value)

    def variants(self):
        arr = (ctypes.c_int * 4)()
        check(self._lib.cg_get_variants(self._h, arr))
        return list(arr)

    def synchronize(self):
        check(self._lib.cg_synchronize(self._h))

    # -- downloads (mod.rs:236-299) --------------------------------------
    def download_all_channels(self):
        out = np.empty(self.num_channels * self.total_elements, dtype=np.float32)
        check(self._lib.cg_download_channels(self._h, fptr(out)))
        return out

    def download_conv_buffer(self):
        """Real part of every kernel's convolution before the 1/n^2 scale."""
        out = np.empty(self.num_kernels * self.total_elements, dtype=np.float32)
        check(self._lib.cg_download_conv_real(self._h, fptr(out)))
        return out

    def download_affinity(self):
        out = np.empty(self.num_channels * self.total_elements, dtype=np.float32)
        check(self._lib.cg_download_affinity(self._h, fptr(out)))
        return out

    def mass_f64(self):
        out = np.zeros(self.num_channels, dtype=np.float64)
        check(self._lib.cg_mass_f64(self._h, dptr(out)))
        return out

    def channel_ptr(self) -> int:
        """Device address of the current state (channel_buffer, mod.rs:202)."""
        p = ctypes.c_void_p()
        check(self._lib.cg_channel_ptr(self._h, ctypes.byref(p)))
        return p.value

    def stream(self) -> int:
        p = ctypes.c_void_p()
        check(self._lib.cg_stream(self._h, ctypes.byref(p)))
        return p.value or 0

    # -- convenience -----------------------------------------------------
    def upload_state(self, state):
        state = np.asarray(state)
        for c in range(self.num_channels):
            if state.dtype == np.float32:
                self.upload_channel_f32(state[c], c)
            else:
                self.upload_channel(state[c], c)

    def state(self):
        return self.download_all_channels().reshape(self.num_channels, self.n, self.n)

    @classmethod
    def from_creature(cls, cr, stream=None):
        sim = cls((cr.n, cr.n), cr.C, cr.K, cr.c0, cr.c1, cr.mu, cr.sigma, cr.weights,
                  cr.temp, stream=stream)
        for k in range(cr.K):
            sim.set_kernel(cr.kspec[k], k)
        sim.upload_state(cr.seed)
        return sim


# ---------------------------------------------------------------------------
# File formats (ml-rs/config.rs) through the C ABI
# ---------------------------------------------------------------------------

def ring_spec_array(specs):
    """A ctypes array of cg_ring_spec from (family, rings, radius, width)."""
    arr = (_abi.cg_ring_spec * len(specs))()
    for i, (fam, rings, radius, width) in enumerate(specs):
        arr[i] = _abi.cg_ring_spec(int(fam), int(rings), float(radius), float(width))
    return arr


def creature_ring_specs(cr):
    """Shell-family specs and padded ring weights (K, 8) of a creature made
    by :func:`cella_nova_gb300.creature.make_creature`."""
    specs = [(_abi.RING_SHELL, len(b), R, 0.0) for R, b in zip(cr.ring_radius, cr.ring_weights)]
    w = np.zeros((cr.K, _abi.MAX_RINGS), dtype=np.float32)
    for k, b in enumerate(cr.ring_weights):
        w[k, :len(b)] = b
    return specs, w


SEED_MAGIC = b"CNSEED01"


def is_seed_bin(path) -> bool:
    try:
        with open(path, "rb") as f:
            return f.read(8) == SEED_MAGIC
    except OSError:
        return False   # the JSON loader reports the unreadable file


def load_config(path):
    """load_config (config.rs:32-47) -> dict in orchestrator order (c0 = input).
    Reads seed/{name}.json or its binary twin (magic CNSEED01)."""
    lib = _abi.load()
    cfg = _abi.cg_config()
    loader = lib.cg_load_config_bin if is_seed_bin(path) else lib.cg_load_config_json
    check(loader(str(path).encode(), ctypes.byref(cfg)))
    try:
        n, C, K = cfg.seed_size, cfg.num_channels, cfg.num_kernels
        seed = np.ctypeslib.as_array(cfg.seed_channels, shape=(C * n * n,)).copy()
        out = {
            "seed_size": n, "num_channels": C, "num_kernels": K,
            "seed_channels": seed.reshape(C, n * n),
            "c0": np.ctypeslib.as_array(cfg.c0, shape=(K,)).copy(),
            "c1": np.ctypeslib.as_array(cfg.c1, shape=(K,)).copy(),
            "growth_mu": np.ctypeslib.as_array(cfg.growth_mu, shape=(K,)).copy(),
            "growth_sigma": np.ctypeslib.as_array(cfg.growth_sigma, shape=(K,)).copy(),
            "growth_weights": np.ctypeslib.as_array(cfg.growth_weights, shape=(K,)).copy(),
            "temp": float(cfg.temp),
        }
    finally:
        lib.cg_free_config(ctypes.byref(cfg))
    return out


def save_config_bin(path, cfg):
    """Write a config dict (orchestrator order, as load_config returns it) as
    a binary seed file."""
    lib = _abi.load()
    K, C, n = int(cfg["num_kernels"]), int(cfg["num_channels"]), int(cfg["seed_size"])
    seed = np.ascontiguousarray(cfg["seed_channels"], dtype=np.float64).reshape(C * n * n)
    arrs = {k: np.ascontiguousarray(cfg[k], dtype=np.uint32) for k in ("c0", "c1")}
    arrs.update({k: np.ascontiguousarray(cfg[k], dtype=np.float32)
                 for k in ("growth_mu", "growth_sigma", "growth_weights")})
    c = _abi.cg_config(n, C, K, dptr(seed), uptr(arrs["c0"]), uptr(arrs["c1"]),
                       fptr(arrs["growth_mu"]), fptr(arrs["growth_sigma"]),
                       fptr(arrs["growth_weights"]), float(cfg.get("temp", 1.0)))
    check(lib.cg_save_config_bin(str(path).encode(), ctypes.byref(c)))


def load_kernels(path, num_kernels, target_size):
    """load_kernels (config.rs:56-125) -> (K, n, n) complex64."""
    lib = _abi.load()
    out = np.empty((num_kernels, target_size, target_size, 2), dtype=np.float32)
    check(lib.cg_load_kernels_bin(str(path).encode(), int(num_kernels), int(target_size),
                                  fptr(out)))
    return out[..., 0] + 1j * out[..., 1]


def setup_simulation(config_path, kernels_path, temp=None, stream=None):
    """main.rs:88-140 / profile.rs:32-89: config + kernels -> ready world."""
    cfg = load_config(config_path)
    n = cfg["seed_size"]
    sim = GpuMaceLenia((n, n), cfg["num_channels"], cfg["num_kernels"], cfg["c0"], cfg["c1"],
                       cfg["growth_mu"], cfg["growth_sigma"], cfg["growth_weights"],
                       cfg["temp"] if temp is None else temp, stream=stream)
    for c in range(cfg["num_channels"]):
        sim.upload_channel(cfg["seed_channels"][c], c)
    ks = load_kernels(kernels_path, cfg["num_kernels"], n)
    for k in range(cfg["num_kernels"]):
        sim.set_kernel(ks[k], k)
    return sim


class GpuMaceLeniaBatch:
    """Many worlds of uneven grid side, channel and kernel count, stepped
    together: each phase is one persistent launch over every world's work and
    each step one CUDA graph.  World w behaves exactly like a
    :class:`GpuMaceLenia` built from the same parameters."""

    def __init__(self, creatures, stream=None):
        self._lib = _abi.load()
        self.creatures = list(creatures)
        nw = len(self.creatures)
        n = np.array([cr.n for cr in self.creatures], dtype=np.int32)
        C = np.array([cr.C for cr in self.creatures], dtype=np.int32)
        K = np.array([cr.K for cr in self.creatures], dtype=np.int32)
        cat = lambda name, dt: np.ascontiguousarray(
            np.concatenate([np.asarray(getattr(cr, name), dtype=dt) for cr in self.creatures]))
        c0, c1 = cat("c0", np.uint32), cat("c1", np.uint32)
        mu, sg, w = cat("mu", np.float32), cat("sigma", np.float32), cat("weights", np.float32)
        temp = np.array([cr.temp for cr in self.creatures], dtype=np.float32)
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        h = ctypes.c_void_p()
        check(self._lib.cg_batch_create(nw, ip(n), ip(C), ip(K), uptr(c0), uptr(c1), fptr(mu),
                                        fptr(sg), fptr(w), fptr(temp),
                                        ctypes.c_void_p(stream) if stream else None,
                                        ctypes.byref(h)))
        self._h = h
        for i, cr in enumerate(self.creatures):
            for k in range(cr.K):
                self.set_kernel(i, k, cr.kspec[k])
            for c in range(cr.C):
                a = np.ascontiguousarray(cr.seed[c], dtype=np.float64)
                check(self._lib.cg_batch_upload_channel(self._h, i, c, dptr(a)))

    def close(self):
        if getattr(self, "_h", None):
            check(self._lib.cg_batch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_kernel(self, world, k, spec):
        a = np.asarray(spec).reshape(-1)
        inter = np.empty((a.size, 2), dtype=np.float32)
        inter[:, 0] = a.real
        inter[:, 1] = a.imag
        check(self._lib.cg_batch_set_kernel(self._h, int(world), int(k), fptr(inter)))

    def run_steps(self, n):
        check(self._lib.cg_batch_step(self._h, int(n)))

    def synchronize(self):
        check(self._lib.cg_batch_synchronize(self._h))

    def state(self, world):
        cr = self.creatures[world]
        out = np.empty(cr.C * cr.n * cr.n, dtype=np.float32)
        check(self._lib.cg_batch_download_channels(self._h, int(world), fptr(out)))
        return out.reshape(cr.C, cr.n, cr.n)

    def mass_f64(self, world):
        out = np.zeros(self.creatures[world].C, dtype=np.float64)
        check(self._lib.cg_batch_mass_f64(self._h, int(world), dptr(out)))
        return out

    def profile(self, nsteps):
        """Average device ms per phase [row FFT, column conv, row inverse +
        growth, diffusion] over nsteps steps."""
        ms = np.zeros(4, dtype=np.float64)
        check(self._lib.cg_batch_profile(self._h, int(nsteps), dptr(ms)))
        return ms

    def stream(self) -> int:
        p = ctypes.c_void_p()
        check(self._lib.cg_batch_stream(self._h, ctypes.byref(p)))
        return p.value or 0

    def info(self):
        items = (ctypes.c_int * 4)()
        grid = (ctypes.c_int * 4)()
        check(self._lib.cg_batch_info(self._h, items, grid))
        return list(items), list(grid)

    def set_variants(self, n, v):
        """Variants [row FFT, column, inverse row + growth, diffusion] of the
        worlds of grid side n."""
        arr = (ctypes.c_int * 4)(*[int(x) for x in v])
        check(self._lib.cg_batch_set_variants(self._h, int(n), arr))

    def set_mode(self, n, mode):
        """Step the worlds of grid side n with one persistent launch per phase
        (0) or as parallel branches of single-world step kernels (1)."""
        check(self._lib.cg_batch_set_mode(self._h, int(n), int(mode)))

    def mode(self, n) -> int:
        v = ctypes.c_int()
        check(self._lib.cg_batch_get_mode(self._h, int(n), ctypes.byref(v)))
        return v.value

    def autotune(self, reps=5):
        """Per grid side present: time every variant of every phase and keep
        the fastest.  Returns {side: (chosen[4], ms[4][5])}, ms -1 where a
        phase lacks a variant at that side."""
        V = _abi.MAX_VARIANTS
        chosen = (ctypes.c_int * 24)()
        ms = np.zeros(24 * V, dtype=np.float64)
        check(self._lib.cg_batch_autotune(self._h, int(reps), chosen, dptr(ms)))
        out = {}
        for i in range(6):
            if chosen[4 * i] >= 0:
                out[64 << i] = (list(chosen[4 * i:4 * i + 4]),
                                ms[4 * V * i:4 * V * (i + 1)].reshape(4, V))
        return out
