/*
 * cella_gpu.h — C ABI of the GB300 (sm_103a) DiffusionLenia step.
 *
 * Drop-in for the `GpuMaceLenia` orchestrator of anima-zetta/cella-nova
 * (ml-rs/orchestrator/mod.rs:45-541) and its file loaders (ml-rs/config.rs).
 * Every entry point takes plain pointers and sizes; none takes a torch or
 * wgpu type, so a Rust host binds it with plain `extern "C"` declarations in
 * place of the wgpu path.
 *
 * Conventions
 *   - Every function returns CG_OK (0) or a negative cg_status.  The reason
 *     for the last failure on the calling thread is cg_last_error().  The
 *     reference panics instead (mod.rs:34, :94, :208, :218; config.rs:33-34).
 *   - c0[k] is the channel kernel k reads, c1[k] the channel its growth term
 *     feeds: the orchestrator's order (mod.rs:52-54), i.e. AFTER the swap
 *     config.rs:40 applies to the JSON fields.  cg_load_config_json applies
 *     that swap.
 *   - The library owns its device buffers; callers own their host arrays,
 *     which are copied.  A handle is not thread-safe; distinct handles are.
 *   - Work is enqueued on the handle's CUDA stream (its own, or the one given
 *     to cg_create) and is asynchronous, like wgpu's queue.submit (mod.rs:385);
 *     downloads block, like map_async + poll(Wait) (mod.rs:255-257).
 *   - Grid sides are powers of two from 16 to 2048 (the reference accepts
 *     only 1024 and 2048, mod.rs:30-39); C <= 16 (compute_1024.wgsl:307);
 *     K <= 64.
 */
#ifndef CELLA_GPU_H
#define CELLA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CG_OK = 0,
    CG_ERR_ARG = -1,         /* bad argument (sizes, indices, NaN parameter) */
    CG_ERR_OOM = -2,         /* device or host allocation failed */
    CG_ERR_CUDA = -3,        /* a CUDA runtime call failed */
    CG_ERR_TIMEOUT = -4,     /* a bounded device wait gave up */
    CG_ERR_IO = -5,          /* file could not be read or written */
    CG_ERR_FORMAT = -6,      /* file contents do not match the format */
    CG_ERR_UNSUPPORTED = -7  /* valid request this library does not serve */
} cg_status;

typedef struct cg_sim cg_sim;
/* A cudaStream_t.  NULL = the library creates its own (non-blocking)
 * stream; to run on the legacy default stream pass cudaStreamLegacy
 * ((cg_stream_t)1). */
typedef void* cg_stream_t;

/* Message of the last failure on this thread ("" if none). */
const char* cg_last_error(void);

/* Library version string. */
const char* cg_version(void);

/* ---------------------------------------------------------------------------
 * Orchestrator (ml-rs/orchestrator/mod.rs)
 * ------------------------------------------------------------------------- */

/* GpuMaceLenia::new, mod.rs:79-198.  n: grid side; C channels; K kernels;
 * c0/c1/mu/sigma/weights: K entries each; temp multiplies the growth sum
 * inside exp (diffusion.rs:58-66).  Kernels start at zero and channels at
 * zero until set_kernel / upload_channel.  stream may be NULL. */
int cg_create(int n, int C, int K, const uint32_t* c0, const uint32_t* c1,
              const float* mu, const float* sigma, const float* weights,
              float temp, cg_stream_t stream, cg_sim** out);

/* Drop for GpuMaceLenia: frees every device buffer of the handle. */
int cg_destroy(cg_sim* sim);

/* GpuMaceLenia::set_kernel, mod.rs:207-214: kernel k's full n*n complex
 * spectrum, interleaved (re, im) f32, row-major, origin at [0,0].
 * The step only uses the spectrum's Hermitian part (the state is real and
 * growth reads the real part of each convolution).  When that part is real
 * to rounding for every kernel (point-symmetric kernels, h(x) = h(-x), as
 * every radially symmetric Lenia ring is), the column pass reads only the
 * real parts, half the bytes; the results agree with the complex form to
 * rounding.  cg_kernels_real reports which form is in use (1 real, 0
 * complex); spectra from cg_set_kernel_device or cg_build_ring_kernels
 * keep the complex form. */
int cg_set_kernel(cg_sim* sim, int k, const float* spec_interleaved);
int cg_kernels_real(cg_sim* sim, int* real);

/* set_kernel from DEVICE memory: kernel k's full n*n complex spectrum,
 * interleaved (re, im) f32, already on the GPU (no host round trip); the
 * buffer must be 16-byte aligned (CG_ERR_ARG otherwise). */
int cg_set_kernel_device(cg_sim* sim, int k, const float* dev_spec_interleaved);

/* All K kernels from their SPATIAL form: dev_h holds K*n*n f32 (kernel k's
 * n x n values, origin at [0][0], as the .bin spectra's inverse FFT), in
 * device memory.  The spectra are taken on the GPU with the step's own row
 * and column FFTs (no normaliser: the kernels as given) and stored as
 * cg_set_kernel would store their fft2; the column pass keeps the complex
 * form.  Uses the handle's spectrum scratch: enqueue it between steps. */
int cg_set_kernels_spatial_device(cg_sim* sim, const float* dev_h);

/* GpuMaceLenia::upload_channel, mod.rs:217-226: channel c from n*n doubles,
 * rounded to f32 (mod.rs:220 casts with `as f32`, round-to-nearest). */
int cg_upload_channel(cg_sim* sim, int c, const double* data);

/* Same as cg_upload_channel from f32 host data (no reference counterpart;
 * used to re-upload a state that was downloaded). */
int cg_upload_channel_f32(cg_sim* sim, int c, const float* data);

/* GpuMaceLenia::iterate, mod.rs:348-386: one step, enqueued. */
int cg_iterate(cg_sim* sim);

/* GpuMaceLenia::run_steps, mod.rs:229-233: nsteps steps, enqueued as CUDA
 * graph launches. */
int cg_step(cg_sim* sim, int nsteps);

/* GpuMaceLenia::iterate_with_encoder, mod.rs:435-466: one step enqueued on
 * the caller's stream instead of the handle's. */
int cg_iterate_on(cg_sim* sim, cg_stream_t stream);

/* GpuMaceLenia::iterate_and_render, mod.rs:390-431: one step, then the render
 * kernel on the new state, in one graph launch (render_main,
 * compute_1024.wgsl:428-443): per pixel the packed word 0x00RRGGBB with R, G,
 * B = u32(sqrt(clamp(1.5 c, 0, 1)) * 255) of channels 0, 1, 2 (0 for channels
 * the world lacks).  Enqueued. */
int cg_iterate_and_render(cg_sim* sim);

/* RenderPhase::run, render.rs:143-153: render the current state without
 * stepping.  Enqueued. */
int cg_render(cg_sim* sim);

/* GpuMaceLenia::download_render, mod.rs:302-335: blocking copy of the render
 * buffer as RGB24 bytes (3*n*n, row-major, R first).  The buffer holds zeros
 * until the first render. */
int cg_download_render(cg_sim* sim, uint8_t* rgb24);

/* Frame streaming (the video loop of main.rs:239-303 without ffmpeg): nframes
 * frames, each steps_per_frame steps of which the last renders, written as
 * RGB24 (3*n*n bytes per frame, the bytes main.rs pipes to ffmpeg) to the
 * file descriptor fd (a file, or the write end of a pipe to an encoder).
 * Each frame is computed and copied while the previous one is written.
 * Blocking; CG_ERR_IO if a write fails. */
int cg_stream_frames(cg_sim* sim, int fd, int nframes, int steps_per_frame);

/* Host buffers in, host buffers out, pipelined: enqueue the upload of `in`
 * (C*n*n f64, what cg_upload_channel takes, all channels), nsteps steps and
 * the download of the resulting state to `out` (C*n*n f32, as
 * cg_download_channels gives it), and return without waiting.  Uploads run
 * on a copy stream into one of two staging buffers, so the upload of the next
 * call overlaps this call's steps and download; the link carries both
 * directions at once.  Replaces a loop of upload_channel / run_steps /
 * download_all_channels (ml-rs/orchestrator/mod.rs:217-263) where the host
 * feeds many inputs.  `in` and `out` must be page-locked (cudaHostAlloc or
 * cudaHostRegister; CG_ERR_ARG otherwise) and stay untouched until
 * cg_host_wait.  Later calls on the handle are ordered after the download. */
int cg_step_host_async(cg_sim* sim, const double* in, float* out, int nsteps);
/* Wait for every cg_step_host_async enqueued so far (and the handle's
 * stream); reports a device-side timeout like the other synchronising calls. */
int cg_host_wait(cg_sim* sim);

/* Failure-path check: runs a kernel whose bounded device-side wait can never
 * complete (an mbarrier nothing arrives on), through the same wait the step
 * kernels use but limited to timeout_ms (1..2000).  The kernel gives up and
 * records the timeout, and this call returns CG_ERR_TIMEOUT exactly as a step
 * whose copy never landed would; the handle stays usable.  Blocking. */
int cg_check_bounded_wait(cg_sim* sim, int timeout_ms);

/* The packed render words themselves (n*n uint32_t), blocking. */
int cg_download_render_packed(cg_sim* sim, uint32_t* out);

/* Device address of the render buffer (n*n uint32_t, owned by the handle),
 * for a consumer on the GPU; valid until cg_destroy. */
int cg_render_ptr(cg_sim* sim, const uint32_t** dev_ptr);

/* GpuMaceLenia::download_all_channels, mod.rs:236-263: blocking copy of the
 * C*n*n f32 state, channel-major. */
int cg_download_channels(cg_sim* sim, float* out);

/* GpuMaceLenia::download_conv_buffer, mod.rs:267-299 (debug): K*n*n f32, the
 * real part of each kernel's convolution before the 1/n^2 scale
 * (growth.rs:87), for the CURRENT state (it runs the convolution again and
 * does not advance the state). */
int cg_download_conv_real(cg_sim* sim, float* out);

/* Affinity A = exp(temp * sum_k w_k G(u_k)) of the current state, C*n*n f32
 * (the reference keeps the pre-exp sum in ml::affinity, mod.rs:112; this
 * build stores the exponential, which is what diffusion reads). */
int cg_download_affinity(cg_sim* sim, float* out);

/* GpuMaceLenia::timed_iterate, mod.rs:469-540: one step with per-phase
 * device times in ms: [0] convolution, [1] growth, [2] diffusion, [3] buffer
 * copy (always 0: the state is ping-ponged, no copy exists). */
int cg_timed_iterate(cg_sim* sim, double ms[4]);

/* Autotuner (no reference counterpart; the reference fixes one register
 * stage split per grid size, ml-rs/shaders/compute_1024.wgsl:55-78 against
 * compute_2048.wgsl:57-84).  Each phase has up to CG_MAX_VARIANTS variants:
 *   0-2  CTA shapes (rows per CTA and threads for the row FFTs, columns per
 *        CTA and threads for the column pass, tile rows and columns per
 *        thread for diffusion), radix-16 plans; bit-identical results.
 *        The forward row FFT's variant 2 is variant 1's tile in a
 *        persistent grid whose CTAs bring each block of rows in with one
 *        bulk copy, the next block's during the current one's transform.
 *   3    for diffusion, at every grid side: variant 1's register tiles in
 *        strips of 8 rows instead of 16; bit-identical results.
 *   3, 4 FFT plans, for the row and column phases at grid sides >= 512:
 *        row FFTs over two real rows as one complex sequence of length n
 *        with radix-16 (3) or radix-8 (4) passes; the column pass with its
 *        forward and inverse plan orders swapped (remainder-first radix
 *        first forward) in the CTA shape of variant 1 (3) or 0 (4).  These
 *        agree with variants 0-2 to rounding (the same step error bar
 *        against FP64), not bit for bit.
 * Diffusion has variants 0-3; the other phases below side 512 have 0-2.
 * cg_autotune times every variant of every phase `reps` times on the live
 * handle (the state is not advanced), keeps the fastest per phase, then
 * picks the graph layout (cg_set_graph_layout) and re-captures the step
 * graphs.  ms_out[4 * CG_MAX_VARIANTS] (phase-major:
 * [row FFT v0..v4, column v0..v4, inverse row + growth v0..v4, diffusion
 * v0..v4], -1 where a variant does not exist) and chosen[4] may be NULL. */
#define CG_MAX_VARIANTS 5
int cg_autotune(cg_sim* sim, int reps, double ms_out[4 * CG_MAX_VARIANTS], int chosen[4]);
/* Set / read the variant of each phase ([row FFT, column, inverse row +
 * growth, diffusion]); a variant the phase lacks at this grid side is
 * CG_ERR_ARG.  Setting re-captures the graphs. */
int cg_set_variants(cg_sim* sim, const int v[4]);
/* Layout of the step graphs: 0, each channel's launches on a forked stream of
 * its own, so the channels' phases overlap; 1, one stream with one launch
 * per phase over all channels.  Both compute the same bits; after the
 * variants, cg_autotune times both (graphs of steps that all read the
 * current state, so the world does not advance) and keeps the faster.
 * Setting re-captures the graphs. */
int cg_set_graph_layout(cg_sim* sim, int layout);
int cg_get_graph_layout(cg_sim* sim, int* layout);
int cg_get_variants(cg_sim* sim, int v[4]);

/* Per-kernel device time, averaged over nsteps steps (1..1024) launched
 * one kernel at a time with CUDA events between them (no reference
 * counterpart; a finer split of timed_iterate, mod.rs:469-540).  Advances
 * the state by nsteps.  ms[0] row FFT, [1] column convolution, [2] inverse
 * row FFT + growth, [3] diffusion. */
int cg_profile_kernels(cg_sim* sim, int nsteps, double ms[4]);

/* Per-channel total mass of the current state, summed in FP64 on the GPU
 * (no reference counterpart: example.rs:547-553 sums in f32 on the CPU).
 * Blocking; out has C entries. */
int cg_mass_f64(cg_sim* sim, double* out);

/* Per-channel FP64 total mass of a C*n*n f32 state that the caller already
 * holds on the device, written to dev_out (C doubles, device memory).  It
 * allocates nothing: no cudaMalloc, cudaFree or allocating library call.  It
 * is for callers that cannot allocate device memory while they run, such as
 * code that works inside a memory budget another component has already
 * reserved, or a loop where cudaMalloc's implicit device-wide
 * synchronisation is not acceptable.  No counterpart in the reference.
 *   - C <= 16 (CG_ERR_ARG beyond): its scratch is a fixed 16 x 296-double
 *     array in device memory, held by every GPU that loads the library
 *     until the process exits.
 *   - The first call on a device looks up that array's device address with
 *     cudaGetSymbolAddress (the device must be current); make that first
 *     call before any stream capture.  The address is cached per device and
 *     per CUDA context: after cudaDeviceReset (or from another context) the
 *     next call looks it up again, so that call is again a first call.
 *   - Work is enqueued on `stream` (NULL = the legacy default stream) and
 *     dev_out is valid once that stream is synchronised.
 *   - All calls share the one array: calls that overlap on the GPU (other
 *     streams, other threads) race and give wrong sums; serialise them. */
int cg_mass_f64_noalloc(const float* dev_state, int n, int C, double* dev_out,
                        cg_stream_t stream);

/* GpuMaceLenia::channel_buffer, mod.rs:202-204: device pointer to the
 * current C*n*n f32 state (valid until the next step or destroy). */
int cg_channel_ptr(cg_sim* sim, float** dev_ptr);

/* The handle's stream (the one work is enqueued on). */
int cg_stream(cg_sim* sim, cg_stream_t* out);

/* Device-side synchronisation of the handle's stream. */
int cg_synchronize(cg_sim* sim);

/* ---------------------------------------------------------------------------
 * Differentiation (no counterpart in the Rust orchestrator; the reference
 * differentiates its PyTorch model, train/diff_lenia_org.py, with autograd).
 * Array arguments here are DEVICE pointers on the handle's device, except
 * those of cg_set_params; work is enqueued on the handle's stream.  The
 * state- and spectrum-sized ones (x, ybar, xbar, kgrad, hbar, x0, ckpt, xT,
 * gT, g0, seg, gtmp, x_in, x_out) must be 16-byte aligned, as every
 * cudaMalloc and PyTorch allocation is (CG_ERR_ARG otherwise): the kernels
 * read them with 16-byte vector loads and bulk copies.
 * ------------------------------------------------------------------------- */

/* Replace mu/sigma/weights (K each, HOST arrays) and temp.  Same checks as
 * cg_create.  The parameters reach the kernels through a device-resident
 * block, updated in stream order (work enqueued earlier keeps the old
 * values); only a change of temp re-captures the step graphs. */
int cg_set_params(cg_sim* sim, const float* mu, const float* sigma, const float* weights,
                  float temp);

/* The same from DEVICE arrays, folded on the device by one kernel enqueued on
 * the handle's stream (capturable in a CUDA graph, e.g. after an optimiser
 * step).  No checks: the values are used as given. */
int cg_set_params_device(cg_sim* sim, const float* dev_mu, const float* dev_sigma,
                         const float* dev_weights);

/* ---------------------------------------------------------------------------
 * On-GPU kernel builder (replaces generate_kernel_json.py:106-146 and
 * example.rs:338-407 on the host): K ring kernels built in device memory,
 * normalised to sum 1, transformed with the step's own row and column FFTs
 * and packed into the handle's kernel spectra (what cg_set_kernel would
 * store for their fft2).  Enqueued on the handle's stream; capturable.
 * ------------------------------------------------------------------------- */
#define CG_MAX_RINGS 8
enum {
    CG_RING_SHELL = 0, /* Lenia shells: r = |x| / radius, ring l = floor(r * rings),
                          t = frac(r * rings), b_l * exp(4 - 1/(t(1-t))) for r < 1 */
    CG_RING_GAUSS = 1  /* the reference generator's ring: d = |x| / radius,
                          sigmoid(-(d-1)*10) * exp(-(d-1/2)^2 / (2 width^2)),
                          radius = global_r * radius of generate_kernel_json.py */
};
typedef struct {
    int family;     /* CG_RING_SHELL or CG_RING_GAUSS */
    int rings;      /* CG_RING_SHELL: 1..CG_MAX_RINGS; ignored for CG_RING_GAUSS */
    float radius;   /* px, > 0 */
    float width;    /* CG_RING_GAUSS: > 0; ignored for CG_RING_SHELL */
} cg_ring_spec;

/* specs: K host descriptors.  dev_ring_weights: K * CG_MAX_RINGS device
 * floats (kernel k's ring weights b_l at k * CG_MAX_RINGS + l), or NULL for
 * all ones.  Uses the handle's spectrum scratch: enqueue it between steps. */
int cg_build_ring_kernels(cg_sim* sim, const cg_ring_spec* specs, const float* dev_ring_weights);

/* Gradient of a loss with respect to the ring weights of the LAST
 * cg_build_ring_kernels (same specs and weights), given dev_hbar = dL/dh
 * (K*n*n device floats, e.g. from cg_kernel_grad_spatial): writes
 * dev_grad[K * CG_MAX_RINGS] (0 past each kernel's ring count). */
int cg_ring_weight_grad(cg_sim* sim, const cg_ring_spec* specs, const float* dev_ring_weights,
                        const float* dev_hbar, float* dev_grad);

/* One step from x_in to x_out (C*n*n f32 each, distinct). */
int cg_step_from(cg_sim* sim, const float* x_in, float* x_out);

/* Vector-Jacobian product of one step at state x: given ybar = dL/dx_next,
 * writes xbar = dL/dx and ACCUMULATES pgrad[3K] (double: dL/dmu, dL/dsigma,
 * dL/dweights) and, if kgrad is not NULL, kgrad (K*(n/2)*n complex f32, the
 * packed kernel-gradient spectra; finish with cg_kernel_grad_spatial).
 * xbar must not alias x or ybar. */
int cg_step_backward(cg_sim* sim, const float* x, const float* ybar, float* xbar,
                     double* pgrad, float* kgrad);

/* hbar[K][n][n] = dL/dh_k for the spatial kernels h_k = Re IFFT(K_k), from
 * the accumulated kgrad (which this overwrites). */
int cg_kernel_grad_spatial(cg_sim* sim, float* kgrad, float* hbar);

/* Zero pgrad[3K] and, if not NULL, kgrad (K*(n/2)*n complex f32) on the
 * handle's stream, before a backward pass accumulates into them. */
int cg_zero_grads(cg_sim* sim, double* pgrad, float* kgrad);

/* T steps from x0 to xT, storing x_{j*every} in ckpt[j], j = 0..(T-1)/every
 * (ckpt holds (T-1)/every + 1 states). */
int cg_unroll(cg_sim* sim, const float* x0, int T, int every, float* ckpt, float* xT);

/* Gradients of an unroll stored by cg_unroll: from gT = dL/dx_T to
 * g0 = dL/dx_0, recomputing each segment of `every` states from its
 * checkpoint into seg (every*C*n*n f32); gtmp is one C*n*n scratch state.
 * pgrad / kgrad accumulate as in cg_step_backward. */
int cg_unroll_backward(cg_sim* sim, const float* ckpt, int T, int every, const float* gT,
                       float* g0, double* pgrad, float* kgrad, float* seg, float* gtmp);

/* ---------------------------------------------------------------------------
 * Batched worlds (no reference counterpart beyond the PyTorch model's batch
 * dimension, train/lenia_org.py:47; here worlds may differ in grid side,
 * channel and kernel count)
 * ------------------------------------------------------------------------- */

typedef struct cg_batch cg_batch;

/* n_worlds worlds; world w has grid side n[w] (64..2048), C[w] channels,
 * K[w] kernels and temp[w].  c0/c1/mu/sigma/weights hold the worlds'
 * per-kernel arrays back to back (world w starts at sum of K[0..w-1]).
 * Each step is one CUDA graph: a persistent launch per phase over the work
 * of every world. */
int cg_batch_create(int n_worlds, const int* n, const int* C, const int* K,
                    const uint32_t* c0, const uint32_t* c1, const float* mu,
                    const float* sigma, const float* weights, const float* temp,
                    cg_stream_t stream, cg_batch** out);
int cg_batch_destroy(cg_batch* b);
/* set_kernel / upload_channel of world `world` (mod.rs:207-226). */
int cg_batch_set_kernel(cg_batch* b, int world, int k, const float* spec_interleaved);
int cg_batch_upload_channel(cg_batch* b, int world, int c, const double* data);
/* nsteps steps of every world (run_steps, mod.rs:229). */
int cg_batch_step(cg_batch* b, int nsteps);
int cg_batch_download_channels(cg_batch* b, int world, float* out);
int cg_batch_mass_f64(cg_batch* b, int world, double* out);
int cg_batch_synchronize(cg_batch* b);
/* Average device ms per phase over nsteps steps (advances the state):
 * [0] row FFT, [1] column convolution, [2] inverse row FFT + growth,
 * [3] diffusion. */
int cg_batch_profile(cg_batch* b, int nsteps, double ms[4]);
/* The batch's stream. */
int cg_batch_stream(cg_batch* b, cg_stream_t* out);
/* Work items and persistent grid size per phase (either pointer may be
 * NULL). */
int cg_batch_info(cg_batch* b, int* items4, int* grid4);

/* Autotuner of the batch: per grid side present and per phase, times the
 * variants that phase has at that side (those of cg_autotune) on the live
 * batch without stepping it, keeps the fastest, then times a step of the
 * side in each mode (cg_batch_set_mode) and keeps the faster.  The sides run
 * concurrently in the step graph, so with two or three sides every
 * combination of their modes is then timed on the whole step and the
 * fastest kept.  Re-captures the step graphs.  chosen[6*4] and
 * ms[6*4*CG_MAX_VARIANTS] (either may be NULL) are indexed by grid side 64,
 * 128, ..., 2048, then phase, then variant; sides the batch lacks give -1,
 * variants a phase lacks give ms -1. */
int cg_batch_autotune(cg_batch* b, int reps, int* chosen, double* ms);
/* Set the variants of the batch's worlds of grid side n (as cg_set_variants
 * does for one world); re-captures the step graphs. */
int cg_batch_set_variants(cg_batch* b, int n, const int v[4]);
/* How the worlds of grid side n are stepped: mode 0, one persistent launch
 * per phase over all of them; mode 1, each world's own step kernels (those
 * of a single world, per channel) with the worlds as parallel branches of
 * the step graph.  Both give the same bits; cg_batch_autotune times both and
 * keeps the faster.  Setting re-captures the step graphs. */
int cg_batch_set_mode(cg_batch* b, int n, int mode);
int cg_batch_get_mode(cg_batch* b, int n, int* mode);

/* ---------------------------------------------------------------------------
 * Gradient-search helpers (the optimisation loop of train/, on the device).
 * Free functions on device arrays, enqueued on `stream` (NULL: the legacy
 * default stream); capturable in a CUDA graph.
 * ------------------------------------------------------------------------- */
#define CG_REDUCE_BLOCKS 296

/* loss = mean((x - target)^2) (FP64, fixed-order reduction; written to
 * dev_loss[0]) and grad = 2 (x - target) / count.  dev_scratch holds
 * CG_REDUCE_BLOCKS doubles. */
int cg_mse_grad(const float* dev_x, const float* dev_target, size_t count, float* dev_grad,
                double* dev_loss, double* dev_scratch, cg_stream_t stream);

/* One Adam step (torch.optim.Adam without weight decay or amsgrad) on count
 * parameters: m = lerp(m, g, 1-beta1), v = beta2 v + (1-beta2) g^2,
 * p -= lr / (1-beta1^t) * m / (sqrt(v) / sqrt(1-beta2^t) + eps) with
 * t = *dev_step + 1.  Exactly one of grad_f32 / grad_f64 is given (the
 * parameter gradients of cg_unroll_backward are FP64). */
int cg_adam_step(float* dev_param, const float* dev_grad_f32, const double* dev_grad_f64,
                 float* dev_m, float* dev_v, size_t count, float lr, float beta1, float beta2,
                 float eps, const int* dev_step, cg_stream_t stream);

/* *dev_step += 1 (after the Adam steps of one iteration). */
int cg_count_step(int* dev_step, cg_stream_t stream);

/* ---------------------------------------------------------------------------
 * File formats (ml-rs/config.rs)
 * ------------------------------------------------------------------------- */

/* Parsed seed/{name}.json (config.rs:14-25).  c0/c1 are in orchestrator
 * order: the loader swaps the JSON fields as config.rs:40 does. */
typedef struct {
    int seed_size, num_channels, num_kernels;
    double* seed_channels;   /* C * n * n, channel-major */
    uint32_t* c0;            /* K: input channel (JSON "c1") */
    uint32_t* c1;            /* K: output channel (JSON "c0") */
    float* growth_mu;        /* K */
    float* growth_sigma;     /* K */
    float* growth_weights;   /* K */
    float temp;              /* optional "temp" key; 1.0 when absent */
} cg_config;

/* load_config, config.rs:32-47. */
int cg_load_config_json(const char* path, cg_config* out);
void cg_free_config(cg_config* cfg);

/* Binary twin of seed/{name}.json (no reference counterpart; it replaces the
 * ~12.6 M numbers of JSON text a 2048^2 three-channel seed takes with raw
 * little-endian values).  The file holds exactly the JSON's fields,
 * c0/c1 in the JSON's order, so JSON -> binary -> cg_config gives the same
 * cg_config as the JSON itself:
 *   "CNSEED01", u32 n, u32 C, u32 K, f32 temp, u32 c0_json[K], u32 c1_json[K],
 *   f32 mu[K], f32 sigma[K], f32 weights[K], zero padding to 8 bytes,
 *   f64 seed[C][n][n]. */
int cg_load_config_bin(const char* path, cg_config* out);
/* Write cfg (orchestrator c0/c1 order, as the loaders return it). */
int cg_save_config_bin(const char* path, const cg_config* cfg);

/* load_kernels, config.rs:56-125: K spectra resampled to target_n (spectral
 * zero-padding when the file holds a smaller grid, config.rs:81-116).
 * out: K * target_n * target_n * 2 floats, caller-allocated.  A file holding
 * a LARGER grid than target_n is rejected (the reference underflows). */
int cg_load_kernels_bin(const char* path, int K, int target_n, float* out);

/* Size of the grid stored in a kernels .bin (config.rs:61-65). */
int cg_kernels_bin_size(const char* path, int K, int* src_n);

#ifdef __cplusplus
}
#endif
#endif /* CELLA_GPU_H */
