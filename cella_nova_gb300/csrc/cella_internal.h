// cella_internal.h — types shared by the host orchestrator and the kernels.
#pragma once
#include <cuda.h>   // CUtensorMap (the encoder is reached through the runtime)
#include <cuda_runtime.h>
#include <stdint.h>

namespace cg {

constexpr int kMaxC = 16;   // compute_1024.wgsl:307 holds at most 16 channels
constexpr int kMaxK = 64;
constexpr int kMinLogN = 4;
constexpr int kMaxLogN = 11;

// Kernels grouped by the channel they read (conv pass) and by the channel
// they feed (growth pass), each group in increasing k.
struct KernelGroups {
    int in_count[kMaxC], in_start[kMaxC];
    int out_count[kMaxC], out_start[kMaxC];
    int in_idx[kMaxK];    // kernels sorted by c0
    int out_idx[kMaxK];   // kernels sorted by c1
};

// Growth parameters per kernel (growth.rs:46-75), pre-scaled on the host:
// mu, c2 = -log2(e) / (2 sigma^2), w2 = 2 w; and per output channel the sum
// of its kernels' weights (in increasing k).
struct GrowthParams {
    float mu[kMaxK];
    float c2[kMaxK];
    float w2[kMaxK];
    float wsum[kMaxC];
};

// Variant of each phase (0 = default); the autotuner picks them.  Variants
// 0-2 are CTA shapes with the same bits; 3 and 4 (row and column phases,
// grid sides from 2^kMinPairLogN) change the FFT plans (step_kernels.cuh).
struct Variants {
    int r2c = 0, col = 0, c2r = 0, diff = 0;
};
constexpr int kMinPairLogN = 9;
constexpr int kMaxVariants = 5;
// Variants phase p (0 r2c, 1 col, 2 c2r, 3 diffusion) has at side 2^logn:
// diffusion four at every side, the FFT phases five from kMinPairLogN on
// (the plan variants) and three below.
__host__ __device__ constexpr int phase_variant_count(int logn, int phase) {
    return phase == 3 ? 4 : (logn < kMinPairLogN ? 3 : kMaxVariants);
}

// Everything one step's launches need.  Planar layouts, all device pointers:
//   x_in, x_out : [C][n][n] f32 state (ping-pong)
//   rowspec     : [C][n/2][n] complex — row spectra, transposed (kx-major)
//   kspec       : [K][n/2+1][n] complex — Hermitian part of each kernel
//                 spectrum scaled by 1/(2 n^2), kx-major; column 0 holds
//                 (K(.,0)+K(.,n/2))/2, column n/2 holds (K(.,0)-K(.,n/2))/2
//   U           : [K][n/2][n] complex — column-inverted products, kx-major
//   A           : [C][n][n] f32 — exp(temp * weighted growth)
//   tw          : W_n^m (m < n), then the per-pass FFT twiddle tables
struct StepArgs {
    int C, K;
    float temp;
    const float* x_in;
    float* x_out;
    float2* rowspec;
    const float2* kspec;
    // optional [K][n/2+1][n] f32: the real parts of kspec, set when every
    // kernel's Hermitian part is real (point-symmetric kernels); the column
    // pass then reads 4 instead of 8 bytes per spectrum value
    const float* kre;
    float2* U;
    float* A;
    const float2* tw;
    float* udbg;   // optional [K][n][n] f32: Re(conv) before the 1/n^2 scale
    int* err;      // device error word (bounded waits that timed out)
    unsigned char* levels;   // optional [3][n][n] render level bytes, written by the diffusion
    KernelGroups groups;
    const GrowthParams* gp;   // device-resident: updated without re-capturing graphs
    Variants var;
};

// Per-kernel constants of the backward pass.
struct AdjointParams {
    int cout[kMaxK];       // c1[k]: the channel kernel k's growth feeds
    float mu[kMaxK];
    float w[kMaxK];
    float inv_s2[kMaxK];   // 1 / sigma^2
    float inv_s3[kMaxK];   // 1 / sigma^3
};

// Everything one backward step's launches need (adjoint.cuh).  Buffers of
// the step (rowspec, U, A) are reused as scratch; x and ybar are read,
// xbar and abar written; pgrad[3K] (d/dmu, d/dsigma, d/dw) and, if given,
// kgrad[K][n/2][n] are accumulated.
struct BwdArgs {
    int C, K;
    float temp;
    const float* x;
    const float* ybar;
    float* xbar;
    float* abar;
    float2* rowspec;
    const float2* kspec;
    float2* U;
    float* A;
    const float2* tw;
    double* pgrad;
    float2* kgrad;
    int* err;
    const float* kre;         // as StepArgs::kre (the forward recompute's column pass)
    KernelGroups groups;
    const GrowthParams* gp;   // device-resident
    const AdjointParams* ap;  // device-resident
    // true: recompute the row spectra, U and A of x first; false: rowspec, U
    // and A already hold them (a cached forward step)
    bool recompute;
    Variants var;   // CTA shapes (the forward phases' tuned variants)
};

// Ring-kernel descriptors for the on-GPU kernel builder (kernels_common.cu).
constexpr int kMaxRings = 8;
constexpr int kRingBlocks = 64;   // blocks per kernel in the builder's sums
struct RingSet {
    int family[kMaxK];    // 0: Lenia shells exp(4 - 1/(t(1-t))), 1: sigmoid-gated Gaussian ring
    int rings[kMaxK];     // shells per kernel (family 0), 1 for family 1
    float radius[kMaxK];  // px: R (family 0), global_r * radius (family 1)
    float width[kMaxK];   // family 1: ring width (in units of radius)
};

// The per-world parameter block the kernels read from device memory.
struct DeviceParams {
    GrowthParams gp;
    AdjointParams ap;
};

// Phase bits for launch_step (timed_iterate splits the step into phases).
enum : int {
    kPhaseRowFwd = 1,
    kPhaseColConv = 2,
    kPhaseGrowth = 4,
    kPhaseDiffusion = 8,
    kPhaseAll = 15,
};

// Per grid size (LOGN = 6..11), defined in kernels_l*.cu.
typedef cudaError_t (*launch_step_fn)(const StepArgs&, int phases, cudaStream_t);
typedef cudaError_t (*pack_kernel_fn)(const float2* full, float2* out, cudaStream_t);
typedef cudaError_t (*prepare_fn)();
typedef int (*twiddle_count_fn)();
typedef cudaError_t (*launch_bwd_fn)(const BwdArgs&, cudaStream_t);
typedef cudaError_t (*launch_step_channel_fn)(const StepArgs&, int phases, int c, cudaStream_t);
typedef cudaError_t (*kspec_cols_fn)(const float2* rows, float2* kspec, const float2* tw,
                                      const double* zsum, int K, cudaStream_t);
typedef cudaError_t (*kgrad_final_fn)(float2* kgrad, float* hbar, int K, const float2* tw,
                                      cudaStream_t);

struct SizeOps {
    launch_step_fn step;
    pack_kernel_fn pack;
    prepare_fn prepare;
    twiddle_count_fn twiddle_count;   // float2 entries of the twiddle buffer
    launch_bwd_fn backward;
    kgrad_final_fn kgrad_final;
    prepare_fn prepare_backward;
    launch_step_channel_fn step_channel;   // phases of one channel
    prepare_fn prepare_builder;
    kspec_cols_fn kspec_cols;   // kernel builder: row spectra -> packed kernel spectra
};

// Fill the twiddle buffer of an n-point grid (host side, double precision).
void build_twiddle_tables(int n, float2* out);

// Status helpers shared by the C ABI translation units (host.cu).
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

// Argument checks of one world (cg_create / cg_batch_create); sets *logn.
int validate_world(int n, int C, int K, const uint32_t* c0, const uint32_t* c1, const float* mu,
                   const float* sigma, const float* weights, float temp, int* logn_out);

// Kernel groups and pre-scaled growth parameters from the per-kernel maps
// (host.cu); used by the single-world and the batched paths alike.
void build_groups(int C, int K, const uint32_t* c0, const uint32_t* c1, const float* mu,
                  const float* sigma, const float* weights, KernelGroups* g, GrowthParams* gp);

const SizeOps* size_ops(int logn);

// Size-independent kernels (kernels_common.cu).
cudaError_t launch_f64_to_f32(const double* in, float* out, size_t count, cudaStream_t s);
// out[i] = in[i].x (the real parts of packed kernel spectra)
cudaError_t launch_real_parts(const float2* in, float* out, size_t count, cudaStream_t s);
// Whether the Hermitian part of a full n x n spectrum (interleaved re, im)
// is real to rounding, i.e. the kernel is point-symmetric (host.cu).
bool hermitian_part_is_real(const float* spec, int n);
cudaError_t launch_mass_f64(const float* x, int C, size_t px, double* partial, int nblocks,
                            double* out, cudaStream_t s);
cudaError_t launch_render(const float* x, int C, size_t px, unsigned* out, cudaStream_t s);
cudaError_t launch_pack_levels(const unsigned char* levels, int C, size_t px, unsigned* out,
                               cudaStream_t s);
// Tensor map over U (K kernels x n/2 rows kx x n float2 y, kx-major) for the
// inverse row pass's 2-D tile loads: boxes of rb values of y by up to 256 kx.
cudaError_t encode_u_map(CUtensorMap* map, const float2* U, int n, int K, int rb);
cudaError_t launch_wait_check(int* err, int timeout_ms, cudaStream_t s);
cudaError_t launch_rgb24(const unsigned* in, unsigned char* out, size_t px, cudaStream_t s);
cudaError_t launch_fold_params(const float* mu, const float* sigma, const float* w, int C, int K,
                               const KernelGroups& g, DeviceParams* p, cudaStream_t s);
// Spatial ring kernels h[K][n][n] (unnormalised), their per-ring sums and
// zsum[k] = sum of h_k (FP64; partial: K * kRingBlocks * kMaxRings).
cudaError_t launch_ring_build(int n, int K, const RingSet& rs, const float* ring_w, float* h,
                              double* partial, double* ring_s, double* zsum, cudaStream_t s);
// d loss / d ring weight from hbar[K][n][n] = d loss / d h (normalised h).
cudaError_t launch_ring_grad(int n, int K, const RingSet& rs, const float* ring_w,
                             const float* hbar, double* partial, const double* ring_s,
                             const double* zsum, float* grad, cudaStream_t s);
constexpr int kMassBlocks = 296;   // 2 per SM on a 148/152-SM part

}  // namespace cg
