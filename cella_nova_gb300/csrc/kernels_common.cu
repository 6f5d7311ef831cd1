// Size-independent kernels: f64 -> f32 channel upload and the FP64 mass sum.
#include <mutex>
#include <unordered_map>

#include "async_copy.cuh"
#include "cella_gpu.h"
#include "cella_internal.h"
#include "render.cuh"

namespace cg {

// upload_channel (ml-rs/orchestrator/mod.rs:217-226) casts f64 to f32 with
// round-to-nearest; done here on the device after a raw f64 copy.
__global__ void k_f64_to_f32(const double* __restrict__ in, float* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}

__global__ void k_real_parts(const float2* __restrict__ in, float* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
        out[i] = in[i].x;
}

cudaError_t launch_real_parts(const float2* in, float* out, size_t count, cudaStream_t s) {
    const int blocks = int((count + 255) / 256 < 4096 ? (count + 255) / 256 : 4096);
    k_real_parts<<<blocks, 256, 0, s>>>(in, out, count);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double* in, float* out, size_t count, cudaStream_t s) {
    const int blocks = int((count + 255) / 256 < 4096 ? (count + 255) / 256 : 4096);
    k_f64_to_f32<<<blocks, 256, 0, s>>>(in, out, count);
    return cudaGetLastError();
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Per-channel partial sums in FP64: block b of channel c sums a fixed
// strided subset, so the result does not depend on scheduling.
// grid (nblocks, C), block 256.
__global__ void k_mass_partial(const float* __restrict__ x, size_t px,
                               double* __restrict__ partial) {
    const int c = blockIdx.y;
    const float* xc = x + size_t(c) * px;
    double s = 0.0;
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < px; i += stride)
        s += double(__ldg(&xc[i]));
    __shared__ double red[8];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        t = warp_sum(t);
        if (threadIdx.x == 0) partial[size_t(c) * gridDim.x + blockIdx.x] = t;
    }
}

// grid (C), block 256: fixed-order reduction of the partials.
__global__ void k_mass_final(const double* __restrict__ partial, int nblocks,
                             double* __restrict__ out) {
    const int c = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) s += partial[size_t(c) * nblocks + i];
    __shared__ double red[8];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        t = warp_sum(t);
        if (threadIdx.x == 0) out[c] = t;
    }
}

cudaError_t launch_mass_f64(const float* x, int C, size_t px, double* partial, int nblocks,
                            double* out, cudaStream_t s) {
    k_mass_partial<<<dim3(nblocks, C), 256, 0, s>>>(x, px, partial);
    k_mass_final<<<C, 256, 0, s>>>(partial, nblocks, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Render (RenderPhase::run, render.rs:143-153): one packed 0x00RRGGBB word
// per pixel from channels 0..2.  A thread takes four adjacent pixels: one
// 16-byte load per channel and one 16-byte store of the four words (the
// pixel count, n*n with n >= 16, is a multiple of four).
// ---------------------------------------------------------------------------
__global__ void k_render(const float* __restrict__ x, int C, size_t px,
                         unsigned* __restrict__ out) {
    const size_t q = px / 4;
    const float4* r4 = reinterpret_cast<const float4*>(x);
    const float4* g4 = reinterpret_cast<const float4*>(x + px);
    const float4* b4 = reinterpret_cast<const float4*>(x + 2 * px);
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < q;
         i += size_t(gridDim.x) * blockDim.x) {
        const float4 r = __ldg(&r4[i]);
        uint4 w = make_uint4(render_level(r.x) << 16, render_level(r.y) << 16,
                             render_level(r.z) << 16, render_level(r.w) << 16);
        if (C > 1) {
            const float4 g = __ldg(&g4[i]);
            w.x |= render_level(g.x) << 8;
            w.y |= render_level(g.y) << 8;
            w.z |= render_level(g.z) << 8;
            w.w |= render_level(g.w) << 8;
        }
        if (C > 2) {
            const float4 b = __ldg(&b4[i]);
            w.x |= render_level(b.x);
            w.y |= render_level(b.y);
            w.z |= render_level(b.z);
            w.w |= render_level(b.w);
        }
        reinterpret_cast<uint4*>(out)[i] = w;
    }
}

// The words from the level planes the diffusion kernels wrote in a rendering
// step: plane c (c < min(C, 3)) holds channel c's levels, one byte per pixel.
// Four pixels per thread: a 4-byte load per plane, one 16-byte store.
__global__ void k_pack_levels(const unsigned char* __restrict__ levels, int C, size_t px,
                              unsigned* __restrict__ out) {
    const size_t q = px / 4;
    const uchar4* r4 = reinterpret_cast<const uchar4*>(levels);
    const uchar4* g4 = reinterpret_cast<const uchar4*>(levels + px);
    const uchar4* b4 = reinterpret_cast<const uchar4*>(levels + 2 * px);
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < q;
         i += size_t(gridDim.x) * blockDim.x) {
        const uchar4 r = r4[i];
        uint4 w = make_uint4(unsigned(r.x) << 16, unsigned(r.y) << 16, unsigned(r.z) << 16,
                             unsigned(r.w) << 16);
        if (C > 1) {
            const uchar4 g = g4[i];
            w.x |= unsigned(g.x) << 8;
            w.y |= unsigned(g.y) << 8;
            w.z |= unsigned(g.z) << 8;
            w.w |= unsigned(g.w) << 8;
        }
        if (C > 2) {
            const uchar4 b = b4[i];
            w.x |= b.x;
            w.y |= b.y;
            w.z |= b.z;
            w.w |= b.w;
        }
        reinterpret_cast<uint4*>(out)[i] = w;
    }
}

// download_render's conversion (mod.rs:322-329): packed words -> RGB24 bytes.
// Four pixels per thread: one 16-byte load, their 12 bytes as three 4-byte
// stores (little-endian: R, G, B of pixel 0 first).
__global__ void k_rgb24(const unsigned* __restrict__ in, unsigned char* __restrict__ out,
                        size_t px) {
    const size_t q = px / 4;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < q;
         i += size_t(gridDim.x) * blockDim.x) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(in) + i);
        const unsigned b[12] = {v.x >> 16 & 255u, v.x >> 8 & 255u, v.x & 255u,
                                v.y >> 16 & 255u, v.y >> 8 & 255u, v.y & 255u,
                                v.z >> 16 & 255u, v.z >> 8 & 255u, v.z & 255u,
                                v.w >> 16 & 255u, v.w >> 8 & 255u, v.w & 255u};
        unsigned* o = reinterpret_cast<unsigned*>(out + 12 * i);
#pragma unroll
        for (int j = 0; j < 3; ++j)
            o[j] = b[4 * j] | b[4 * j + 1] << 8 | b[4 * j + 2] << 16 | b[4 * j + 3] << 24;
    }
}

int cuda_fail(cudaError_t e, const char* what);
static_assert(kMassBlocks == CG_REDUCE_BLOCKS, "reduction scratch size");

static int grid_for(size_t count) {
    return int((count + 255) / 256 < 4096 ? (count + 255) / 256 : 4096);
}

cudaError_t launch_render(const float* x, int C, size_t px, unsigned* out, cudaStream_t s) {
    k_render<<<grid_for(px / 4), 256, 0, s>>>(x, C, px, out);
    return cudaGetLastError();
}

cudaError_t launch_pack_levels(const unsigned char* levels, int C, size_t px, unsigned* out,
                               cudaStream_t s) {
    k_pack_levels<<<grid_for(px / 4), 256, 0, s>>>(levels, C, px, out);
    return cudaGetLastError();
}

cudaError_t launch_rgb24(const unsigned* in, unsigned char* out, size_t px, cudaStream_t s) {
    k_rgb24<<<grid_for(px / 4), 256, 0, s>>>(in, out, px);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The growth-parameter folding of build_groups / build_adjoint_params, on the
// device, so parameters produced on the device (an optimiser step) reach the
// kernels without a host round trip.  Same formulas and summation order as
// the host, hence the same bits.  c1 (AdjointParams::cout) is left as is.
// ---------------------------------------------------------------------------
__global__ void k_fold_params(const float* __restrict__ mu, const float* __restrict__ sigma,
                              const float* __restrict__ w, int C, int K,
                              const __grid_constant__ KernelGroups g,
                              DeviceParams* __restrict__ p) {
    const int t = threadIdx.x;
    if (t < K) {
        const float m = mu[t], wk = w[t];
        const double sg = double(sigma[t]);
        p->gp.mu[t] = m;
        p->gp.c2[t] = float(-1.4426950408889634 / (2.0 * sg * sg));
        p->gp.w2[t] = 2.0f * wk;
        p->ap.mu[t] = m;
        p->ap.w[t] = wk;
        p->ap.inv_s2[t] = float(1.0 / (sg * sg));
        p->ap.inv_s3[t] = float(1.0 / (sg * sg * sg));
    }
    if (t < C) {
        float ws = 0.f;
        for (int i = 0; i < g.out_count[t]; ++i) ws += w[g.out_idx[g.out_start[t] + i]];
        p->gp.wsum[t] = ws;
    }
}

cudaError_t launch_fold_params(const float* mu, const float* sigma, const float* w, int C, int K,
                               const KernelGroups& g, DeviceParams* p, cudaStream_t s) {
    k_fold_params<<<1, 64, 0, s>>>(mu, sigma, w, C, K, g, p);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// On-GPU ring-kernel builder, spatial part.  Pixel (y, x) of the origin-
// centred kernel sits at the wrapped offsets dy, dx in [-n/2, n/2) (the
// ifftshift of generate_kernel_json.py:137 / example.rs:403).  Family 0 is
// the Lenia shell kernel of the synthetic creatures: r = |d| / R, ring
// l = floor(r B), t = frac(r B), value b_l exp(4 - 1/(t(1-t))) for r < 1.
// Family 1 is the reference generator's Gaussian ring
// (generate_kernel_json.py:106-146, example.rs:338-407): d = |d| / radius,
// sigmoid(-(d-1) 10) exp(-(d-1/2)^2 / (2 w^2)), sigmoid(x) = (tanh(x/2)+1)/2.
// Values are unnormalised; the sums per ring (FP64, fixed order) give the
// normaliser, which the spectrum packing divides by.
// ---------------------------------------------------------------------------
struct RingValue {
    int ring;      // -1: zero
    float core;    // shell / Gaussian value before the ring weight
};

__device__ __forceinline__ RingValue ring_value(const RingSet& rs, int k, int n, size_t p) {
    const int y = int(p / size_t(n)), x = int(p % size_t(n)), h = n / 2;
    const float dy = float(((y + h) & (n - 1)) - h), dx = float(((x + h) & (n - 1)) - h);
    const float dist = sqrtf(dy * dy + dx * dx);
    RingValue v{-1, 0.f};
    if (rs.family[k] == 0) {
        const float r = dist / rs.radius[k];
        const float rb = r * float(rs.rings[k]);
        const float fl = floorf(rb);
        const float t = rb - fl;
        if (r < 1.f && t > 0.f && t < 1.f) {
            v.ring = int(fl);
            v.core = expf(4.f - 1.f / (t * (1.f - t)));
        }
    } else {
        const float d = dist / rs.radius[k];
        const float sig = 0.5f * tanhf(-(d - 1.f) * 10.f * 0.5f) + 0.5f;
        const float df = d - 0.5f, w = rs.width[k];
        v.ring = 0;
        v.core = sig * expf(-(df * df) / (2.f * w * w));
    }
    return v;
}

// Per block: acc[l] summed over the block's threads, written to
// partial[(k * gridDim.x + block) * kMaxRings + l].
__device__ void block_sums(double (&acc)[kMaxRings], double* __restrict__ partial, int k) {
    __shared__ double red[8][kMaxRings];
#pragma unroll
    for (int l = 0; l < kMaxRings; ++l) {
        double v = warp_sum(acc[l]);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][l] = v;
    }
    __syncthreads();
    if (threadIdx.x < kMaxRings) {
        double s = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
        partial[(size_t(k) * gridDim.x + blockIdx.x) * kMaxRings + threadIdx.x] = s;
    }
}

// grid (kRingBlocks, K), block 256.
__global__ void k_ring_build(int n, const __grid_constant__ RingSet rs,
                             const float* __restrict__ ring_w, float* __restrict__ h,
                             double* __restrict__ partial) {
    const int k = blockIdx.y;
    const size_t px = size_t(n) * n;
    double acc[kMaxRings];
#pragma unroll
    for (int l = 0; l < kMaxRings; ++l) acc[l] = 0.0;
    float wl[kMaxRings];
#pragma unroll
    for (int l = 0; l < kMaxRings; ++l) wl[l] = ring_w ? ring_w[k * kMaxRings + l] : 1.f;
    float* hk = h + size_t(k) * px;
    for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < px;
         p += size_t(gridDim.x) * blockDim.x) {
        const RingValue v = ring_value(rs, k, n, p);
        float out = 0.f;
#pragma unroll
        for (int l = 0; l < kMaxRings; ++l)
            if (v.ring == l) {
                acc[l] += double(v.core);
                out = wl[l] * v.core;
            }
        hk[p] = out;
    }
    block_sums(acc, partial, k);
}

// grid K, block 32: ring_s[k][l] = sum over blocks (fixed order), zsum[k] =
// sum_l w_l ring_s[k][l].
__global__ void k_ring_final(const __grid_constant__ RingSet rs, const float* __restrict__ ring_w,
                             const double* __restrict__ partial, int nblocks,
                             double* __restrict__ ring_s, double* __restrict__ zsum) {
    const int k = blockIdx.x, l = threadIdx.x;
    __shared__ double s[kMaxRings];
    if (l < kMaxRings) {
        double a = 0.0;
        for (int b = 0; b < nblocks; ++b) a += partial[(size_t(k) * nblocks + b) * kMaxRings + l];
        s[l] = a;
        ring_s[k * kMaxRings + l] = a;
    }
    __syncthreads();
    if (l == 0) {
        double z = 0.0;
        for (int i = 0; i < rs.rings[k] && i < kMaxRings; ++i)
            z += double(ring_w ? ring_w[k * kMaxRings + i] : 1.f) * s[i];
        zsum[k] = z;
    }
}

// grid (kRingBlocks, K), block 256: G_l = sum over ring l of hbar * core.
__global__ void k_ring_grad(int n, const __grid_constant__ RingSet rs,
                            const float* __restrict__ hbar, double* __restrict__ partial) {
    const int k = blockIdx.y;
    const size_t px = size_t(n) * n;
    double acc[kMaxRings];
#pragma unroll
    for (int l = 0; l < kMaxRings; ++l) acc[l] = 0.0;
    const float* hb = hbar + size_t(k) * px;
    for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < px;
         p += size_t(gridDim.x) * blockDim.x) {
        const RingValue v = ring_value(rs, k, n, p);
        const double g = double(__ldg(&hb[p])) * double(v.core);
#pragma unroll
        for (int l = 0; l < kMaxRings; ++l)
            if (v.ring == l) acc[l] += g;
    }
    block_sums(acc, partial, k);
}

// grid K, block 32: h = sum_l b_l S_l / Z, Z = sum_l b_l s_l, so
// dL/db_l = (G_l - s_l sum_m b_m G_m / Z) / Z.
__global__ void k_ring_grad_final(const __grid_constant__ RingSet rs,
                                  const float* __restrict__ ring_w,
                                  const double* __restrict__ partial, int nblocks,
                                  const double* __restrict__ ring_s,
                                  const double* __restrict__ zsum, float* __restrict__ grad) {
    const int k = blockIdx.x, l = threadIdx.x;
    __shared__ double G[kMaxRings];
    if (l < kMaxRings) {
        double a = 0.0;
        for (int b = 0; b < nblocks; ++b) a += partial[(size_t(k) * nblocks + b) * kMaxRings + l];
        G[l] = a;
    }
    __syncthreads();
    if (l < kMaxRings) {
        const int B = rs.rings[k];
        double bg = 0.0;
        for (int m = 0; m < B && m < kMaxRings; ++m)
            bg += double(ring_w ? ring_w[k * kMaxRings + m] : 1.f) * G[m];
        const double z = zsum[k];
        const double g = (l < B && z != 0.0) ? (G[l] - ring_s[k * kMaxRings + l] * bg / z) / z : 0.0;
        grad[k * kMaxRings + l] = float(g);
    }
}

cudaError_t launch_ring_build(int n, int K, const RingSet& rs, const float* ring_w, float* h,
                              double* partial, double* ring_s, double* zsum, cudaStream_t s) {
    k_ring_build<<<dim3(kRingBlocks, K), 256, 0, s>>>(n, rs, ring_w, h, partial);
    k_ring_final<<<K, 32, 0, s>>>(rs, ring_w, partial, kRingBlocks, ring_s, zsum);
    return cudaGetLastError();
}

cudaError_t launch_ring_grad(int n, int K, const RingSet& rs, const float* ring_w,
                             const float* hbar, double* partial, const double* ring_s,
                             const double* zsum, float* grad, cudaStream_t s) {
    k_ring_grad<<<dim3(kRingBlocks, K), 256, 0, s>>>(n, rs, hbar, partial);
    k_ring_grad_final<<<K, 32, 0, s>>>(rs, ring_w, partial, kRingBlocks, ring_s, zsum, grad);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Tensor maps.  cuTensorMapEncodeTiled is a driver function; the runtime
// hands out its address, so the library links no driver library itself.
// U is viewed as a 2-D array of floats: rows = K * n/2 (kernel, kx), each
// 2n floats (n float2 over y), so a box of 2 rb floats by R rows is the
// tile (rb values of y) x (R values of kx) the inverse row pass needs,
// landing kx-major in shared memory.
// ---------------------------------------------------------------------------
namespace {
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}
}  // namespace

cudaError_t encode_u_map(CUtensorMap* map, const float2* U, int n, int K, int rb) {
    const EncodeTiledFn fn = encode_tiled_fn();
    if (!fn) return cudaErrorNotSupported;
    const int M = n / 2;
    const cuuint64_t dims[2] = {cuuint64_t(2) * n, cuuint64_t(K) * M};
    const cuuint64_t strides[1] = {cuuint64_t(n) * sizeof(float2)};
    const cuuint32_t box[2] = {cuuint32_t(2 * rb), cuuint32_t(M < 256 ? M : 256)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2*>(U), dims,
                          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Check of the bounded-wait path: one CTA waits on an mbarrier that no copy
// and no thread ever completes, through the same mbar_wait the step kernels
// use, with a short limit.  The wait gives up, records the timeout in the
// error word and the kernel returns: no hang, no fault.
// ---------------------------------------------------------------------------
__global__ void k_wait_check(int* err, unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    mbar_wait(&bar, 0, err, limit_ns);   // phase 0 never completes
    __syncthreads();
}

cudaError_t launch_wait_check(int* err, int timeout_ms, cudaStream_t s) {
    k_wait_check<<<1, 32, 0, s>>>(err, 1000000ull * unsigned(timeout_ms));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Gradient-search helpers: the MSE loss with its gradient, and an Adam step
// (the update rule of torch.optim.Adam, which train/ uses) whose step count
// lives on the device, so a captured graph can replay it.
// ---------------------------------------------------------------------------
__global__ void k_mse_partial(const float* __restrict__ x, const float* __restrict__ t,
                              size_t count, float* __restrict__ g, double* __restrict__ partial) {
    double s = 0.0;
    const float scale = float(2.0 / double(count));
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < count; i += stride) {
        const float d = __ldg(&x[i]) - __ldg(&t[i]);
        g[i] = scale * d;
        s += double(d) * double(d);
    }
    __shared__ double red[8];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void k_mse_final(const double* __restrict__ partial, int nblocks, size_t count,
                            double* __restrict__ loss) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) s += partial[i];
    __shared__ double red[8];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) *loss = v / double(count);
    }
}

template <class G>
__global__ void k_adam(float* __restrict__ p, const G* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t count, float lr, float b1, float b2,
                       float eps, const int* __restrict__ step) {
    const float t = float(*step + 1);   // the step being taken, 1-based
    const float bc1 = 1.f - powf(b1, t);
    const float bc2s = sqrtf(1.f - powf(b2, t));
    const float step_size = lr / bc1;
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < count; i += stride) {
        const float gi = float(g[i]);
        const float mi = fmaf(1.f - b1, gi - m[i], m[i]);          // lerp toward g
        const float vi = fmaf(1.f - b2, gi * gi, b2 * v[i]);
        m[i] = mi;
        v[i] = vi;
        p[i] -= step_size * (mi / (sqrtf(vi) / bc2s + eps));
    }
}

__global__ void k_count_step(int* step) { *step += 1; }

}  // namespace cg

extern "C" int cg_mse_grad(const float* x, const float* target, size_t count, float* grad,
                           double* loss, double* scratch, cg_stream_t stream) {
    using namespace cg;
    if (!x || !target || !grad || !loss || !scratch)
        return fail(CG_ERR_ARG, "cg_mse_grad: NULL pointer");
    if (count == 0) return fail(CG_ERR_ARG, "cg_mse_grad: empty input");
    auto st = static_cast<cudaStream_t>(stream);
    k_mse_partial<<<kMassBlocks, 256, 0, st>>>(x, target, count, grad, scratch);
    k_mse_final<<<1, 256, 0, st>>>(scratch, kMassBlocks, count, loss);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CG_OK : cuda_fail(e, "launching the MSE loss");
}

extern "C" int cg_adam_step(float* param, const float* grad_f32, const double* grad_f64,
                            float* m, float* v, size_t count, float lr, float beta1, float beta2,
                            float eps, const int* step, cg_stream_t stream) {
    using namespace cg;
    if (!param || !m || !v || !step || (!grad_f32) == (!grad_f64))
        return fail(CG_ERR_ARG, "cg_adam_step: NULL pointer, or not exactly one gradient");
    if (count == 0) return CG_OK;
    auto st = static_cast<cudaStream_t>(stream);
    const int blocks = grid_for(count);
    if (grad_f32)
        k_adam<float><<<blocks, 256, 0, st>>>(param, grad_f32, m, v, count, lr, beta1, beta2, eps,
                                             step);
    else
        k_adam<double><<<blocks, 256, 0, st>>>(param, grad_f64, m, v, count, lr, beta1, beta2,
                                              eps, step);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CG_OK : cuda_fail(e, "launching the Adam step");
}

extern "C" int cg_count_step(int* step, cg_stream_t stream) {
    using namespace cg;
    if (!step) return fail(CG_ERR_ARG, "cg_count_step: NULL pointer");
    k_count_step<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(step);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CG_OK : cuda_fail(e, "launching the step counter");
}

namespace cg {

// ---------------------------------------------------------------------------
// Mass reduction without device allocation (cg_mass_f64_noalloc).
//
// The per-block partial sums live in this fixed array instead of a buffer
// from cudaMalloc.  Every GPU that loads the library holds it (37,888 bytes)
// until the process exits.  Host code cannot pass the array's name to a
// kernel: on the host that name is only a stand-in, not a device address, so
// the address is looked up with cudaGetSymbolAddress once per device and
// context, while that device is current, and cached.  The cache key holds
// the current context's unique ID (cuCtxGetId, never reused within a
// process), so after cudaDeviceReset, or in another context on the same
// device, the first call looks the address up again instead of using one
// from a context that no longer exists.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxC = kMaxC;
static __device__ __align__(256) double g_mass_scratch[kNoAllocMaxC * kMassBlocks];

int fail(int code, const char* fmt, ...);

namespace {
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// The unique ID of the calling thread's current context (0 if there is none
// or the driver lacks cuCtxGetId).
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx &&
        get_id(ctx, &id) == CUDA_SUCCESS)
        return id;
    return 0;
}
}  // namespace

static cudaError_t mass_scratch_address(double** out) {
    static std::mutex mu;
    static std::unordered_map<int, std::pair<unsigned long long, double*>> by_device;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    auto it = by_device.find(dev);
    // a thread on which the runtime has not yet made the device's context
    // current reads ID 0 and takes the lookup, which makes it current
    const unsigned long long ctx = current_context_id();
    if (it == by_device.end() || ctx == 0 || it->second.first != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_mass_scratch);
        if (e != cudaSuccess) return e;
        // cudaGetSymbolAddress has initialised the context: read its ID now
        by_device[dev] = {current_context_id(), static_cast<double*>(p)};
        it = by_device.find(dev);
    }
    *out = it->second.second;
    return cudaSuccess;
}

}  // namespace cg

extern "C" int cg_mass_f64_noalloc(const float* dev_state, int n, int C, double* dev_out,
                                   cg_stream_t stream) {
    using namespace cg;
    if (!dev_state || !dev_out) return fail(CG_ERR_ARG, "cg_mass_f64_noalloc: NULL pointer");
    if (n < 1) return fail(CG_ERR_ARG, "cg_mass_f64_noalloc: grid side %d < 1", n);
    if (C < 1 || C > kNoAllocMaxC)
        return fail(CG_ERR_ARG,
                    "cg_mass_f64_noalloc: %d channels; its fixed scratch holds at most %d", C,
                    kNoAllocMaxC);
    double* scratch = nullptr;
    cudaError_t e = mass_scratch_address(&scratch);
    if (e != cudaSuccess)
        return fail(CG_ERR_CUDA, "cg_mass_f64_noalloc: scratch address: %s", cudaGetErrorString(e));
    // k_mass_partial overwrites every slot it uses, so nothing needs clearing.
    e = launch_mass_f64(dev_state, C, size_t(n) * size_t(n), scratch, kMassBlocks, dev_out,
                        static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return fail(CG_ERR_CUDA, "cg_mass_f64_noalloc: launch: %s", cudaGetErrorString(e));
    return CG_OK;
}
