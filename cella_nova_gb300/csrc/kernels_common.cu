// Size-independent kernels: f64 -> f32 channel upload and the FP64 mass sum.
#include <mutex>
#include <unordered_map>

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
// Render the current state on its own (RenderPhase::run, render.rs:143-153):
// one packed 0x00RRGGBB word per pixel from channels 0..2, the same levels the
// diffusion epilogue writes.
// ---------------------------------------------------------------------------
__global__ void k_render(const float* __restrict__ x, int C, size_t px,
                         unsigned* __restrict__ out) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < px;
         i += size_t(gridDim.x) * blockDim.x) {
        unsigned v = render_level(__ldg(&x[i])) << 16;
        if (C > 1) v |= render_level(__ldg(&x[px + i])) << 8;
        if (C > 2) v |= render_level(__ldg(&x[2 * px + i]));
        out[i] = v;
    }
}

// download_render's conversion (mod.rs:322-329): packed words -> RGB24 bytes.
__global__ void k_rgb24(const unsigned* __restrict__ in, unsigned char* __restrict__ out,
                        size_t px) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < px;
         i += size_t(gridDim.x) * blockDim.x) {
        const unsigned v = __ldg(&in[i]);
        out[3 * i] = static_cast<unsigned char>(v >> 16);
        out[3 * i + 1] = static_cast<unsigned char>(v >> 8);
        out[3 * i + 2] = static_cast<unsigned char>(v);
    }
}

static int grid_for(size_t count) {
    return int((count + 255) / 256 < 4096 ? (count + 255) / 256 : 4096);
}

cudaError_t launch_render(const float* x, int C, size_t px, unsigned* out, cudaStream_t s) {
    k_render<<<grid_for(px), 256, 0, s>>>(x, C, px, out);
    return cudaGetLastError();
}

cudaError_t launch_rgb24(const unsigned* in, unsigned char* out, size_t px, cudaStream_t s) {
    k_rgb24<<<grid_for(px), 256, 0, s>>>(in, out, px);
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
// Mass reduction without device allocation (cg_mass_f64_noalloc).
//
// The per-block partial sums live in this fixed array instead of a buffer
// from cudaMalloc.  Every GPU that loads the library holds it (37,888 bytes)
// until the process exits.  Host code cannot pass the array's name to a
// kernel: on the host that name is only a stand-in, not a device address, so
// the address is looked up once per device with cudaGetSymbolAddress while
// that device is current, and cached.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxC = kMaxC;
static __device__ __align__(256) double g_mass_scratch[kNoAllocMaxC * kMassBlocks];

int fail(int code, const char* fmt, ...);

static cudaError_t mass_scratch_address(double** out) {
    static std::mutex mu;
    static std::unordered_map<int, double*> by_device;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    auto it = by_device.find(dev);
    if (it == by_device.end()) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_mass_scratch);
        if (e != cudaSuccess) return e;
        it = by_device.emplace(dev, static_cast<double*>(p)).first;
    }
    *out = it->second;
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
