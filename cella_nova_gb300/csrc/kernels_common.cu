// Size-independent kernels: f64 -> f32 channel upload and the FP64 mass sum.
#include "cella_internal.h"

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

}  // namespace cg
