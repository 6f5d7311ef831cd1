// On-GPU kernel-spectrum builder, grid-size specific part: from the row
// spectra of K spatial kernels (k_row_r2c over the kernels as if they were
// channels), the forward column FFT and the packing set_kernel's
// k_pack_kernel produces from a full spectrum, scaled by 1 / sum(h_k) so the
// kernel is normalised to sum 1 (generate_kernel_json.py:131-134,
// example.rs:384-392) without a second pass over the spatial values.
#pragma once

#include "adjoint.cuh"

namespace cg {

// grid (M/TW, K), CT threads.  rows: [K][M][N] (rowspec layout: 2x the row
// DFT, X[0] + i X[M] packed in column 0); zsum[k] = sum of kernel k's spatial
// values, or zsum = nullptr for no normaliser (the spectra of the kernels as
// given).  kspec: [K][M+1][N] packed as k_pack_kernel writes it.
template <int LOGN>
__global__ void __launch_bounds__(256) k_kspec_cols(const float2* __restrict__ rows,
                                                     float2* __restrict__ kspec,
                                                     const float2* __restrict__ tw,
                                                     const double* __restrict__ zsum) {
    using G = Geo<LOGN>;
    constexpr int N = G::N, M = G::M, TW = G::TW, T = G::CT;
    extern __shared__ __align__(128) float2 sm_kb[];
    const int k = blockIdx.y, kx0 = blockIdx.x * TW;
    const float2* src = rows + (size_t(k) * M + kx0) * N;
    auto ld = [&](int s, int i, int, int) { return __ldg(&src[size_t(s) * N + i]); };
    SmemRows cols{sm_kb, G::CP};
    FftPasses<N, 1, false, T, TW, false>::run(ld, cols, cols, cols, tw + G::TW_COL_FWD);
    __syncthreads();
    // P = 2 K^ (column kx >= 1); kspec holds K^ / (2 N^2 sum h)
    const double z = zsum ? zsum[k] : 1.0;
    const float scale = z != 0.0 ? float(1.0 / (4.0 * double(N) * double(N) * z)) : 0.f;
    float2* out = kspec + size_t(k) * (M + 1) * N;
    for (int e = threadIdx.x; e < TW * N; e += T) {
        const int s = e / N, i = e % N;
        const float2 p = sm_kb[s * G::CP + pidx(i)];
        if (kx0 + s == 0) {
            // P = 2 (A + i B), A = K^(0, ky), B = K^(M, ky) (both Hermitian
            // in ky); row 0 holds (A + B) / (4 N^2 sum h), row M (A - B) / ...
            const float2 pm = cconj(sm_kb[pidx((N - i) & (N - 1))]);
            const float2 u = make_float2(0.25f * (p.x + pm.x), 0.25f * (p.y + pm.y));   // A
            const float2 d = make_float2(0.25f * (p.x - pm.x), 0.25f * (p.y - pm.y));
            const float2 b = make_float2(d.y, -d.x);                                    // B = d / i
            out[i] = make_float2((u.x + b.x) * scale, (u.y + b.y) * scale);
            out[size_t(M) * N + i] = make_float2((u.x - b.x) * scale, (u.y - b.y) * scale);
        } else {
            out[size_t(kx0 + s) * N + i] = make_float2(p.x * scale, p.y * scale);
        }
    }
}

template <int LOGN>
cudaError_t prepare_builder() {
    using G = Geo<LOGN>;
    return cudaFuncSetAttribute(k_kspec_cols<LOGN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(size_t(G::TW) * G::CP * sizeof(float2)));
}

template <int LOGN>
cudaError_t launch_kspec_cols(const float2* rows, float2* kspec, const float2* tw,
                              const double* zsum, int K, cudaStream_t st) {
    using G = Geo<LOGN>;
    k_kspec_cols<LOGN><<<dim3(G::M / G::TW, K), G::CT, size_t(G::TW) * G::CP * sizeof(float2),
                         st>>>(rows, kspec, tw, zsum);
    return cudaGetLastError();
}

}  // namespace cg
