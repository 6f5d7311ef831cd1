// adjoint.cuh — hand-written adjoint (vector-Jacobian product) of one
// DiffusionLenia step, templated on log2 of the grid side.
//
// Forward step (step_kernels.cuh; reference: train/diff_lenia_org.py:27-53):
//   u_k = h_k (*) x_{c0[k]},  e_k = exp(-(u_k-mu_k)^2 / (2 sigma_k^2)),
//   a_c = sum_{c1[k]=c} w_k (2 e_k - 1),  A = exp(temp a),
//   Z = box(A),  q = x / Z,  P = box(q),  x' = A P.
// Given ybar = dL/dx', one backward step is four launches, after
//   1. the row spectra, U and A of this x: recomputed by the step's own
//      kernels, or (cg_unroll_backward) kept from the segment's recompute,
//   2. k_diffusion_bwd: qbar = box(ybar A), xbar = qbar / Z,
//      Zbar = -qbar q / Z, Abar = ybar P + box(Zbar), abar = temp A Abar,
//   3. k_growth_bwd: u from U by the inverse row FFT; ebar = 2 w abar,
//      ubar = -ebar e (u-mu)/sigma^2, and the sums of
//      d/dw = (2e-1) abar, d/dmu = ebar e (u-mu)/sigma^2,
//      d/dsigma = ebar e (u-mu)^2/sigma^3; then the forward row FFT of ubar,
//      written over U,
//   4. k_col_conv_adj: the adjoint of a convolution with h is a convolution
//      with h(-m), whose spectrum is conj(K): per input channel, the sum over
//      its kernels of colFFT(ubar_k) conj(K_k), then one inverse column FFT,
//      written over the row spectra.  With a kernel-gradient buffer it also
//      accumulates sum_t colFFT(ubar_k) conj(colFFT(x_c0k)) = 4 FFT2(hbar_k)
//      (packed like U) from the same column transforms, from which k_col_inv
//      and k_row_c2r_add (scale 1/(4 n^2)) give the spatial kernel gradient
//      hbar_k = ubar (*) x(-.),
//   5. k_row_c2r_add: the inverse row FFT of that, added to xbar.
#pragma once
#include "step_kernels.cuh"

namespace cg {


// ---------------------------------------------------------------------------
// 2. Diffusion backward (one channel tile per CTA, 256 threads).
// ---------------------------------------------------------------------------
// A and ybar (2-pixel halo) and the state (1-pixel halo) arrive by 16-byte
// loads: their tiles reach 4 pixels past the tile on each side, so every
// load stays aligned (n is a multiple of 4, also across the toroidal wrap).
template <int LOGN, int V = 0>
struct DiffBwdGeo {
    static constexpr int TX = Geo<LOGN, V>::TX, TY = Geo<LOGN, V>::TY;
    static constexpr int AS = TX + 8, AH = TY + 4, HW = TX + 2, QH = TY + 2, V4 = AS / 4;
    static constexpr size_t SMEM = size_t(2 * AH * AS + QH * AS + 2 * QH * HW) * sizeof(float);
    static_assert(TX % 4 == 0, "tile shape");
};

template <int LOGN, int V = 0>
__device__ __forceinline__ void diffusion_bwd_body(const float* __restrict__ A,
                                                   const float* __restrict__ x,
                                                   const float* __restrict__ ybar,
                                                   float* __restrict__ xbar,
                                                   float* __restrict__ abar, float temp, int c,
                                                   int x0, int y0, float* smf) {
    using D = DiffBwdGeo<LOGN, V>;
    constexpr int N = Geo<LOGN, V>::N, TX = D::TX, TY = D::TY;
    constexpr int AS = D::AS, AH = D::AH, HW = D::HW, QH = D::QH, V4 = D::V4;
    // sA, sY: row r <-> y0 + r - 2; sX: row r <-> y0 + r - 1; column q <-> x0 - 4 + q
    auto sA = reinterpret_cast<float (*)[AS]>(smf);
    auto sY = reinterpret_cast<float (*)[AS]>(smf + AH * AS);
    auto sX = reinterpret_cast<float (*)[AS]>(smf + 2 * AH * AS);
    auto sQ = reinterpret_cast<float (*)[HW]>(smf + 2 * AH * AS + QH * AS);
    auto sZb = reinterpret_cast<float (*)[HW]>(smf + 2 * AH * AS + QH * AS + QH * HW);
    const size_t plane = size_t(c) * N * N;
    const float* Ap = A + plane;
    const float* Yp = ybar + plane;
    const float* Xp = x + plane;
    for (int i = threadIdx.x; i < AH * V4; i += blockDim.x) {
        const int r = i / V4, v = i % V4;
        const int cx = (x0 - 4 + 4 * v) & (N - 1);
        const size_t g = size_t((y0 + r - 2) & (N - 1)) * N + cx;
        *reinterpret_cast<float4*>(&sA[r][4 * v]) = __ldg(reinterpret_cast<const float4*>(Ap + g));
        *reinterpret_cast<float4*>(&sY[r][4 * v]) = __ldg(reinterpret_cast<const float4*>(Yp + g));
        if (r < QH)
            *reinterpret_cast<float4*>(&sX[r][4 * v]) = __ldg(reinterpret_cast<const float4*>(
                Xp + size_t((y0 + r - 1) & (N - 1)) * N + cx));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < QH * HW; i += blockDim.x) {
        const int r = i / HW, q = i % HW;
        float z = 0.f, qb = 0.f;
#pragma unroll
        for (int di = 0; di < 3; ++di)
#pragma unroll
            for (int dj = 0; dj < 3; ++dj) {
                const float a = sA[r + di][q + dj + 2];
                z += a;
                qb = fmaf(sY[r + di][q + dj + 2], a, qb);
            }
        const int gy = (y0 + r - 1) & (N - 1), gx = (x0 + q - 1) & (N - 1);
        const float xv = sX[r][q + 3];
        const float qv = xv / z;
        sQ[r][q] = qv;
        sZb[r][q] = -qb * qv / z;
        if (r >= 1 && r <= TY && q >= 1 && q <= TX) xbar[plane + size_t(gy) * N + gx] = qb / z;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TY * TX; i += blockDim.x) {
        const int r = i / TX, q = i % TX;
        float P = 0.f, SZ = 0.f;
#pragma unroll
        for (int di = 0; di < 3; ++di)
#pragma unroll
            for (int dj = 0; dj < 3; ++dj) {
                P += sQ[r + di][q + dj];
                SZ += sZb[r + di][q + dj];
            }
        const float a = sA[r + 2][q + 4];
        const float Ab = fmaf(sY[r + 2][q + 4], P, SZ);
        abar[plane + size_t(y0 + r) * N + x0 + q] = temp * a * Ab;
    }
}

template <int LOGN, int V = 0>
__global__ void __launch_bounds__(256) k_diffusion_bwd(const float* __restrict__ A,
                                                        const float* __restrict__ x,
                                                        const float* __restrict__ ybar,
                                                        float* __restrict__ xbar,
                                                        float* __restrict__ abar, float temp) {
    extern __shared__ __align__(128) float sm_dbwd[];
    pdl_wait();
    pdl_launch_dependents();
    diffusion_bwd_body<LOGN, V>(A, x, ybar, xbar, abar, temp, blockIdx.z, blockIdx.x * Geo<LOGN, V>::TX,
                             blockIdx.y * Geo<LOGN, V>::TY, sm_dbwd);
}

// Gather RB rows of a kx-major spectrum (src[kx * N + s]) into the row
// buffer (transposed) with per-element async copies; waits for them.
template <int LOGN, int V = 0>
__device__ __forceinline__ void gather_rows(const float2* __restrict__ src, float2* buf) {
    using G = Geo<LOGN, V>;
    for_row_tile<LOGN, V>([&](int s, int kx, int pk) {
        cp_async8(&buf[s * G::RP + pk], &src[size_t(kx) * G::N + s]);
    });
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
}

// Inverse row FFT of RB packed rows in `buf`; `out(s, i, v)` receives the
// pixel pair (x[2i], x[2i+1]) of row s.
template <int LOGN, int V, class OUT>
__device__ __forceinline__ void c2r_rows(float2* buf, const float2* __restrict__ tw, OUT& out) {
    using G = Geo<LOGN, V>;
    SmemRows rows{buf, G::RP};
    // m = j + q (M / R): m = 0 only in slot q = 0 (compile-time)
    auto ld0 = [&](int s, int m, int, int q) -> float2 {
        const float2* row = buf + s * G::RP;
        if (q == 0 && m == 0) {
            const float2 x = row[0];
            return make_float2(x.x + x.y, x.x - x.y);
        }
        const float2 a = row[pidx(m)];
        const float2 b = cconj(row[pidx(G::M - m)]);
        const float2 E = cadd(a, b);
        const float2 O = cmulc(csub(a, b), __ldg(&tw[m]));
        return make_float2(E.x - O.y, E.y + O.x);
    };
    auto st = [&](int s, int i, float2 v, int, int) { out(s, i, v); };
    FftPasses<G::M, 1, true, G::RT, G::RB, false, G::ROW_MR>::run(ld0, rows, rows, st, tw + G::TW_ROW);
}

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < int(blockDim.x >> 5); ++i) t += red[i];
    return t;
}

// ---------------------------------------------------------------------------
// 3. Growth backward, one kernel's RB rows per CTA (RT threads):
//    U[k] rows -> u -> ubar -> forward row FFT -> written over U[k].
// ---------------------------------------------------------------------------
template <int LOGN, int V = 0>
__device__ __forceinline__ void growth_bwd_body(float2* __restrict__ U,
                                                const float* __restrict__ abar,
                                                const float2* __restrict__ tw,
                                                const AdjointParams& ap, int k, int cout, int y0,
                                                double* __restrict__ pgrad, int K, float2* sm,
                                                double* red) {
    using G = Geo<LOGN, V>;
    float2* Uk = U + size_t(k) * G::M * G::N + y0;
    gather_rows<LOGN, V>(Uk, sm);
    const float mu = ap.mu[k], w = ap.w[k], is2 = ap.inv_s2[k], is3 = ap.inv_s3[k];
    const float* ab = abar + (size_t(cout) * G::N + y0) * G::N;
    float pw = 0.f, pmu = 0.f, psg = 0.f;
    auto out = [&](int s, int i, float2 v) {
        const float2 a = reinterpret_cast<const float2*>(ab + size_t(s) * G::N)[i];
        float ub[2];
        const float uu[2] = {v.x, v.y}, aa[2] = {a.x, a.y};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float d = uu[h] - mu;
            const float e = expf(-0.5f * d * d * is2);
            const float eb = 2.f * w * aa[h];
            const float t = eb * e * d;
            ub[h] = -t * is2;
            pw = fmaf(2.f * e - 1.f, aa[h], pw);
            pmu = fmaf(t, is2, pmu);
            psg = fmaf(t * d, is3, psg);
        }
        sm[s * G::RP + pidx(i)] = make_float2(ub[0], ub[1]);
    };
    c2r_rows<LOGN, V>(sm, tw, out);
    SmemRows rows{sm, G::RP};
    FftPasses<G::M, 1, false, G::RT, G::RB, false, G::ROW_MR>::run(rows, rows, rows, rows, tw + G::TW_ROW);
    r2c_finish<LOGN, V>(sm, tw, Uk);
    const double sw = block_sum(double(pw), red);
    const double smu = block_sum(double(pmu), red);
    const double ssg = block_sum(double(psg), red);
    if (threadIdx.x == 0) {
        atomicAdd(&pgrad[k], smu);
        atomicAdd(&pgrad[K + k], ssg);
        atomicAdd(&pgrad[2 * K + k], sw);
    }
}

template <int LOGN, int V = 0>
__global__ void __launch_bounds__(Geo<LOGN, V>::RT, 512 / Geo<LOGN, V>::RT) k_growth_bwd(float2* __restrict__ U,
                                                     const float* __restrict__ abar,
                                                     const float2* __restrict__ tw,
                                                     const AdjointParams* __restrict__ app,
                                                     double* __restrict__ pgrad, int K) {
    extern __shared__ __align__(128) float2 sm_gbwd[];
    __shared__ double red[16];
    pdl_wait();
    pdl_launch_dependents();
    const int k = blockIdx.y;
    growth_bwd_body<LOGN, V>(U, abar, tw, *app, k, app->cout[k], blockIdx.x * Geo<LOGN, V>::RB, pgrad, K,
                          sm_gbwd, red);
}

// ---------------------------------------------------------------------------
// 4. Adjoint column pass: per input channel c and TW columns,
//    sum over kernels k with c0[k] == c of colFFT(Ubar_k) conj(K_k)
//    (column 0: P conj(alpha) + conj P(-ky) conj(beta)), then one inverse
//    column FFT, written over the row spectra of c.
// ---------------------------------------------------------------------------
template <int LOGN, int V = 0>
__device__ __forceinline__ bool col_conv_adj_body(float2* __restrict__ rowspec,
                                                  const float2* __restrict__ kspec,
                                                  const float2* __restrict__ U,
                                                  float2* __restrict__ kgrad,
                                                  const float2* __restrict__ tw,
                                                  const KernelGroups& groups, int c, int kx0,
                                                  float2* sm, uint64_t* barp, uint32_t& phase,
                                                  int* err) {
    using G = Geo<LOGN, V>;
    constexpr int N = G::N, M = G::M, TW = G::TW, T = G::CT;
    float2* W = sm;
    float2* KS = sm + G::KSOFF;
    float2* Wx = KS + TW * N;   // with kgrad: colFFT of this channel's row spectra
    uint64_t& bar = *barp;
    const int cnt = groups.in_count[c], base = groups.in_start[c];
    float2* dst = rowspec + (size_t(c) * M + kx0) * N;
    constexpr uint32_t kTileBytes = uint32_t(TW) * N * sizeof(float2);
    constexpr int RL = last_radix(N);
    constexpr int JL = N / RL;
    constexpr int IPTL = (TW * JL + T - 1) / T;
    float2 acc[IPTL][RL];
#pragma unroll
    for (int it = 0; it < IPTL; ++it)
#pragma unroll
        for (int r = 0; r < RL; ++r) acc[it][r] = make_float2(0.f, 0.f);

    auto issue = [&](const float2* src) {
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(&bar, kTileBytes);
            bulk_g2s(KS, src, kTileBytes, &bar);
        }
    };
    auto wait_tile = [&]() -> bool {
        const bool ok = mbar_wait(&bar, phase & 1, err);
        if (__syncthreads_or(!ok)) {
            mbar_wait(&bar, phase & 1, nullptr);
            return false;
        }
        ++phase;
        return true;
    };
    auto ld_in = [&](int s, int i, int, int) { return KS[s * N + i]; };
    SmemRows wrows{W, G::CP};
    if (kgrad) {   // X = colFFT(row spectra of x), read before dst is overwritten
        issue(dst);
        if (!wait_tile()) return false;
        SmemRows xrows{Wx, G::CP};
        FftPasses<N, 1, false, T, TW, false>::run(ld_in, xrows, xrows, xrows, tw + G::TW_COL_FWD);
    }

    for (int gi = 0; gi < cnt; ++gi) {
        const int k = groups.in_idx[base + gi];
        float2* kg = kgrad ? kgrad + (size_t(k) * M + kx0) * N : nullptr;
        // this thread's kernel-gradient values, loaded now so that they land
        // during the column FFT below (only this CTA touches them)
        float2 kgv[IPTL][RL];
        if (kg) {
#pragma unroll
            for (int it = 0; it < IPTL; ++it) {
                const int item = threadIdx.x + it * T;
                if ((TW * JL) % T == 0 || item < TW * JL) {
                    const int s = item / JL, j = item % JL;
#pragma unroll
                    for (int r = 0; r < RL; ++r) kgv[it][r] = kg[size_t(s) * N + j + r * JL];
                }
            }
        }
        issue(U + (size_t(k) * M + kx0) * N);
        if (!wait_tile()) return false;
        const float2* ktile = kspec + (size_t(k) * (M + 1) + kx0) * N;
        fft_with_hook<N, false, T, TW, false>(ld_in, wrows, wrows, wrows, tw + G::TW_COL_FWD,
                                             [&]() { issue(ktile); });
        if (!wait_tile()) return false;
        const float2* kb = kspec + (size_t(k) * (M + 1) + M) * N;
#pragma unroll
        for (int it = 0; it < IPTL; ++it) {
            const int item = threadIdx.x + it * T;
            if ((TW * JL) % T == 0 || item < TW * JL) {
                const int s = item / JL, j = item % JL;
#pragma unroll
                for (int r = 0; r < RL; ++r) {
                    const int i = j + r * JL;
                    const float2 p = W[s * G::CP + pidx(i)];
                    float2 g = cmulc(p, KS[s * N + i]);
                    float2 pm;
                    if (kx0 + s == 0) {
                        pm = cconj(W[pidx((N - i) & (N - 1))]);
                        g = cadd(g, cmulc(pm, __ldg(&kb[i])));
                    }
                    acc[it][r] = cadd(acc[it][r], g);
                    if (kg) {
                        // kgrad_k += colFFT(ubar_k) conj(X); column 0 carries the
                        // kx = 0 and kx = n/2 spectra (FA = (P + conj P(-)) / 2,
                        // FB = (P - conj P(-)) / (2i)) and stores FA conj(XA) +
                        // i FB conj(XB)
                        const float2 px = Wx[s * G::CP + pidx(i)];
                        float2 v;
                        if (kx0 + s == 0) {
                            const float2 pxm = cconj(Wx[pidx((N - i) & (N - 1))]);
                            const float2 au = make_float2(0.5f * (p.x + pm.x), 0.5f * (p.y + pm.y));
                            const float2 du = make_float2(0.5f * (p.x - pm.x), 0.5f * (p.y - pm.y));
                            const float2 bu = make_float2(du.y, -du.x);
                            const float2 ax = make_float2(0.5f * (px.x + pxm.x), 0.5f * (px.y + pxm.y));
                            const float2 dx = make_float2(0.5f * (px.x - pxm.x), 0.5f * (px.y - pxm.y));
                            const float2 bx = make_float2(dx.y, -dx.x);
                            const float2 g0 = cmulc(au, ax), gm = cmulc(bu, bx);
                            v = make_float2(g0.x - gm.y, g0.y + gm.x);   // g0 + i gm
                        } else {
                            v = cmulc(p, px);
                        }
                        kg[size_t(s) * N + i] = cadd(kgv[it][r], v);
                    }
                }
            }
        }
        __syncthreads();
    }
    auto ld_acc = [&](int, int, int it, int r) { return acc[it][r]; };
    auto gst = [&](int s, int i, float2 v, int, int) { dst[size_t(s) * N + i] = v; };
    FftPasses<N, 1, true, T, TW, true>::run(ld_acc, wrows, wrows, gst, tw + G::TW_COL_INV);
    return true;
}

// Shared memory of the adjoint column pass: the forward pass's W and
// staging tile, then the row-spectrum transform X for the kernel gradient.
template <int LOGN, int V = 0>
struct AdjColGeo {
    static constexpr size_t SMEM =
        Geo<LOGN, V>::COL_SMEM + size_t(Geo<LOGN, V>::TW) * Geo<LOGN, V>::CP * sizeof(float2);
};

template <int LOGN, int V = 0>
__global__ void __launch_bounds__(Geo<LOGN, V>::CT, 512 / Geo<LOGN, V>::CT) k_col_conv_adj(float2* __restrict__ rowspec,
                                                          const float2* __restrict__ kspec,
                                                          const float2* __restrict__ U,
                                                          float2* __restrict__ kgrad,
                                                          const float2* __restrict__ tw,
                                                          const __grid_constant__ KernelGroups groups,
                                                          int* err) {
    extern __shared__ __align__(128) float2 sm_cadj[];
    __shared__ __align__(8) uint64_t bar;
    pdl_wait();
    pdl_launch_dependents();
    init_tile_barrier(&bar);
    uint32_t phase = 0;
    col_conv_adj_body<LOGN, V>(rowspec, kspec, U, kgrad, tw, groups, blockIdx.y,
                            blockIdx.x * Geo<LOGN, V>::TW, sm_cadj, &bar, phase, err);
}

// ---------------------------------------------------------------------------
// 5. Inverse row FFT of RB rows of a kx-major spectrum, scaled, written to
//    (or added to) a real [C or K][n][n] array.  grid (N/RB, planes), RT.
// ---------------------------------------------------------------------------
template <int LOGN, int V = 0>
__global__ void __launch_bounds__(Geo<LOGN, V>::RT, 512 / Geo<LOGN, V>::RT) k_row_c2r_add(const float2* __restrict__ src,
                                                      float* __restrict__ dst,
                                                      const float2* __restrict__ tw, float scale,
                                                      int accumulate) {
    using G = Geo<LOGN, V>;
    extern __shared__ __align__(128) float2 sm_c2ra[];
    pdl_wait();
    pdl_launch_dependents();
    const int c = blockIdx.y, y0 = blockIdx.x * G::RB;
    gather_rows<LOGN, V>(src + size_t(c) * G::M * G::N + y0, sm_c2ra);
    float* d = dst + (size_t(c) * G::N + y0) * G::N;
    auto out = [&](int s, int i, float2 v) {
        float2* p = reinterpret_cast<float2*>(d + size_t(s) * G::N) + i;
        float2 o = make_float2(v.x * scale, v.y * scale);
        if (accumulate) {
            const float2 old = *p;
            o.x += old.x;
            o.y += old.y;
        }
        *p = o;
    };
    c2r_rows<LOGN, V>(sm_c2ra, tw, out);
}

// Plain inverse column FFT of a kx-major [planes][M][N] spectrum, in place.
// grid (M/TW, planes), CT.
template <int LOGN, int V = 0>
__global__ void __launch_bounds__(Geo<LOGN, V>::CT) k_col_inv(float2* __restrict__ spec,
                                                  const float2* __restrict__ tw) {
    using G = Geo<LOGN, V>;
    constexpr int N = G::N, M = G::M, TW = G::TW, T = G::CT;
    extern __shared__ __align__(128) float2 sm_ci[];
    float2* col = spec + (size_t(blockIdx.y) * M + blockIdx.x * TW) * N;
    auto ld = [&](int s, int i, int, int) { return col[size_t(s) * N + i]; };
    SmemRows rows{sm_ci, G::CP};
    auto st = [&](int s, int i, float2 v, int, int) { col[size_t(s) * N + i] = v; };
    FftPasses<N, 1, true, T, TW, false>::run(ld, rows, rows, st, tw + G::TW_COL_FWD);
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
template <int LOGN, int V>
cudaError_t prepare_backward_variant() {
    using G = Geo<LOGN, V>;
    cudaError_t e;
    const void* fns[5] = {reinterpret_cast<const void*>(k_diffusion_bwd<LOGN, V>),
                          reinterpret_cast<const void*>(k_growth_bwd<LOGN, V>),
                          reinterpret_cast<const void*>(k_col_conv_adj<LOGN, V>),
                          reinterpret_cast<const void*>(k_row_c2r_add<LOGN, V>),
                          reinterpret_cast<const void*>(k_col_inv<LOGN, V>)};
    const size_t smem[5] = {DiffBwdGeo<LOGN, V>::SMEM, G::R2C_SMEM, AdjColGeo<LOGN, V>::SMEM,
                            G::R2C_SMEM, size_t(G::TW) * G::CP * sizeof(float2)};
    for (int i = 0; i < 5; ++i)
        if ((e = cudaFuncSetAttribute(fns[i], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(smem[i]))) != cudaSuccess)
            return e;
    return cudaSuccess;
}

template <int LOGN>
cudaError_t prepare_backward() {
    cudaError_t e = prepare_backward_variant<LOGN, 0>();
    if (e == cudaSuccess) e = prepare_backward_variant<LOGN, 1>();
    if (e == cudaSuccess) e = prepare_backward_variant<LOGN, 2>();
    return e;
}

// The adjoint kernels take the CTA shapes of the forward phases they mirror
// (the handle's tuned variants): the inverse row pass for the growth adjoint
// and the final row transform, the column pass for the adjoint column pass.
// The diffusion adjoint keeps one tile shape of its own (64 x 16, variant 1's
// Geo tile): the forward's tuned diffusion variant says nothing about it, and
// the three tiles measured within 1 % of each other in the backward.
constexpr int kDiffBwdVariant = 1;

// The backward step's kernels, launched like the forward ones
// (launch_pdl: each may start while the one before it drains).
template <int LOGN, int V>
cudaError_t launch_diff_bwd(const BwdArgs& a, cudaStream_t st) {
    using G = Geo<LOGN, V>;
    return launch_pdl(k_diffusion_bwd<LOGN, V>, dim3(G::N / G::TX, G::N / G::TY, a.C), 256,
                      DiffBwdGeo<LOGN, V>::SMEM, st, a.A, a.x, a.ybar, a.xbar, a.abar, a.temp);
}
template <int LOGN, int V>
cudaError_t launch_growth_bwd(const BwdArgs& a, cudaStream_t st) {
    using G = Geo<LOGN, V>;
    return launch_pdl(k_growth_bwd<LOGN, V>, dim3(G::N / G::RB, a.K), G::RT, G::R2C_SMEM, st,
                      a.U, a.abar, a.tw, a.ap, a.pgrad, a.K);
}
template <int LOGN, int V>
cudaError_t launch_col_adj(const BwdArgs& a, cudaStream_t st) {
    using G = Geo<LOGN, V>;
    return launch_pdl(k_col_conv_adj<LOGN, V>, dim3(G::M / G::TW, a.C), G::CT,
                      AdjColGeo<LOGN, V>::SMEM, st, a.rowspec, a.kspec, a.U, a.kgrad, a.tw,
                      a.groups, a.err);
}
template <int LOGN, int V>
cudaError_t launch_c2r_add(const BwdArgs& a, cudaStream_t st) {
    using G = Geo<LOGN, V>;
    return launch_pdl(k_row_c2r_add<LOGN, V>, dim3(G::N / G::RB, a.C), G::RT, G::R2C_SMEM, st,
                      static_cast<const float2*>(a.rowspec), a.xbar, a.tw, 1.f, 1);
}

template <int LOGN>
cudaError_t launch_backward(const BwdArgs& a, cudaStream_t st) {
    StepArgs f{};
    f.C = a.C;
    f.K = a.K;
    f.temp = a.temp;
    f.x_in = a.x;
    f.x_out = nullptr;
    f.rowspec = a.rowspec;
    f.kspec = a.kspec;
    f.kre = a.kre;
    f.U = a.U;
    f.A = a.A;
    f.tw = a.tw;
    f.udbg = nullptr;
    f.err = a.err;
    f.groups = a.groups;
    f.gp = a.gp;
    f.var = a.var;
    if (a.recompute) {
        const cudaError_t e = launch_step<LOGN>(f, kPhaseRowFwd | kPhaseColConv | kPhaseGrowth, st);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = launch_diff_bwd<LOGN, kDiffBwdVariant>(a, st);
    if (e != cudaSuccess) return e;
    // the adjoint kernels exist in the CTA shapes of variants 0-2: the plan
    // variants take the shape they share (row passes: two rows per CTA as
    // in variant 2; column pass: Geo::CVS)
    const int vrow = a.var.c2r > 2 ? 2 : a.var.c2r;
    const int vcol = a.var.col == 3 ? 1 : (a.var.col == 4 ? 0 : a.var.col);
    CG_VARIANT_SWITCH(vrow, e = launch_growth_bwd, a, st)
    if (e != cudaSuccess) return e;
    CG_VARIANT_SWITCH(vcol, e = launch_col_adj, a, st)
    if (e != cudaSuccess) return e;
    CG_VARIANT_SWITCH(vrow, e = launch_c2r_add, a, st)
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

// hbar[K][n][n] = inverse 2-D transform of the accumulated kgrad / (4 n^2)
// (kgrad is transformed in place).
template <int LOGN>
cudaError_t launch_kgrad_final(float2* kgrad, float* hbar, int K, const float2* tw,
                               cudaStream_t st) {
    using G = Geo<LOGN>;
    k_col_inv<LOGN, 0><<<dim3(G::M / G::TW, K), G::CT, size_t(G::TW) * G::CP * sizeof(float2), st>>>(
        kgrad, tw);
    k_row_c2r_add<LOGN, 0><<<dim3(G::N / G::RB, K), G::RT, G::R2C_SMEM, st>>>(
        kgrad, hbar, tw, 1.f / (4.f * float(G::N) * float(G::N)), 0);
    return cudaGetLastError();
}

}  // namespace cg
