// step_kernels.cuh — the four kernels of one DiffusionLenia step, templated
// on log2 of the grid side.
//
// Reference step (ml-rs/orchestrator/mod.rs:348-386) and what replaces it:
//   copy_to_conv + fft_row + fft_col per channel  (convolution.rs:627-679)
//       -> k_row_r2c: real-to-complex row FFT, written kx-major
//   slot copies + complex_mul + ifft_col per kernel (convolution.rs:688-763)
//       -> k_col_conv: column FFT of each input channel once, then for every
//          kernel reading that channel: multiply, inverse column FFT
//   ifft_row + mcl_growth  (convolution.rs:765-772, growth.rs:253-261)
//       -> k_row_c2r_growth: complex-to-real row FFT with the bump G(u), the
//          per-output weighted sum and exp(temp * .) fused into the epilogue
//   diffusion_pass1 + pass2 + state copy (diffusion.rs:280-302, mod.rs:377)
//       -> k_diffusion: one halo-tiled toroidal 3x3 kernel, ping-pong output
//
// Only the real part of each convolution is used (growth reads .x,
// compute_1024.wgsl:314), and the state is real, so the product with a
// kernel spectrum K equals the product with its Hermitian part
// (K(f) + conj K(-f))/2; the half spectrum (kx in [0, n/2]) therefore holds
// all the information.  Rows are stored as n/2 complex values with X[n/2]
// (real) packed into the imaginary part of X[0] (real).
#pragma once
#include "cella_internal.h"
#include "fft.cuh"

namespace cg {

template <int LOGN>
struct Geo {
    static constexpr int N = 1 << LOGN;
    static constexpr int M = N / 2;
    // Row kernels: RB rows per CTA, RT threads.
    static constexpr int RB0 = 8192 / M;
    static constexpr int RB = RB0 < 8 ? 8 : (RB0 > N ? N : RB0);
    static constexpr int RT = 512;
    static constexpr int RP = padded_len(M) + 1;   // odd pitch: conflict-free column reads
    static constexpr size_t ROW_SMEM = size_t(RB) * RP * sizeof(float2);
    // Column kernel: TW columns per CTA, CT threads, spectrum + work buffer.
    static constexpr int TW = 2;
    static constexpr int CT = 256;
    static constexpr int CP = padded_len(N) + 1;
    static constexpr size_t COL_SMEM = size_t(2 * TW) * CP * sizeof(float2);
    // Diffusion tile.
    static constexpr int TX = N < 64 ? N : 64;
    static constexpr int TY = N < 32 ? N : 32;
};

// ---------------------------------------------------------------------------
// Forward row pass: state rows -> packed half spectra, kx-major.
//   z[j] = x[2j] + i x[2j+1];  Z = FFT_M(z);
//   X[k] = E[k] + W_N^k O[k],  E = Z[k] + conj Z[M-k],  O = -i (Z[k] - conj Z[M-k])
// (E and O are twice the spectra of the even and odd samples), X[0] and
// X[M] are real and share slot 0.  Output scale: 2 x rfft.
// grid (N/RB, C), block RT.
// ---------------------------------------------------------------------------
template <int LOGN>
__global__ void __launch_bounds__(512) k_row_r2c(const float* __restrict__ state,
                                                  float2* __restrict__ rowspec,
                                                  const float2* __restrict__ tw) {
    using G = Geo<LOGN>;
    extern __shared__ float2 sm[];
    const int c = blockIdx.y;
    const int y0 = blockIdx.x * G::RB;
    const float2* src =
        reinterpret_cast<const float2*>(state + (size_t(c) * G::N + y0) * G::N);
    auto ld0 = [&](int s, int i) { return __ldg(&src[size_t(s) * G::M + i]); };
    auto smld = [&](int s, int i) { return sm[s * G::RP + pidx(i)]; };
    auto smst = [&](int s, int i, float2 v, int, int) { sm[s * G::RP + pidx(i)] = v; };
    FftPasses<G::M, 1, false, G::RT, G::RB, 2>::run(ld0, smld, smst, smst, tw);

    constexpr int H = G::M / 2;
    for (int item = threadIdx.x; item < G::RB * (H + 1); item += G::RT) {
        const int s = item / (H + 1), k = item % (H + 1);
        float2* row = sm + s * G::RP;
        if (k == 0) {
            const float2 z = row[0];
            row[0] = make_float2(2.f * (z.x + z.y), 2.f * (z.x - z.y));
        } else {
            const float2 a = row[pidx(k)], b = row[pidx(G::M - k)];
            const float2 E = make_float2(a.x + b.x, a.y - b.y);
            const float2 D = make_float2(a.x - b.x, a.y + b.y);
            const float2 O = make_float2(D.y, -D.x);
            const float2 wo = cmul(__ldg(&tw[k]), O);
            row[pidx(k)] = cadd(E, wo);
            if (k != H) row[pidx(G::M - k)] = cconj(csub(E, wo));
        }
    }
    __syncthreads();

    float2* dst = rowspec + size_t(c) * G::M * G::N + y0;
    for (int item = threadIdx.x; item < G::RB * G::M; item += G::RT) {
        const int s = item % G::RB, kx = item / G::RB;
        dst[size_t(kx) * G::N + s] = sm[s * G::RP + pidx(kx)];
    }
}

// ---------------------------------------------------------------------------
// Column pass: for TW consecutive kx of input channel c, the forward column
// FFT once, then for every kernel k with c0[k] == c the product with the
// kernel's half spectrum and the inverse column FFT, written to U[k].
// Column 0 carries two real-row spectra (kx = 0 and kx = n/2): with
// P = FA + i FB its column FFT, the kernel products recombine as
//   P(ky) alpha(ky) + conj P(-ky) beta(ky),
// alpha/beta = (K(.,0) +- K(.,n/2))/2 (prepared by k_pack_kernel).
// grid (M/TW, C), block CT.
// ---------------------------------------------------------------------------
template <int LOGN>
__global__ void __launch_bounds__(256) k_col_conv(const float2* __restrict__ rowspec,
                                                   const float2* __restrict__ kspec,
                                                   float2* __restrict__ U,
                                                   const float2* __restrict__ tw,
                                                   const KernelGroups groups) {
    using G = Geo<LOGN>;
    const int c = blockIdx.y;
    const int cnt = groups.in_count[c];
    if (cnt == 0) return;
    extern __shared__ float2 sm[];
    float2* F = sm;
    float2* W = sm + G::TW * G::CP;
    const int kx0 = blockIdx.x * G::TW;

    const float2* src = rowspec + (size_t(c) * G::M + kx0) * G::N;
    auto ld0 = [&](int s, int i) { return __ldg(&src[size_t(s) * G::N + i]); };
    auto fld = [&](int s, int i) { return F[s * G::CP + pidx(i)]; };
    auto fst = [&](int s, int i, float2 v, int, int) { F[s * G::CP + pidx(i)] = v; };
    FftPasses<G::N, 1, false, G::CT, G::TW, 1>::run(ld0, fld, fst, fst, tw);

    auto wld = [&](int s, int i) { return W[s * G::CP + pidx(i)]; };
    auto wst = [&](int s, int i, float2 v, int, int) { W[s * G::CP + pidx(i)] = v; };
    const int base = groups.in_start[c];
    for (int gi = 0; gi < cnt; ++gi) {
        const int k = groups.in_idx[base + gi];
        const float2* ks = kspec + (size_t(k) * (G::M + 1) + kx0) * G::N;
        const float2* kb = kspec + (size_t(k) * (G::M + 1) + G::M) * G::N;
        auto ldm = [&](int s, int i) {
            const float2 p = F[s * G::CP + pidx(i)];
            const float2 kv = __ldg(&ks[size_t(s) * G::N + i]);
            if (kx0 + s == 0) {
                const float2 pm = cconj(F[pidx((G::N - i) & (G::N - 1))]);
                return cadd(cmul(p, kv), cmul(pm, __ldg(&kb[i])));
            }
            return cmul(p, kv);
        };
        float2* dst = U + (size_t(k) * G::M + kx0) * G::N;
        auto gst = [&](int s, int i, float2 v, int, int) { dst[size_t(s) * G::N + i] = v; };
        FftPasses<G::N, 1, true, G::CT, G::TW, 1>::run(ldm, wld, wst, gst, tw);
    }
}

// ---------------------------------------------------------------------------
// Inverse row pass + growth: for every output channel c and every kernel k
// with c1[k] == c (in increasing k, as mcl_growth_main accumulates,
// compute_1024.wgsl:313-320): C2R of the rows of U[k], then
//   u = value (the 1/n^2 of growth.rs:87 is folded into kspec),
//   g = 2 exp(-(u-mu)^2 / (2 sigma^2)) - 1,  acc += w g;
// then A[c] = exp(temp * acc) (diffusion.rs:58-66 applies temp inside exp).
// C2R: Z[m] = E + i O, E = X[m] + conj X[M-m], O = (X[m] - conj X[M-m]) W_N^-m,
// z = IFFT_M(Z) = (x[2j], x[2j+1]).
// grid (N/RB), block RT.
// ---------------------------------------------------------------------------
template <int LOGN>
__global__ void __launch_bounds__(512) k_row_c2r_growth(const float2* __restrict__ U,
                                                         float* __restrict__ A,
                                                         const float2* __restrict__ tw,
                                                         const KernelGroups groups,
                                                         const GrowthParams gp, int C,
                                                         float temp, float* __restrict__ udbg,
                                                         float udbg_scale) {
    using G = Geo<LOGN>;
    extern __shared__ float2 sm[];
    const int y0 = blockIdx.x * G::RB;
    constexpr int RL = last_radix(G::M);
    constexpr int JL = G::M / RL;
    constexpr int ITEMS = G::RB * JL;
    constexpr int IPT = (ITEMS + G::RT - 1) / G::RT;

    auto smld = [&](int s, int i) { return sm[s * G::RP + pidx(i)]; };
    auto smst = [&](int s, int i, float2 v, int, int) { sm[s * G::RP + pidx(i)] = v; };
    auto ld0 = [&](int s, int m) -> float2 {
        const float2* row = sm + s * G::RP;
        if (m == 0) {
            const float2 x = row[0];
            return make_float2(x.x + x.y, x.x - x.y);
        }
        const float2 a = row[pidx(m)];
        const float2 b = cconj(row[pidx(G::M - m)]);
        const float2 E = cadd(a, b);
        const float2 O = cmulc(csub(a, b), __ldg(&tw[m]));
        return make_float2(E.x - O.y, E.y + O.x);
    };

    for (int c = 0; c < C; ++c) {
        float2 acc[IPT][RL];
#pragma unroll
        for (int it = 0; it < IPT; ++it)
#pragma unroll
            for (int r = 0; r < RL; ++r) acc[it][r] = make_float2(0.f, 0.f);

        const int cnt = groups.out_count[c], base = groups.out_start[c];
        for (int gi = 0; gi < cnt; ++gi) {
            const int k = groups.out_idx[base + gi];
            const float2* src = U + size_t(k) * G::M * G::N + y0;
            for (int item = threadIdx.x; item < G::RB * G::M; item += G::RT) {
                const int s = item % G::RB, kx = item / G::RB;
                sm[s * G::RP + pidx(kx)] = __ldg(&src[size_t(kx) * G::N + s]);
            }
            __syncthreads();
            const float mu = gp.mu[k], is2 = gp.inv_s2[k], w = gp.w[k];
            float* ud = udbg ? udbg + (size_t(k) * G::N + y0) * G::N : nullptr;
            auto gst = [&](int s, int i, float2 v, int it, int r) {
                const float dx = v.x - mu, dy = v.y - mu;
                const float gx = 2.f * expf(-0.5f * dx * dx * is2) - 1.f;
                const float gy = 2.f * expf(-0.5f * dy * dy * is2) - 1.f;
                acc[it][r].x += gx * w;
                acc[it][r].y += gy * w;
                if (ud) {
                    reinterpret_cast<float2*>(ud + size_t(s) * G::N)[i] =
                        make_float2(v.x * udbg_scale, v.y * udbg_scale);
                }
            };
            FftPasses<G::M, 1, true, G::RT, G::RB, 2>::run(ld0, smld, smst, gst, tw);
        }

        float* Ac = A + (size_t(c) * G::N + y0) * G::N;
#pragma unroll
        for (int it = 0; it < IPT; ++it) {
            const int item = threadIdx.x + it * G::RT;
            if (ITEMS % G::RT == 0 || item < ITEMS) {
                const int s = item / JL, j = item % JL;
#pragma unroll
                for (int r = 0; r < RL; ++r) {
                    const int i = j + r * JL;
                    reinterpret_cast<float2*>(Ac + size_t(s) * G::N)[i] =
                        make_float2(expf(temp * acc[it][r].x), expf(temp * acc[it][r].y));
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Diffusion: Z = toroidal 3x3 sum of A, new = A * (3x3 sum of state / Z),
// summed in the reference's order (example.rs:275-301,
// compute_1024.wgsl:356-411).  One channel tile per CTA; A is read with a
// 2-pixel halo and the state with a 1-pixel halo, so both passes and the
// state copy of mod.rs:377-383 collapse into one kernel writing x_out.
// grid (N/TX, N/TY, C), block 256.
// ---------------------------------------------------------------------------
template <int LOGN>
__global__ void __launch_bounds__(256) k_diffusion(const float* __restrict__ A,
                                                    const float* __restrict__ x,
                                                    float* __restrict__ out) {
    using G = Geo<LOGN>;
    constexpr int N = G::N, TX = G::TX, TY = G::TY;
    constexpr int AW = TX + 4, AH = TY + 4, QW = TX + 2, QH = TY + 2;
    __shared__ float sA[AH][AW];
    __shared__ float sQ[QH][QW];
    const int c = blockIdx.z;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const float* Ac = A + size_t(c) * N * N;
    const float* xc = x + size_t(c) * N * N;
    for (int i = threadIdx.x; i < AH * AW; i += blockDim.x) {
        const int r = i / AW, q = i % AW;
        const int gy = (y0 + r - 2) & (N - 1), gx = (x0 + q - 2) & (N - 1);
        sA[r][q] = __ldg(&Ac[size_t(gy) * N + gx]);
    }
    for (int i = threadIdx.x; i < QH * QW; i += blockDim.x) {
        const int r = i / QW, q = i % QW;
        const int gy = (y0 + r - 1) & (N - 1), gx = (x0 + q - 1) & (N - 1);
        sQ[r][q] = __ldg(&xc[size_t(gy) * N + gx]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < QH * QW; i += blockDim.x) {
        const int r = i / QW, q = i % QW;
        // Z as an unevaluated float pair (zh + zl): TwoSum keeps every
        // rounding error, so zh + zl is the 3x3 sum to ~1e-14.  A plain f32
        // sum is off by a fixed relative amount wherever A is constant
        // (G = -1 for every kernel across a whole region), which drifts the
        // total mass by ~1e-8 per step; with the exact Z the only errors
        // left are the unbiased roundings of q, the sum of q and the product.
        float zh = sA[r][q], zl = 0.f;
#pragma unroll
        for (int t = 1; t < 9; ++t) {
            const float b = sA[r + t / 3][q + t % 3];
            const float s = zh + b;
            const float bb = s - zh;
            zl += (zh - (s - bb)) + (b - bb);
            zh = s;
        }
        const float z = zh + zl;
        zl = zl - (z - zh);
        zh = z;
        // q = x / (zh + zl), from the exact remainder of x / zh
        const float xv = sQ[r][q];
        const float q0 = xv / zh;
        const float rem = fmaf(-q0, zh, xv);
        sQ[r][q] = q0 + (rem - q0 * zl) / zh;
    }
    __syncthreads();
    float* oc = out + size_t(c) * N * N;
    for (int i = threadIdx.x; i < TY * TX; i += blockDim.x) {
        const int r = i / TX, q = i % TX;
        float s = 0.f;
#pragma unroll
        for (int di = 0; di < 3; ++di)
#pragma unroll
            for (int dj = 0; dj < 3; ++dj) s += sQ[r + di][q + dj];
        oc[size_t(y0 + r) * N + x0 + q] = sA[r + 2][q + 2] * s;
    }
}

// ---------------------------------------------------------------------------
// Kernel spectrum packing (set_kernel, mod.rs:207-214): full n x n spectrum
// [ky][kx] -> Hermitian part, scaled by 1/(2 n^2), kx-major [kx][ky] for
// kx in [1, n/2), with the alpha/beta pair in columns 0 and n/2.
// ---------------------------------------------------------------------------
template <int LOGN>
__global__ void k_pack_kernel(const float2* __restrict__ full, float2* __restrict__ out) {
    using G = Geo<LOGN>;
    constexpr int N = G::N, M = G::M;
    constexpr float scale = 0.5f / (2.0f * float(N) * float(N));
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * N) return;
    const int kx = i / N, ky = i % N;
    auto herm = [&](int fy, int fx) {
        const float2 a = full[size_t(fy) * N + fx];
        const float2 b = full[size_t((N - fy) & (N - 1)) * N + ((N - fx) & (N - 1))];
        return make_float2((a.x + b.x) * scale, (a.y - b.y) * scale);
    };
    if (kx == 0) {
        const float2 k0 = herm(ky, 0), km = herm(ky, M);
        out[ky] = make_float2(0.5f * (k0.x + km.x), 0.5f * (k0.y + km.y));
        out[size_t(M) * N + ky] = make_float2(0.5f * (k0.x - km.x), 0.5f * (k0.y - km.y));
    } else {
        out[size_t(kx) * N + ky] = herm(ky, kx);
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers for one grid size.
// ---------------------------------------------------------------------------
template <int LOGN>
cudaError_t prepare_size() {
    using G = Geo<LOGN>;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_row_r2c<LOGN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(G::ROW_SMEM))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_row_c2r_growth<LOGN>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(G::ROW_SMEM))) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_col_conv<LOGN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(G::COL_SMEM));
}

template <int LOGN>
cudaError_t launch_step(const StepArgs& a, int phases, cudaStream_t st) {
    using G = Geo<LOGN>;
    if (phases & kPhaseRowFwd)
        k_row_r2c<LOGN><<<dim3(G::N / G::RB, a.C), G::RT, G::ROW_SMEM, st>>>(a.x_in, a.rowspec,
                                                                            a.tw);
    if (phases & kPhaseColConv)
        k_col_conv<LOGN><<<dim3(G::M / G::TW, a.C), G::CT, G::COL_SMEM, st>>>(
            a.rowspec, a.kspec, a.U, a.tw, a.groups);
    if (phases & kPhaseGrowth)
        k_row_c2r_growth<LOGN><<<G::N / G::RB, G::RT, G::ROW_SMEM, st>>>(
            a.U, a.A, a.tw, a.groups, a.gp, a.C, a.temp, a.udbg, float(G::N) * float(G::N));
    if (phases & kPhaseDiffusion)
        k_diffusion<LOGN><<<dim3(G::N / G::TX, G::N / G::TY, a.C), 256, 0, st>>>(a.A, a.x_in,
                                                                                 a.x_out);
    return cudaGetLastError();
}

template <int LOGN>
cudaError_t launch_pack(const float2* full, float2* out, cudaStream_t st) {
    using G = Geo<LOGN>;
    const int total = G::M * G::N;
    k_pack_kernel<LOGN><<<(total + 255) / 256, 256, 0, st>>>(full, out);
    return cudaGetLastError();
}

}  // namespace cg

#define CG_DEFINE_SIZE_OPS(LOGN)                                                        \
    namespace cg {                                                                      \
    extern const SizeOps size_ops_l##LOGN;                                              \
    const SizeOps size_ops_l##LOGN = {launch_step<LOGN>, launch_pack<LOGN>,             \
                                      prepare_size<LOGN>};                              \
    }
