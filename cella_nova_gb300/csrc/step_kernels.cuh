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
#include "async_copy.cuh"
#include "fft.cuh"
#include "render.cuh"

namespace cg {

// Geometry of one grid size.  V selects a variant (the autotuner times
// them): row kernels V=1 / V=2 halve / quarter the rows per CTA and the
// threads (the forward row pass's variant 2 streams variant 1's tile
// instead, R2CShape); the column kernel V=1 halves and V=2 doubles the
// columns and the threads per CTA (work per thread is unchanged); diffusion
// V=1 keeps its sums in registers (DiffGeoReg, 16-row strips; V=3 the same
// in 8-row strips, DiffTile) and V=2 uses 64 tile rows with two columns per
// thread instead of 32 rows (the diffusion adjoint takes V=1 as 16 tile
// rows).  Variants 0-2, and diffusion's 3, compute the same bits.
//
// Variants 3 and 4 (grid sides of at least kMinPairLogN) change the FFT
// plans instead of only the shapes, and agree with the others to rounding:
// the row passes transform two real rows as one complex sequence of length
// n (PairGeo, pair_rows.cuh) with radix-16 (V=3) or radix-8 (V=4) plans;
// the column pass runs the remainder-first plan forward and the greedy plan
// inverse (the order of variants 0-2 reversed) in the CTA shape of V=1
// (V=3) or V=0 (V=4).  Layouts in memory do not depend on V.
template <int LOGN, int V = 0>
struct Geo {
    static_assert(V >= 0 && V <= 4, "variant");
    static_assert(V <= 2 || LOGN >= kMinPairLogN, "plan variants need n >= 512");
    static constexpr int N = 1 << LOGN;
    static constexpr int M = N / 2;
    // Row kernels: RB rows per CTA, RT threads, radix-16 plans (ROW_MR).  The
    // row pitch RP keeps the accesses of a half-warp that spans the rows
    // (kx-major transposes, and the row-fastest passes of the inverse row
    // pass) conflict-free: odd for RB >= 16 (16 rows of one column), 2 mod 16
    // for RB = 8 (8 rows x 2 columns), 4 mod 16 for RB = 4, 8 mod 16 for
    // RB = 2 (2 rows x 8 columns).
    static constexpr int RB0 = 8192 / M;
    static constexpr int RB1 = RB0 < 8 ? 8 : (RB0 > N ? N : RB0);
    static constexpr int RB = (V == 1) ? RB1 / 2 : (V == 2 ? RB1 / 4 : RB1);
    static constexpr int RT = (V == 0) ? 512 : (V == 1 ? 256 : 128);
    static constexpr int ROW_MR = 16;
    static constexpr int RP = padded_len(M) + (RB >= 16 ? 1 : (RB == 8 ? 2 : (RB == 4 ? 4 : 8)));
    static constexpr size_t R2C_SMEM = size_t(RB) * RP * sizeof(float2);
    // Inverse row pass: the padded work rows, then one landing tile for a
    // kernel's U tile (RB values of y by M values of kx, kx-major), filled by
    // 2-D tensor copies of boxes of UBOX kx; 128-byte aligned.
    static constexpr int UBOX = M < 256 ? M : 256;
    static constexpr int C2R_LAND = (RB * RP + 15) & ~15;
    static constexpr int C2R_TILE = RB * M;
    static_assert((C2R_TILE * sizeof(float2)) % 128 == 0 && (RB * UBOX * sizeof(float2)) % 128 == 0,
                  "tensor-copy destination alignment");
    static constexpr size_t C2R_SMEM = (size_t(C2R_LAND) + size_t(C2R_TILE)) * sizeof(float2);
    static_assert(C2R_SMEM <= 227 * 1024, "inverse row pass shared memory");
    // Column kernel: TW columns per CTA, CT threads; a padded work buffer
    // and an unpadded staging tile that bulk copies fill.  TW = 4096/N keeps
    // 256 butterflies per radix-16 pass (one per thread) at every size.
    // CVS: the CTA shape of the column pass (V=3 takes V=1's, V=4 V=0's);
    // COL_SWAP: the remainder-first plan forward, the greedy plan inverse.
    static constexpr int CVS = (V == 3) ? 1 : (V == 4 ? 0 : V);
    static constexpr bool COL_SWAP = (V >= 3);
    static constexpr int TW0 = 4096 / N;
    static constexpr int TW1 = TW0 < 2 ? 2 : (TW0 > M ? M : TW0);
    static constexpr int TW = (CVS == 1) ? (TW1 > 1 ? TW1 / 2 : 1)
                                         : (CVS == 2 ? (2 * TW1 > M ? M : 2 * TW1) : TW1);
    static constexpr int CT = (CVS == 1) ? 128 : (CVS == 2 ? 512 : 256);
    // Resident CTAs per SM the compiler must allow for (the register cap) in
    // the single-world column pass: the small-CTA variant asks for five, which
    // ptxas meets without spills (96 registers at n = 2048; 66.0 against
    // 67.6 us).  Six CTAs of the swapped-plan variant 3 (80 registers, no
    // spills) ran at 62.1 against 61.1 us, so it keeps five.  On the inverse
    // row pass, three CTAs of 256 threads (80 registers) ran at 121 against
    // 92 us and five of the 128-thread variant at 63.5 against 63.7 us; only
    // the paired variant 3 takes a cap there (pair_rows.cuh).
    static constexpr int COL_MINB = (CVS == 1) ? 5 : 512 / CT;
    static constexpr int CP = padded_len(N) + 1;
    // the staging tile is a bulk-copy (TMA) destination: 16-byte aligned
    static constexpr int KSOFF = (TW * CP + 1) & ~1;
    static_assert((KSOFF * sizeof(float2)) % 16 == 0, "bulk-copy destination alignment");
    static constexpr size_t COL_SMEM = (size_t(KSOFF) + size_t(TW) * N) * sizeof(float2);
    // Twiddle buffer: W_N^m (m < N), then the pass tables of the column
    // forward plan (greedy radix 16, length N), the column inverse plan
    // (remainder first), the row plan (greedy, length M) and the radix-8
    // plan of length N (the paired row passes of V=4).
    static constexpr int TW_COL_FWD = N;
    static constexpr int TW_COL_INV = TW_COL_FWD + tw_size(N, false);
    static constexpr int TW_ROW = TW_COL_INV + tw_size(N, true);
    static constexpr int TW_PAIR8 = TW_ROW + tw_size(M, false);
    static constexpr int TW_TOTAL = TW_PAIR8 + tw_size(N, false, 8);
    // Diffusion tile.
    static constexpr int TX = N < 64 ? N : 64;
    static constexpr int TY0 = (V == 1) ? 16 : (V == 2 ? 64 : 32);
    static constexpr int TY = N < TY0 ? N : TY0;
};

}  // namespace cg
#include "pair_rows.cuh"
namespace cg {

// ---------------------------------------------------------------------------
// Forward row pass: state rows -> packed half spectra, kx-major.
//   z[j] = x[2j] + i x[2j+1];  Z = FFT_M(z);
//   X[k] = E[k] + W_N^k O[k],  E = Z[k] + conj Z[M-k],  O = -i (Z[k] - conj Z[M-k])
// (E and O are twice the spectra of the even and odd samples), X[0] and
// X[M] are real and share slot 0.  Output scale: 2 x rfft.
// grid (N/RB, C), block RT.
// ---------------------------------------------------------------------------
// Visit the RB x M elements (row s, column kx) of a kx-major row tile with
// the RT threads of a row kernel: thread t owns row s = t % RB and columns
// t / RB + i * (RT / RB), so both the padded shared index pidx(kx) and the
// global address advance by constants (pidx(kx + STEP) = pidx(kx) +
// pidx(STEP) when STEP is a multiple of 16).  f(s, kx, pidx(kx)).
template <int LOGN, int V, class F>
__device__ __forceinline__ void for_row_tile(F f) {
    using G = Geo<LOGN, V>;
    static_assert(G::RT % G::RB == 0, "a thread keeps one row");
    constexpr int STEP = G::RT / G::RB;
    const int s = threadIdx.x % G::RB, kx0 = threadIdx.x / G::RB;
    if constexpr (G::M % STEP == 0 && STEP % 16 == 0) {
        const int pk0 = pidx(kx0);
#pragma unroll
        for (int i = 0; i < G::M / STEP; ++i) f(s, kx0 + i * STEP, pk0 + i * pidx(STEP));
    } else {
        for (int kx = kx0; kx < G::M; kx += STEP) f(s, kx, pidx(kx));
    }
}

template <int LOGN, int V = 0>
__device__ __forceinline__ void r2c_finish(float2* sm, const float2* __restrict__ tw,
                                           float2* __restrict__ dst);

template <int LOGN, int V = 0>
__device__ __forceinline__ void row_r2c_body(const float* __restrict__ state,
                                             float2* __restrict__ rowspec,
                                             const float2* __restrict__ tw, int c, int y0,
                                             float2* sm) {
    using G = Geo<LOGN, V>;
    const float2* src =
        reinterpret_cast<const float2*>(state + (size_t(c) * G::N + y0) * G::N);
    auto ld0 = [&](int s, int i, int, int) { return __ldg(&src[size_t(s) * G::M + i]); };
    SmemRows rows{sm, G::RP};
    // the first pass reads global memory: no load-store barrier
    FftPasses<G::M, 1, false, G::RT, G::RB, false, G::ROW_MR, false, false, true>::run(
        ld0, rows, rows, rows, tw + G::TW_ROW);
    r2c_finish<LOGN, V>(sm, tw, rowspec + size_t(c) * G::M * G::N + y0);
}

// Even/odd split of RB transformed rows in shared memory (X[k] from Z[k],
// Z[M-k]; X[0], X[M] packed in slot 0), stored straight to the kx-major
// rows dst[kx * N + s].  The row index runs fastest over the threads, so RB
// consecutive lanes write one column's RB rows (a full sector for RB = 4),
// and the shared reads stay conflict-free with the row pitch RP.
template <int LOGN, int V>
__device__ __forceinline__ void r2c_finish(float2* sm, const float2* __restrict__ tw,
                                           float2* __restrict__ dst) {
    using G = Geo<LOGN, V>;
    constexpr int H = G::M / 2, RB = G::RB;
    auto split = [&](int s, int k, float2& lo, float2& hi) {   // X[k], conj X[M-k] for 0 < k <= H
        const float2* row = sm + s * G::RP;
        const float2 a = row[pidx(k)], b = row[pidx(G::M - k)];
        const float2 E = make_float2(a.x + b.x, a.y - b.y);
        const float2 D = make_float2(a.x - b.x, a.y + b.y);
        const float2 O = make_float2(D.y, -D.x);
        const float2 wo = cmul(__ldg(&tw[k]), O);
        lo = cadd(E, wo);
        hi = cconj(csub(E, wo));
    };
    // k = 0 (slot 0 holds X[0] and X[M]) and k = H (its own mirror) take the
    // first 2 RB threads, so the loop over 0 < k < H tests nothing per item
    if (threadIdx.x < RB) {
        const int s = threadIdx.x;
        const float2 z = sm[s * G::RP];
        dst[s] = make_float2(2.f * (z.x + z.y), 2.f * (z.x - z.y));
    } else if (threadIdx.x < 2 * RB) {
        const int s = threadIdx.x - RB;
        float2 lo, hi;
        split(s, H, lo, hi);
        dst[size_t(H) * G::N + s] = lo;
    }
    for (int item = threadIdx.x + RB; item < RB * H; item += G::RT) {
        const int s = item % RB, k = item / RB;
        float2 lo, hi;
        split(s, k, lo, hi);
        dst[size_t(k) * G::N + s] = lo;
        dst[size_t(G::M - k) * G::N + s] = hi;
    }
}

// The forward row pass of variant V on the RB rows from y0 (R2CShape).
template <int LOGN, int V>
__device__ __forceinline__ void row_r2c_variant(const float* __restrict__ state,
                                                float2* __restrict__ rowspec,
                                                const float2* __restrict__ tw, int c, int y0,
                                                float2* sm) {
    if constexpr (R2CShape<LOGN, V>::PAIR)
        pair_r2c_body<typename R2CShape<LOGN, V>::P>(state, rowspec, tw, c, y0, sm);
    else
        row_r2c_body<LOGN, V>(state, rowspec, tw, c, y0, sm);
}

__device__ __forceinline__ void init_tile_barrier(uint64_t* bar) {
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
}

// The streaming form of the forward row pass (R2CShape<LOGN, 2>): this CTA
// takes blocks blockIdx.x, blockIdx.x + gridDim.x, ... of `count`;
// item(i, src, dst) names block i's RB state rows (contiguous) and its
// destination in the kx-major row spectra.  The rows arrive by one bulk copy
// into the staging tile; the next block's copy is issued once the first FFT
// pass has read the tile, so it lands while the remaining passes and the
// stores run.  Same arithmetic as variant 1, so the same bits.  Returns
// false if a bounded wait timed out (the error word is set).  `bar` is an
// initialised mbarrier; `phase` counts its completed phases.
template <int LOGN, class ITEM>
__device__ __forceinline__ bool row_r2c_stream(ITEM item, int count,
                                               const float2* __restrict__ tw, float2* sm,
                                               uint64_t* barp, uint32_t& phase, int* err) {
    using Sh = R2CShape<LOGN, 2>;
    using G = typename Sh::G;
    const float2* stg = sm + Sh::STG;
    uint64_t& bar = *barp;
    auto issue = [&](int i) {   // all threads call; thread 0 copies
        const float* src;
        float2* dst;
        item(i, src, dst);
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(&bar, Sh::kBlockBytes);
            bulk_g2s(const_cast<float2*>(stg), src, Sh::kBlockBytes, &bar);
        }
    };
    if (int(blockIdx.x) < count) issue(blockIdx.x);
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        const bool ok = mbar_wait(&bar, phase & 1u, err);
        if (__syncthreads_or(!ok)) {
            // one more bounded chance for the copy in flight to land before
            // this CTA's shared memory is released
            mbar_wait(&bar, phase & 1u, nullptr);
            return false;
        }
        ++phase;
        const float* src;
        float2* dst;
        item(i, src, dst);
        auto ld0 = [&](int s, int j, int, int) { return stg[s * G::M + j]; };
        SmemRows rows{sm, G::RP};
        // the first pass reads the staging tile and writes the work rows: no
        // load-store barrier (the wait above ordered the previous block's
        // reads of the work rows)
        fft_with_hook<G::M, false, G::RT, G::RB, false, G::ROW_MR, false, false, true>(
            ld0, rows, rows, rows, tw + G::TW_ROW, [&]() {
                if (i + int(gridDim.x) < count) issue(i + gridDim.x);
            });
        r2c_finish<LOGN, 1>(sm, tw, dst);
        __syncthreads();
    }
    return true;
}

// grid (N/RB, C) for the block variants; for the streaming variant a
// persistent grid over the nc * N/RB blocks of channels cbase.. (gridDim.x
// CTAs, gridDim.y = 1).
template <int LOGN, int V = 0>
__global__ void __launch_bounds__(R2CShape<LOGN, V>::RT, R2CShape<LOGN, V>::MINB)
    k_row_r2c(const float* __restrict__ state, float2* __restrict__ rowspec,
              const float2* __restrict__ tw, int cbase, int nc, int* err) {
    extern __shared__ __align__(128) float2 sm_r2c[];
    using Sh = R2CShape<LOGN, V>;
    pdl_wait();
    pdl_launch_dependents();
    if constexpr (Sh::STREAM) {
        constexpr int N = 1 << LOGN, NB = N / Sh::RB;
        __shared__ __align__(8) uint64_t bar;
        init_tile_barrier(&bar);
        uint32_t phase = 0;
        auto item = [&](int i, const float*& src, float2*& dst) {
            const int c = cbase + i / NB, y0 = (i % NB) * Sh::RB;
            src = state + (size_t(c) * N + y0) * N;
            dst = rowspec + size_t(c) * (N / 2) * N + y0;
        };
        row_r2c_stream<LOGN>(item, nc * NB, tw, sm_r2c, &bar, phase, err);
    } else {
        row_r2c_variant<LOGN, V>(state, rowspec, tw, blockIdx.y + cbase, blockIdx.x * Sh::RB,
                                 sm_r2c);
    }
}

// ---------------------------------------------------------------------------
// Column pass: for TW consecutive kx of input channel c, the forward column
// FFT once, then for every kernel k with c0[k] == c the product with the
// kernel's half spectrum and the inverse column FFT, written to U[k].
//
// Data movement: the input columns and each kernel's spectrum columns are
// contiguous (kx-major layouts), so each arrives by one 1-D bulk copy (TMA)
// into the staging tile KS, tracked by an mbarrier; the next kernel's copy
// is issued as soon as the current one has been consumed by the first
// inverse pass, and lands while the remaining passes run.  The forward
// spectrum never returns to shared memory: the forward plan ends with the
// radix the inverse plan starts with, so each thread keeps exactly the
// values its first inverse pass needs in registers (F).
//
// Column 0 carries two real-row spectra (kx = 0 and kx = n/2): with
// P = FA + i FB its column FFT, the kernel products recombine as
//   P(ky) alpha(ky) + conj P(-ky) beta(ky),
// alpha/beta = (K(.,0) +- K(.,n/2))/2 (prepared by k_pack_kernel); P(-ky)
// lives in another thread, so that tile swaps column 0 through W first.
// grid (M/TW, C), block CT.
// ---------------------------------------------------------------------------
// Returns false if a bounded wait timed out (the error word is set).  `bar`
// is an initialised mbarrier owned by the caller and `phase` counts its
// completed phases, so one CTA can run many tiles back to back.
// KRE: the kernel spectra are real (point-symmetric kernels) and come from
// kre, the real parts of kspec: half the bytes per kernel tile, and each
// product is two multiplications instead of a complex one.
template <int LOGN, int V = 0, bool KRE = false>
__device__ __forceinline__ bool col_conv_body(const float2* __restrict__ rowspec,
                                              const float2* __restrict__ kspec,
                                              const float* __restrict__ kre,
                                              float2* __restrict__ U,
                                              const float2* __restrict__ tw,
                                              const KernelGroups& groups, int c, int kx0,
                                              float2* sm, uint64_t* barp, uint32_t& phase,
                                              int* err) {
    using G = Geo<LOGN, V>;
    constexpr int N = G::N, M = G::M, TW = G::TW, T = G::CT;
    const int cnt = groups.in_count[c];
    if (cnt == 0) return true;
    float2* W = sm;
    float2* KS = sm + G::KSOFF;
    const float* KR = reinterpret_cast<const float*>(KS);   // the real kernel tile (KRE)
    uint64_t& bar = *barp;
    const int base = groups.in_start[c];
    constexpr uint32_t kTileBytes = uint32_t(TW) * N * sizeof(float2);
    constexpr uint32_t kKernelBytes = KRE ? uint32_t(TW) * N * sizeof(float) : kTileBytes;
    auto issue_bytes = [&](const void* src, uint32_t bytes) {   // all threads call; thread 0 copies
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(&bar, bytes);
            bulk_g2s(KS, src, bytes, &bar);
        }
    };
    auto issue = [&](const float2* src) { issue_bytes(src, kTileBytes); };
    auto wait_tile = [&]() -> bool {
        const bool ok = mbar_wait(&bar, phase & 1, err);
        if (__syncthreads_or(!ok)) {
            // give the copy in flight one more bounded chance to land before
            // this CTA's shared memory is released
            mbar_wait(&bar, phase & 1, nullptr);
            return false;
        }
        ++phase;
        return true;
    };
    auto issue_kernel = [&](int gi) {
        const int k = groups.in_idx[base + gi];
        const size_t off = (size_t(k) * (M + 1) + kx0) * N;
        if constexpr (KRE) issue_bytes(kre + off, kKernelBytes);
        else issue_bytes(kspec + off, kKernelBytes);
    };

    issue(rowspec + (size_t(c) * M + kx0) * N);
    if (!wait_tile()) return false;

    // forward plan: greedy (variants 0-2) or remainder first (COL_SWAP);
    // the inverse plan is the other one
    constexpr bool FREM = G::COL_SWAP;
    const float2* tw_fwd = tw + (FREM ? G::TW_COL_INV : G::TW_COL_FWD);
    const float2* tw_inv = tw + (FREM ? G::TW_COL_FWD : G::TW_COL_INV);
    constexpr int RL = plan_last_radix(N, FREM);
    static_assert(PassRadix<N, 1, !FREM>::R == RL,
                  "the inverse must start with the radix the forward ends with");
    constexpr int JL = N / RL;
    constexpr int IPTL = (TW * JL + T - 1) / T;
    float2 F[IPTL][RL];
    auto ld_in = [&](int s, int i, int, int) { return KS[s * N + i]; };
    SmemRows wrows{W, G::CP};
    auto keep = [&](int, int, float2 v, int it, int r) { F[it][r] = v; };
    // forward: the first pass reads the staging tile, the last one keeps its
    // values in registers (no load-store barriers)
    fft_with_hook<N, false, T, TW, FREM, 16, false, false, false>(
        ld_in, wrows, wrows, keep, tw_fwd, [&]() { issue_kernel(0); });

    for (int gi = 0; gi < cnt; ++gi) {
        if (!wait_tile()) return false;
        if (kx0 == 0) {   // publish column 0 for the conj P(-ky) reads
#pragma unroll
            for (int it = 0; it < IPTL; ++it) {
                const int item = threadIdx.x + it * T;
                if ((TW * JL) % T == 0 || item < TW * JL) {
                    if (item / JL == 0) {
#pragma unroll
                        for (int r = 0; r < RL; ++r) W[pidx(item % JL + r * JL)] = F[it][r];
                    }
                }
            }
            __syncthreads();
        }
        const int k = groups.in_idx[base + gi];
        const float2* kb = kspec + (size_t(k) * (M + 1) + M) * N;
        const float* kbr = KRE ? kre + (size_t(k) * (M + 1) + M) * N : nullptr;
        float2* dst = U + (size_t(k) * M + kx0) * N;
        auto gst = [&](int s, int i, float2 v, int, int) { dst[size_t(s) * N + i] = v; };
        // The inverse, in two forms chosen per CTA: the one holding column 0
        // (kx0 == 0, its sequence 0) recombines p alpha + conj P(-ky) beta,
        // reading another thread's P(-ky) from W, so its first pass keeps
        // the load-store barrier; every other CTA multiplies only, with no
        // per-value test and no barrier there.  The last pass writes global
        // memory.
        auto inverse = [&](auto col0) {
            constexpr bool C0 = decltype(col0)::value;
            auto ld_mul = [&](int s, int i, int it, int r) {
                const float2 p = F[it][r];
                if constexpr (KRE) {
                    // the roundings are pinned (no contraction left to the
                    // compiler), so that every CTA shape gives the same bits
                    const float kv = KR[s * N + i];
                    if (C0 && s == 0) {   // p alpha + conj P(-ky) beta
                        const float2 pm = cconj(W[pidx((N - i) & (N - 1))]);
                        const float b = __ldg(&kbr[i]);
                        return make_float2(__fmaf_rn(p.x, kv, __fmul_rn(pm.x, b)),
                                           __fmaf_rn(p.y, kv, __fmul_rn(pm.y, b)));
                    }
                    return make_float2(__fmul_rn(p.x, kv), __fmul_rn(p.y, kv));
                } else {
                    const float2 kv = KS[s * N + i];
                    if (C0 && s == 0) {
                        const float2 pm = cconj(W[pidx((N - i) & (N - 1))]);
                        return cadd(cmul(p, kv), cmul(pm, __ldg(&kb[i])));
                    }
                    return cmul(p, kv);
                }
            };
            fft_with_hook<N, true, T, TW, !FREM, 16, false, C0, false>(
                ld_mul, wrows, wrows, gst, tw_inv, [&]() {
                if (gi + 1 < cnt) issue_kernel(gi + 1);
            });
        };
        if (kx0 == 0)
            inverse(std::true_type{});
        else
            inverse(std::false_type{});
    }
    return true;
}

template <int LOGN, int V = 0, bool KRE = false>
__global__ void __launch_bounds__(Geo<LOGN, V>::CT, Geo<LOGN, V>::COL_MINB)
    k_col_conv(const float2* __restrict__ rowspec, const float2* __restrict__ kspec,
               const float* __restrict__ kre, float2* __restrict__ U,
               const float2* __restrict__ tw, const __grid_constant__ KernelGroups groups,
               int* err, int cbase) {
    extern __shared__ __align__(128) float2 sm_col[];
    __shared__ __align__(8) uint64_t bar;
    pdl_wait();
    pdl_launch_dependents();
    const int c = blockIdx.y + cbase;
    if (groups.in_count[c] == 0) return;
    init_tile_barrier(&bar);
    uint32_t phase = 0;
    col_conv_body<LOGN, V, KRE>(rowspec, kspec, kre, U, tw, groups, c,
                                blockIdx.x * Geo<LOGN, V>::TW, sm_col, &bar, phase, err);
}

// ---------------------------------------------------------------------------
// Inverse row pass + growth, one output channel per CTA: for every kernel k
// with c1[k] == c (in increasing k, as mcl_growth_main accumulates,
// compute_1024.wgsl:313-320): C2R of the rows of U[k], then
//   u = value (the 1/n^2 of growth.rs:87 is folded into kspec),
//   g = 2 exp(-(u-mu)^2 / (2 sigma^2)) - 1,  acc += w g;
// then A[c] = exp(temp * acc) (diffusion.rs:58-66 applies temp inside exp).
// The exponential of the bump is ex2.approx (a few ulp, like expf) on a
// host-folded scale c2 = -log2(e) / (2 sigma^2); so is A, as
// 2^(temp log2(e) acc - temp log2(e) sum(w)) with one fma for the argument.
// C2R: Z[m] = E + i O, E = X[m] + conj X[M-m], O = (X[m] - conj X[M-m]) W_N^-m,
// z = IFFT_M(Z) = (x[2j], x[2j+1]).
// The tile of U[k] a CTA needs (RB values of y for every kx; U is kx-major)
// arrives by 2-D tensor copies (TMA): the transpose happens in the copy
// engine, the tile lands kx-major (element (kx, s) at kx * RB + s) and an
// mbarrier tracks it.  The next kernel's tile is issued into the same
// landing tile as soon as the first FFT pass has read it, and lands while
// the remaining passes and the growth run.  The FFT runs with the row
// index fastest (SFAST), so a warp's first-pass reads from the landing tile
// are contiguous and its exchanges through the padded work rows stay free
// of bank conflicts.  `umap` is encode_u_map's map of U (kernel parameter
// space, or global memory with `umap_global`).
// Returns false if a bounded wait timed out (the error word is set).  `bar`
// is an initialised mbarrier owned by the caller and `phase` counts its
// completed phases, so one CTA can run many tiles back to back.
// grid (N/RB, C), block RT.
// ---------------------------------------------------------------------------
template <int LOGN, int V = 0, bool DBG = false>
__device__ __forceinline__ bool row_c2r_growth_body(const CUtensorMap* umap, bool umap_global,
                                                    float* __restrict__ A,
                                                    const float2* __restrict__ tw,
                                                    const KernelGroups& groups,
                                                    const GrowthParams& gp, float temp,
                                                    float* __restrict__ udbg, float udbg_scale,
                                                    int c, int y0, float2* sm, uint64_t* barp,
                                                    uint32_t& phase, int* err) {
    using G = Geo<LOGN, V>;
    constexpr int M = G::M, RB = G::RB;
    constexpr int RL = last_radix(M, G::ROW_MR);
    constexpr int JL = M / RL;
    constexpr int ITEMS = RB * JL;
    constexpr int IPT = (ITEMS + G::RT - 1) / G::RT;
    constexpr uint32_t kTileBytes = uint32_t(G::C2R_TILE) * sizeof(float2);
    static_assert(G::RT % RB == 0, "a thread keeps one row in every pass");
    const int cnt = groups.out_count[c], base = groups.out_start[c];
    float2* land = sm + G::C2R_LAND;
    uint64_t& bar = *barp;
    if (umap_global && threadIdx.x == 0) tensormap_acquire(umap);

    auto issue = [&](int gi) {   // all threads call; thread 0 copies
        const int k = groups.out_idx[base + gi];
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(&bar, kTileBytes);
#pragma unroll
            for (int q = 0; q < M / G::UBOX; ++q)
                tensor2d_g2s(land + q * G::UBOX * RB, umap, 2 * y0, k * M + q * G::UBOX, &bar);
        }
    };
    auto wait_tile = [&]() -> bool {
        const bool ok = mbar_wait(&bar, phase & 1u, err);
        if (__syncthreads_or(!ok)) {
            // give the copy in flight one more bounded chance to land before
            // this CTA's shared memory is released
            mbar_wait(&bar, phase & 1u, nullptr);
            return false;
        }
        ++phase;
        return true;
    };

    float2 acc[IPT][RL];
#pragma unroll
    for (int it = 0; it < IPT; ++it)
#pragma unroll
        for (int r = 0; r < RL; ++r) acc[it][r] = make_float2(0.f, 0.f);

    // this thread's row: the same in every pass (RT is a multiple of RB)
    const int srow = threadIdx.x % RB;
    SmemRows rows{sm, G::RP};
    if (cnt > 0) issue(0);
    for (int gi = 0; gi < cnt; ++gi) {
        if (!wait_tile()) return false;
        const float2* lt = land + srow;   // lt[kx * RB]
        // m = j + q (M / R): m = 0 only in slot q = 0 (compile-time)
        auto ld0 = [&](int, int m, int, int q) -> float2 {
            if (q == 0 && m == 0) {
                const float2 x = lt[0];
                return make_float2(x.x + x.y, x.x - x.y);
            }
            const float2 a = lt[m * RB];
            const float2 b = cconj(lt[(M - m) * RB]);
            const float2 E = cadd(a, b);
            const float2 O = cmulc(csub(a, b), __ldg(&tw[m]));
            return make_float2(E.x - O.y, E.y + O.x);
        };
        const int k = groups.out_idx[base + gi];
        const float mu = gp.mu[k], c2 = gp.c2[k], w2 = gp.w2[k];
        float* ud = DBG ? udbg + (size_t(k) * G::N + y0) * G::N : nullptr;
        // w G = w (2 e - 1) with e = exp(-(u-mu)^2 / (2 sigma^2)) = 2^(d^2 c2):
        // accumulate 2 w e here, subtract sum(w) once per channel below.
        auto gst = [&](int s, int i, float2 v, int it, int r) {
            const float dx = v.x - mu, dy = v.y - mu;
            acc[it][r].x = fmaf(w2, ex2_approx(dx * dx * c2), acc[it][r].x);
            acc[it][r].y = fmaf(w2, ex2_approx(dy * dy * c2), acc[it][r].y);
            if constexpr (DBG)
                reinterpret_cast<float2*>(ud + size_t(s) * G::N)[i] =
                    make_float2(v.x * udbg_scale, v.y * udbg_scale);
        };
        // the first pass reads the landing tile and the last one keeps its
        // values in registers: neither needs its load-store barrier
        fft_with_hook<M, true, G::RT, RB, false, G::ROW_MR, true, false, false>(
            ld0, rows, rows, gst, tw + G::TW_ROW, [&]() {
                if (gi + 1 < cnt) issue(gi + 1);   // the first pass has read the tile
            });
    }

    float* Ac = A + (size_t(c) * G::N + y0) * G::N;
    const float tl = temp * 1.44269504088896341f;   // temp log2(e)
    const float toff = -tl * gp.wsum[c];
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        const int item = threadIdx.x + it * G::RT;
        if (ITEMS % G::RT == 0 || item < ITEMS) {
            int s, j;
            item_pos<RB, JL, true>(item, s, j);
#pragma unroll
            for (int r = 0; r < RL; ++r) {
                const int i = j + r * JL;
                reinterpret_cast<float2*>(Ac + size_t(s) * G::N)[i] =
                    make_float2(ex2_approx(fmaf(tl, acc[it][r].x, toff)),
                                ex2_approx(fmaf(tl, acc[it][r].y, toff)));
            }
        }
    }
    return true;
}

// The inverse row pass + growth of variant V on the RB rows from y0
// (C2RShape).  DBG: also write each kernel's u (scaled by udbg_scale) to
// udbg, for the debug read of the convolution buffer; the step's own
// kernels are built without it, so the per-value store costs them nothing.
template <int LOGN, int V, bool DBG = false>
__device__ __forceinline__ bool row_c2r_growth_variant(
    const CUtensorMap* umap, bool umap_global, float* __restrict__ A,
    const float2* __restrict__ tw, const KernelGroups& groups, const GrowthParams& gp, float temp,
    float* __restrict__ udbg, float udbg_scale, int c, int y0, float2* sm, uint64_t* barp,
    uint32_t& phase, int* err) {
    if constexpr (C2RShape<LOGN, V>::PAIR)
        return pair_c2r_growth_body<typename C2RShape<LOGN, V>::P, DBG>(
            umap, umap_global, A, tw, groups, gp, temp, udbg, udbg_scale, c, y0, sm, barp, phase,
            err);
    else
        return row_c2r_growth_body<LOGN, V, DBG>(umap, umap_global, A, tw, groups, gp, temp,
                                                 udbg, udbg_scale, c, y0, sm, barp, phase, err);
}

template <int LOGN, int V = 0, bool DBG = false>
__global__ void __launch_bounds__(C2RShape<LOGN, V>::RT, C2RShape<LOGN, V>::MINB)
    k_row_c2r_growth(const __grid_constant__ CUtensorMap umap, float* __restrict__ A,
                     const float2* __restrict__ tw, const __grid_constant__ KernelGroups groups,
                     const GrowthParams* __restrict__ gp, float temp, float* __restrict__ udbg,
                     float udbg_scale, int* err, int cbase) {
    extern __shared__ __align__(128) float2 sm_c2r[];
    __shared__ __align__(8) uint64_t bar;
    pdl_wait();
    pdl_launch_dependents();
    init_tile_barrier(&bar);
    uint32_t phase = 0;
    row_c2r_growth_variant<LOGN, V, DBG>(&umap, false, A, tw, groups, *gp, temp, udbg, udbg_scale,
                                    blockIdx.y + cbase, blockIdx.x * C2RShape<LOGN, V>::RB,
                                    sm_c2r, &bar, phase, err);
}

// ---------------------------------------------------------------------------
// Diffusion: Z = toroidal 3x3 sum of A, new = A * (3x3 sum of state / Z)
// (example.rs:272-303, compute_1024.wgsl:341-413).  One channel tile per
// CTA; A is read with a 2-pixel halo and the state with a 1-pixel halo, so
// both passes and the state copy of mod.rs:377-383 collapse into one kernel
// writing x_out.
//
// Mass conservation needs Z to be the exact sum of the nine A values: a
// rounded f32 sum is off by the same relative amount wherever A is constant
// (G = -1 for every kernel over a whole region), which drifts the total mass
// by ~1e-8 per step.  Each A is split into a 12-bit head and an exact tail;
// sums of up to nine heads are exact in f32 as long as the nine values lie
// within a factor 2^8 of each other, and the tails are summed in f32
// (relative weight 2^-12), so zh + zl is Z to ~1e-11.  q = x / Z comes from a
// reciprocal refined with the exact remainder, i.e. ~correctly rounded.
// grid (N/TX, N/TY, C), DiffGeo2::THREADS threads.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float head12(float a) {
    return __int_as_float(__float_as_int(a) & 0xFFFFF000);
}

// Horizontal 3-sums come from shared memory, vertical ones are carried in
// registers down a column: NSEG segments of rows per tile; in the Z phase one
// thread owns one of the TX+2 halo columns of a segment, in the output phase
// one of the TX columns.  Every sum keeps a fixed order ((a + b) + c, heads
// and tails apart), so all tile shapes give the same bits.  The A tile is read with 16-byte loads (a 4-pixel side
// halo keeps them aligned; the toroidal wrap stays aligned because n is a
// multiple of 4).
template <int LOGN, int V = 0>
struct DiffGeo2 {
    using G = Geo<LOGN, V>;
    static constexpr int N = G::N, TX = G::TX, TY = G::TY;
    static constexpr int NSEG = 4;
    static constexpr int AS = TX + 8, AH = TY + 4, HW = TX + 2, QH = TY + 2;
    static constexpr int ZR = (QH + NSEG - 1) / NSEG;   // Z rows per segment, at most
    static constexpr int OR = TY / NSEG;                // output rows per segment
    static constexpr int THREADS = ((HW * NSEG + 31) / 32) * 32;
    static constexpr int V4 = AS / 4;          // 16-byte loads per A row
    static constexpr int LR = THREADS / V4;    // A rows per sweep of the block
    static constexpr int SWEEPS = (AH + LR - 1) / LR;
    static constexpr size_t SMEM = size_t(2 * AH * AS + QH * HW) * sizeof(float);
    static_assert(TY % NSEG == 0 && TX % 4 == 0, "tile shape");
};

template <int LOGN, int V = 0>
__device__ __forceinline__ void diffusion2_body(const float* __restrict__ A,
                                                const float* __restrict__ x,
                                                float* __restrict__ out, int c, int x0, int y0,
                                                float* smf, unsigned char* levels) {
    using D = DiffGeo2<LOGN, V>;
    constexpr int N = D::N, TX = D::TX, AS = D::AS, AH = D::AH, HW = D::HW, QH = D::QH;
    constexpr int MASK = N * N - 1;            // row offsets wrap as (row * N) & MASK
    float* sAh = smf;                  // [AH][AS]: row a <-> y0 + a - 2, column j <-> x0 - 4 + j
    float* sAl = smf + AH * AS;
    float* sQ = smf + 2 * AH * AS;     // [QH][HW]: row b <-> y0 + b - 1, column q <-> x0 - 1 + q
    const float* Ac = A + size_t(c) * N * N;
    const float* xc = x + size_t(c) * N * N;
    const int t = threadIdx.x;

    // this thread's Z column and rows, and the state there (loaded first)
    const bool zthr = t < HW * D::NSEG;
    const int zq = t % HW, zseg = t / HW;
    const int zr0 = zseg * QH / D::NSEG, zn = (zseg + 1) * QH / D::NSEG - zr0;
    float xv[D::ZR];
    if (zthr) {
        const float* xcol = xc + ((x0 + zq - 1) & (N - 1));
        const int base = (y0 + zr0 - 1) * N;
#pragma unroll
        for (int i = 0; i < D::ZR; ++i)
            if (i < zn) xv[i] = __ldg(xcol + ((base + i * N) & MASK));
    }
    // the A tile, split into 12-bit heads and exact tails
    if (t < D::LR * D::V4) {
        const int v = t % D::V4, r0 = t / D::V4;
        const float* acol = Ac + ((x0 - 4 + 4 * v) & (N - 1));
        const int base = (y0 + r0 - 2) * N;
        float4 av[D::SWEEPS];
#pragma unroll
        for (int i = 0; i < D::SWEEPS; ++i)
            if (r0 + i * D::LR < AH)
                av[i] = __ldg(reinterpret_cast<const float4*>(acol + ((base + i * D::LR * N) & MASK)));
#pragma unroll
        for (int i = 0; i < D::SWEEPS; ++i) {
            if (r0 + i * D::LR < AH) {
                const float4 a = av[i];
                const float4 h = make_float4(head12(a.x), head12(a.y), head12(a.z), head12(a.w));
                const int o = (r0 + i * D::LR) * AS + 4 * v;
                *reinterpret_cast<float4*>(sAh + o) = h;
                *reinterpret_cast<float4*>(sAl + o) =
                    make_float4(a.x - h.x, a.y - h.y, a.z - h.z, a.w - h.w);
            }
        }
    }
    __syncthreads();

    // Z = zh + zl down this thread's column, then q = x / Z
    if (zthr) {
        const float* ph = sAh + zr0 * AS + zq + 2;   // A columns x0 - 2 + zq .. x0 + zq
        const float* pl = sAl + zr0 * AS + zq + 2;
        float* pq = sQ + zr0 * HW + zq;
        float h0 = ph[0] + ph[1] + ph[2], l0 = pl[0] + pl[1] + pl[2];
        float h1 = ph[AS] + ph[AS + 1] + ph[AS + 2], l1 = pl[AS] + pl[AS + 1] + pl[AS + 2];
#pragma unroll
        for (int i = 0; i < D::ZR; ++i) {
            if (i >= zn) break;
            const int o = (i + 2) * AS;
            const float h2 = ph[o] + ph[o + 1] + ph[o + 2];
            const float l2 = pl[o] + pl[o + 1] + pl[o + 2];
            const float zh = h0 + h1 + h2;
            const float zt = l0 + l1 + l2;
            pq[i * HW] = div_head_tail(xv[i], zh, zt);
            h0 = h1;
            l0 = l1;
            h1 = h2;
            l1 = l2;
        }
    }
    __syncthreads();

    // new = A * (3x3 sum of q), down this thread's output column
    if (t < TX * D::NSEG) {
        const int fq = t % TX, r0 = (t / TX) * D::OR;
        const float* pq = sQ + r0 * HW + fq;
        const float* pa = sAh + (r0 + 2) * AS + fq + 4;
        const float* pb = sAl + (r0 + 2) * AS + fq + 4;
        const int p0 = (y0 + r0) * N + x0 + fq;
        float* oc = out + size_t(c) * N * N + p0;
        unsigned char* lv = levels ? levels + size_t(c) * N * N + p0 : nullptr;
        const bool draw = levels != nullptr && c < 3;
        float s0 = pq[0] + pq[1] + pq[2];
        float s1 = pq[HW] + pq[HW + 1] + pq[HW + 2];
#pragma unroll
        for (int i = 0; i < D::OR; ++i) {
            const int o = (i + 2) * HW;
            const float s2 = pq[o] + pq[o + 1] + pq[o + 2];
            const float a = pa[i * AS] + pb[i * AS];
            const float v = a * ((s0 + s1) + s2);
            oc[i * N] = v;
            if (draw) lv[i * N] = render_level_byte(v);
            s0 = s1;
            s1 = s2;
        }
    }
}

// The same arithmetic with two adjacent columns per thread: four consecutive
// values (two 8-byte shared loads) give the horizontal 3-sums of both, so
// the shared-memory pipe sees a third of the loads.  Output threads own 4
// rows of a column pair; Z threads ZR rows of a halo-column pair.
template <int LOGN, int V = 0>
struct DiffGeoPair {
    using G = Geo<LOGN, V>;
    static constexpr int N = G::N, TX = G::TX, TY = G::TY;
    static constexpr int AS = TX + 8, AH = TY + 4, QH = TY + 2, QS = TX + 4;
    static constexpr int OG = TX / 2;                   // output column pairs
    static constexpr int ZG = (TX + 2 + 1) / 2;         // halo column pairs
    static constexpr int OR = 4;                        // output rows per thread
    static constexpr int THREADS = ((OG * (TY / OR) + 31) / 32) * 32;
    static constexpr int NSZ = THREADS / ZG;            // Z row segments
    static constexpr int ZR = (QH + NSZ - 1) / NSZ;     // Z rows per segment, at most
    static constexpr int V4 = AS / 4;
    static constexpr int LR = THREADS / V4;
    static constexpr int SWEEPS = (AH + LR - 1) / LR;
    static constexpr size_t SMEM = size_t(2 * AH * AS + QH * QS) * sizeof(float);
    static_assert(TY % OR == 0 && TX % 4 == 0 && NSZ >= 1 && LR >= 1, "tile shape");
    static_assert(2 * ZG + 4 <= AS && 2 * ZG <= QS, "pairs stay inside the tiles");
};

template <int LOGN, int V = 0>
__device__ __forceinline__ void diffusion_pair_body(const float* __restrict__ A,
                                                    const float* __restrict__ x,
                                                    float* __restrict__ out, int c, int x0,
                                                    int y0, float* smf, unsigned char* levels) {
    using D = DiffGeoPair<LOGN, V>;
    constexpr int N = D::N, AS = D::AS, AH = D::AH, QH = D::QH, QS = D::QS;
    constexpr int MASK = N * N - 1;
    float* sAh = smf;                  // [AH][AS]: row a <-> y0 + a - 2, column j <-> x0 - 4 + j
    float* sAl = smf + AH * AS;
    float* sQ = smf + 2 * AH * AS;     // [QH][QS]: row b <-> y0 + b - 1, column q <-> x0 - 1 + q
    const float* Ac = A + size_t(c) * N * N;
    const float* xc = x + size_t(c) * N * N;
    const int t = threadIdx.x;

    const int zu = t % D::ZG, zs = t / D::ZG;
    const int zr0 = zs * D::ZR;
    const int zn = zs < D::NSZ ? min(D::ZR, QH - zr0) : 0;
    float xv[D::ZR][2];
    if (zn > 0) {
        const float* xa = xc + ((x0 + 2 * zu - 1) & (N - 1));
        const float* xb = xc + ((x0 + 2 * zu) & (N - 1));
        const int base = (y0 + zr0 - 1) * N;
#pragma unroll
        for (int i = 0; i < D::ZR; ++i) {
            if (i < zn) {
                const int o = (base + i * N) & MASK;
                xv[i][0] = __ldg(xa + o);
                xv[i][1] = __ldg(xb + o);
            }
        }
    }
    if (t < D::LR * D::V4) {
        const int v = t % D::V4, r0 = t / D::V4;
        const float* acol = Ac + ((x0 - 4 + 4 * v) & (N - 1));
        const int base = (y0 + r0 - 2) * N;
        float4 av[D::SWEEPS];
#pragma unroll
        for (int i = 0; i < D::SWEEPS; ++i)
            if (r0 + i * D::LR < AH)
                av[i] = __ldg(reinterpret_cast<const float4*>(acol + ((base + i * D::LR * N) & MASK)));
#pragma unroll
        for (int i = 0; i < D::SWEEPS; ++i) {
            if (r0 + i * D::LR < AH) {
                const float4 a = av[i];
                const float4 h = make_float4(head12(a.x), head12(a.y), head12(a.z), head12(a.w));
                const int o = (r0 + i * D::LR) * AS + 4 * v;
                *reinterpret_cast<float4*>(sAh + o) = h;
                *reinterpret_cast<float4*>(sAl + o) =
                    make_float4(a.x - h.x, a.y - h.y, a.z - h.z, a.w - h.w);
            }
        }
    }
    __syncthreads();

    // o[m] = (p[m] + p[m+1]) + p[m+2], m < 2, from two 8-byte loads
    auto sum3x2 = [](const float* p, float& o0, float& o1) {
        const float2 a = *reinterpret_cast<const float2*>(p);
        const float2 b = *reinterpret_cast<const float2*>(p + 2);
        o0 = a.x + a.y + b.x;
        o1 = a.y + b.x + b.y;
    };
    if (zn > 0) {
        const float* ph = sAh + zr0 * AS + 2 * zu + 2;   // A columns x0 - 2 + 2 zu ..
        const float* pl = sAl + zr0 * AS + 2 * zu + 2;
        float* pq = sQ + zr0 * QS + 2 * zu;
        float h0[2], l0[2], h1[2], l1[2];
        sum3x2(ph, h0[0], h0[1]);
        sum3x2(pl, l0[0], l0[1]);
        sum3x2(ph + AS, h1[0], h1[1]);
        sum3x2(pl + AS, l1[0], l1[1]);
#pragma unroll
        for (int i = 0; i < D::ZR; ++i) {
            if (i >= zn) break;
            float h2[2], l2[2], q[2];
            sum3x2(ph + (i + 2) * AS, h2[0], h2[1]);
            sum3x2(pl + (i + 2) * AS, l2[0], l2[1]);
#pragma unroll
            for (int m = 0; m < 2; ++m) {
                const float zh = h0[m] + h1[m] + h2[m];
                const float zt = l0[m] + l1[m] + l2[m];
                q[m] = div_head_tail(xv[i][m], zh, zt);
                h0[m] = h1[m];
                l0[m] = l1[m];
                h1[m] = h2[m];
                l1[m] = l2[m];
            }
            *reinterpret_cast<float2*>(pq + i * QS) = make_float2(q[0], q[1]);
        }
    }
    __syncthreads();

    const int ou = t % D::OG, os = t / D::OG;
    if (os < D::TY / D::OR) {
        const int r0 = os * D::OR;
        const float* pq = sQ + r0 * QS + 2 * ou;
        const float* pa = sAh + (r0 + 2) * AS + 2 * ou + 4;
        const float* pb = sAl + (r0 + 2) * AS + 2 * ou + 4;
        const int p0 = (y0 + r0) * N + x0 + 2 * ou;
        float* oc = out + size_t(c) * N * N + p0;
        unsigned char* lv = levels ? levels + size_t(c) * N * N + p0 : nullptr;
        const bool draw = levels != nullptr && c < 3;
        float s0[2], s1[2];
        sum3x2(pq, s0[0], s0[1]);
        sum3x2(pq + QS, s1[0], s1[1]);
#pragma unroll
        for (int i = 0; i < D::OR; ++i) {
            float s2[2];
            sum3x2(pq + (i + 2) * QS, s2[0], s2[1]);
            const float2 ah = *reinterpret_cast<const float2*>(pa + i * AS);
            const float2 al = *reinterpret_cast<const float2*>(pb + i * AS);
            const float2 v = make_float2((ah.x + al.x) * ((s0[0] + s1[0]) + s2[0]),
                                         (ah.y + al.y) * ((s0[1] + s1[1]) + s2[1]));
            *reinterpret_cast<float2*>(oc + i * N) = v;
            if (draw)
                *reinterpret_cast<uchar2*>(lv + i * N) =
                    make_uchar2(render_level_byte(v.x), render_level_byte(v.y));
            s0[0] = s1[0];
            s0[1] = s1[1];
            s1[0] = s2[0];
            s1[1] = s2[1];
        }
    }
}

// The same arithmetic without shared memory: a thread owns 4 adjacent columns
// and walks down TYR rows.  Per row it loads A at its columns +-2 and the
// state at +-1 with three 16-byte loads each (the side ones overlap its
// neighbours' and hit L1), splits A into heads and tails, and keeps the
// horizontal 3-sums of the last three rows (heads, tails, q) in registers;
// the vertical sums come from those slots.  Every sum keeps the order of
// diffusion2_body, so the bits are the same.  A CTA is RS strips of TX/4
// threads: TX columns by RS * TYR rows.  Strips of STRIP rows (variant 1:
// 16, variant 3: 8; fewer at small sides) trade the four halo rows each
// strip re-reads against twice the CTAs and half the unrolled body.
template <int LOGN, int STRIP = 16>
struct DiffGeoReg {
    static constexpr int N = 1 << LOGN;
    static constexpr int TX = N < 128 ? N : 128;
    static constexpr int TYR = N / 4 < STRIP ? N / 4 : STRIP;
    static constexpr int RS = 4;
    static constexpr int TY = RS * TYR;
    static constexpr int THREADS = TX / 4 * RS;
    static_assert(TX % 4 == 0 && N % TY == 0, "tile shape");
};

template <int LOGN, int STRIP>
__device__ __forceinline__ void diffusion_reg_body(const float* __restrict__ A,
                                                   const float* __restrict__ x,
                                                   float* __restrict__ out, int c, int x0,
                                                   int y0, unsigned char* levels) {
    using D = DiffGeoReg<LOGN, STRIP>;
    constexpr int N = D::N, MASK = N * N - 1;
    const int col = x0 + 4 * (threadIdx.x % (D::TX / 4));   // first of this thread's columns
    const int ys = y0 + (threadIdx.x / (D::TX / 4)) * D::TYR;
    const float* Ac = A + size_t(c) * N * N;
    const float* xc = x + size_t(c) * N * N;
    float* oc = out + size_t(c) * N * N;
    const int cl = (col - 4) & (N - 1), cr = (col + 4) & (N - 1);
    unsigned char* lv = levels ? levels + size_t(c) * N * N : nullptr;
    const bool draw = levels != nullptr && c < 3;
    // columns col-4 .. col+7 of row y (toroidal)
    auto ld3 = [&](const float* p, int y, float4& l, float4& m, float4& r) {
        const float* row = p + ((y * N) & MASK);
        l = __ldg(reinterpret_cast<const float4*>(row + cl));
        m = __ldg(reinterpret_cast<const float4*>(row + col));
        r = __ldg(reinterpret_cast<const float4*>(row + cr));
    };

    // slot k % 3 holds the sums of iteration k: heads / tails over Z columns
    // col-1 .. col+4 (hs, ls), q over output columns col .. col+3 (qs), and
    // A at the output columns (am)
    float hs[3][6], ls[3][6], qs[3][4];
    float4 am[3];
    // the loads of the next row are issued before this row's arithmetic
    float4 nal, nac, nar;
    float4 nxl = make_float4(0.f, 0.f, 0.f, 0.f), nxm = nxl, nxr = nxl;
    ld3(Ac, ys - 2, nal, nac, nar);
#pragma unroll
    for (int k = 0; k < D::TYR + 4; ++k) {
        const int ya = ys - 2 + k;   // A row of this iteration
        const int b = k % 3;
        const float4 al = nal, ac = nac, ar = nar;
        const float4 xl = nxl, xm = nxm, xr = nxr;   // state row ya - 1 (k >= 2)
        if (k + 1 < D::TYR + 4) ld3(Ac, ya + 1, nal, nac, nar);
        if (k + 1 >= 2 && k + 1 < D::TYR + 4) ld3(xc, ya, nxl, nxm, nxr);
        {
            const float a[8] = {al.z, al.w, ac.x, ac.y, ac.z, ac.w, ar.x, ar.y};
            float H[8], L[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                H[i] = head12(a[i]);
                L[i] = a[i] - H[i];
            }
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                hs[b][j] = H[j] + H[j + 1] + H[j + 2];
                ls[b][j] = L[j] + L[j + 1] + L[j + 2];
            }
            am[b] = ac;
        }
        if (k >= 2) {   // Z and q at row ya - 1
            const int t0 = (k - 2) % 3, t1 = (k - 1) % 3;
            const float xv[6] = {xl.w, xm.x, xm.y, xm.z, xm.w, xr.x};
            float q[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                const float zh = hs[t0][j] + hs[t1][j] + hs[b][j];
                const float zt = ls[t0][j] + ls[t1][j] + ls[b][j];
                q[j] = div_head_tail(xv[j], zh, zt);
            }
#pragma unroll
            for (int o = 0; o < 4; ++o) qs[b][o] = q[o] + q[o + 1] + q[o + 2];
        }
        if (k >= 4) {   // output row ya - 2
            const int s0 = (k - 2) % 3, s1 = (k - 1) % 3;
            const float4 a = am[s0];
            const float4 v = make_float4(a.x * ((qs[s0][0] + qs[s1][0]) + qs[b][0]),
                                         a.y * ((qs[s0][1] + qs[s1][1]) + qs[b][1]),
                                         a.z * ((qs[s0][2] + qs[s1][2]) + qs[b][2]),
                                         a.w * ((qs[s0][3] + qs[s1][3]) + qs[b][3]));
            const int p = (ya - 2) * N + col;
            *reinterpret_cast<float4*>(oc + p) = v;
            if (draw)
                *reinterpret_cast<uchar4*>(lv + p) =
                    make_uchar4(render_level_byte(v.x), render_level_byte(v.y),
                                render_level_byte(v.z), render_level_byte(v.w));
        }
    }
}

// The diffusion phase's variants: 0 the shared-memory tile body, 1 and 3
// the register body in 16- and 8-row strips, 2 the column-pair body.  All
// four give the same bits.  TX x TY is the tile of one CTA (one work item).
constexpr int kDiffVariants = 4;
template <int LOGN, int V, int KIND = (V == 1 || V == 3) ? 1 : (V == 2 ? 2 : 0)>
struct DiffTile;
template <int LOGN, int V>
struct DiffTile<LOGN, V, 1> {
    static constexpr bool REG = true, PAIR = false;
    static constexpr int STRIP = (V == 3) ? 8 : 16;
    using D = DiffGeoReg<LOGN, STRIP>;
    static constexpr int THREADS = D::THREADS, TX = D::TX, TY = D::TY;
    static constexpr size_t SMEM = 0;
};
template <int LOGN, int V>
struct DiffTile<LOGN, V, 2> {
    static constexpr bool REG = false, PAIR = true;
    using D = DiffGeoPair<LOGN, V>;
    static constexpr int THREADS = D::THREADS, TX = D::TX, TY = D::TY;
    static constexpr size_t SMEM = D::SMEM;
};
template <int LOGN, int V>
struct DiffTile<LOGN, V, 0> {
    static constexpr bool REG = false, PAIR = false;
    using D = DiffGeo2<LOGN, V>;
    static constexpr int THREADS = D::THREADS, TX = D::TX, TY = D::TY;
    static constexpr size_t SMEM = D::SMEM;
};

template <int LOGN, int V>
__device__ __forceinline__ void diffusion_tile(const float* __restrict__ A,
                                               const float* __restrict__ x,
                                               float* __restrict__ out, int c, int x0, int y0,
                                               float* smf, unsigned char* levels) {
    using T = DiffTile<LOGN, V>;
    if constexpr (T::REG)
        diffusion_reg_body<LOGN, T::STRIP>(A, x, out, c, x0, y0, levels);
    else if constexpr (T::PAIR)
        diffusion_pair_body<LOGN, V>(A, x, out, c, x0, y0, smf, levels);
    else
        diffusion2_body<LOGN, V>(A, x, out, c, x0, y0, smf, levels);
}

template <int LOGN, int V = 0>
__global__ void __launch_bounds__(DiffTile<LOGN, V>::THREADS)
    k_diffusion(const float* __restrict__ A, const float* __restrict__ x, float* __restrict__ out,
                int cbase, unsigned char* __restrict__ levels) {
    extern __shared__ __align__(128) float sm_diff[];
    pdl_wait();
    pdl_launch_dependents();
    diffusion_tile<LOGN, V>(A, x, out, blockIdx.z + cbase, blockIdx.x * DiffTile<LOGN, V>::TX,
                            blockIdx.y * DiffTile<LOGN, V>::TY, sm_diff, levels);
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
template <int LOGN, int V>
cudaError_t prepare_variant() {
    using G = Geo<LOGN, V>;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_row_r2c<LOGN, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(R2CShape<LOGN, V>::SMEM))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_row_c2r_growth<LOGN, V>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(C2RShape<LOGN, V>::SMEM))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_col_conv<LOGN, V, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(G::COL_SMEM))) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_col_conv<LOGN, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(G::COL_SMEM));
}

template <int LOGN>
cudaError_t prepare_c2r_debug() {
    return cudaFuncSetAttribute(k_row_c2r_growth<LOGN, 0, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(C2RShape<LOGN, 0>::SMEM));
}

template <int LOGN, int V>
cudaError_t prepare_diffusion() {
    return cudaFuncSetAttribute(k_diffusion<LOGN, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(DiffTile<LOGN, V>::SMEM));
}

template <int LOGN>
cudaError_t prepare_size() {
    cudaError_t e = prepare_variant<LOGN, 0>();
    if (e == cudaSuccess) e = prepare_variant<LOGN, 1>();
    if (e == cudaSuccess) e = prepare_variant<LOGN, 2>();
    if constexpr (LOGN >= kMinPairLogN) {
        if (e == cudaSuccess) e = prepare_variant<LOGN, 3>();
        if (e == cudaSuccess) e = prepare_variant<LOGN, 4>();
    }
    if (e == cudaSuccess) e = prepare_c2r_debug<LOGN>();
    if (e == cudaSuccess) e = prepare_diffusion<LOGN, 0>();
    if (e == cudaSuccess) e = prepare_diffusion<LOGN, 1>();
    if (e == cudaSuccess) e = prepare_diffusion<LOGN, 2>();
    if (e == cudaSuccess) e = prepare_diffusion<LOGN, 3>();
    return e;
}

// One phase for channels [c_lo, c_lo + nc) (r2c/col: the channels read;
// c2r/diffusion: the channels written) in variant V.  Every step kernel is
// launched with programmatic stream serialization (pdl_wait): within a
// stream, and within the step graphs captured from it, a kernel's CTAs are
// dispatched while the kernel before it drains.
template <class... KArgs, class... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, int threads, size_t smem,
                       cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <int LOGN, int V>
cudaError_t launch_r2c(const StepArgs& a, int c_lo, int nc, cudaStream_t st) {
    using R = R2CShape<LOGN, V>;
    constexpr int NB = (1 << LOGN) / R::RB;
    dim3 grid(NB, nc);
    if constexpr (R::STREAM) {   // persistent: the CTAs that fit at once
        int dev = 0, sms = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_row_r2c<LOGN, V>, R::RT,
                                                              R::SMEM);
        if (e != cudaSuccess) return e;
        const int ctas = (per_sm > 0 ? per_sm : 1) * sms;
        grid = dim3(NB * nc < ctas ? NB * nc : ctas, 1);
    }
    return launch_pdl(k_row_r2c<LOGN, V>, grid, R::RT, R::SMEM, st, a.x_in, a.rowspec, a.tw, c_lo,
                      nc, a.err);
}
template <int LOGN, int V>
cudaError_t launch_col(const StepArgs& a, int c_lo, int nc, cudaStream_t st) {
    using G = Geo<LOGN, V>;
    const dim3 grid(G::M / G::TW, nc);
    if (a.kre)
        return launch_pdl(k_col_conv<LOGN, V, true>, grid, G::CT, G::COL_SMEM, st, a.rowspec,
                          a.kspec, a.kre, a.U, a.tw, a.groups, a.err, c_lo);
    return launch_pdl(k_col_conv<LOGN, V>, grid, G::CT, G::COL_SMEM, st, a.rowspec, a.kspec,
                      static_cast<const float*>(nullptr), a.U, a.tw, a.groups, a.err, c_lo);
}
template <int LOGN, int V, bool DBG>
cudaError_t launch_c2r_shape(const StepArgs& a, int c_lo, int nc, cudaStream_t st) {
    using R = C2RShape<LOGN, V>;
    constexpr int N = 1 << LOGN;
    CUtensorMap umap;   // passed by value: a graph capture keeps its own copy
    const cudaError_t e = encode_u_map(&umap, a.U, N, a.K, R::RB);
    if (e != cudaSuccess) return e;
    return launch_pdl(k_row_c2r_growth<LOGN, V, DBG>, dim3(N / R::RB, nc), R::RT, R::SMEM, st,
                      umap, a.A, a.tw, a.groups, a.gp, a.temp, a.udbg, float(N) * float(N), a.err,
                      c_lo);
}
// The inverse row pass in variant V; with a debug buffer (a.udbg, the debug
// read of the convolution), variant 0's shape built with the debug store.
template <int LOGN, int V>
cudaError_t launch_c2r(const StepArgs& a, int c_lo, int nc, cudaStream_t st) {
    if (a.udbg) return launch_c2r_shape<LOGN, 0, true>(a, c_lo, nc, st);
    return launch_c2r_shape<LOGN, V, false>(a, c_lo, nc, st);
}
template <int LOGN, int V>
cudaError_t launch_diff(const StepArgs& a, int c_lo, int nc, cudaStream_t st) {
    constexpr int N = 1 << LOGN;
    using D = DiffTile<LOGN, V>;
    return launch_pdl(k_diffusion<LOGN, V>, dim3(N / D::TX, N / D::TY, nc), D::THREADS,
                      D::SMEM, st, a.A, a.x_in, a.x_out, c_lo, a.levels);
}

#define CG_VARIANT_SWITCH(v, FN, ...)            \
    switch (v) {                                  \
        case 1: FN<LOGN, 1>(__VA_ARGS__); break;  \
        case 2: FN<LOGN, 2>(__VA_ARGS__); break;  \
        default: FN<LOGN, 0>(__VA_ARGS__); break; \
    }

// The same over all five variants of the row and column phases (3 and 4
// exist from kMinPairLogN on; below it they fall back to variant 0, which
// the host never selects there).
#define CG_VARIANT_SWITCH5(v, FN, ...)                                      \
    if constexpr (LOGN >= kMinPairLogN) {                                   \
        switch (v) {                                                        \
            case 1: FN<LOGN, 1>(__VA_ARGS__); break;                        \
            case 2: FN<LOGN, 2>(__VA_ARGS__); break;                        \
            case 3: FN<LOGN, kMinPairLogN <= LOGN ? 3 : 0>(__VA_ARGS__); break; \
            case 4: FN<LOGN, kMinPairLogN <= LOGN ? 4 : 0>(__VA_ARGS__); break; \
            default: FN<LOGN, 0>(__VA_ARGS__); break;                       \
        }                                                                   \
    } else {                                                                \
        CG_VARIANT_SWITCH(v, FN, __VA_ARGS__)                               \
    }

// The diffusion phase's four variants (every size).
#define CG_DIFF_SWITCH(v, FN, ...)               \
    switch (v) {                                  \
        case 1: FN<LOGN, 1>(__VA_ARGS__); break;  \
        case 2: FN<LOGN, 2>(__VA_ARGS__); break;  \
        case 3: FN<LOGN, 3>(__VA_ARGS__); break;  \
        default: FN<LOGN, 0>(__VA_ARGS__); break; \
    }

// The given phases for channels [c_lo, c_hi), each in the variant a.var
// names.
template <int LOGN>
cudaError_t launch_step_range(const StepArgs& a, int phases, int c_lo, int c_hi,
                              cudaStream_t st) {
    const int nc = c_hi - c_lo;
    if (nc <= 0) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    if (phases & kPhaseRowFwd) { CG_VARIANT_SWITCH5(a.var.r2c, e = launch_r2c, a, c_lo, nc, st) }
    if (e != cudaSuccess) return e;
    if (phases & kPhaseColConv) { CG_VARIANT_SWITCH5(a.var.col, e = launch_col, a, c_lo, nc, st) }
    if (e != cudaSuccess) return e;
    if (phases & kPhaseGrowth) { CG_VARIANT_SWITCH5(a.var.c2r, e = launch_c2r, a, c_lo, nc, st) }
    if (e != cudaSuccess) return e;
    if (phases & kPhaseDiffusion) {
        CG_DIFF_SWITCH(a.var.diff, e = launch_diff, a, c_lo, nc, st)
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

template <int LOGN>
cudaError_t launch_step(const StepArgs& a, int phases, cudaStream_t st) {
    return launch_step_range<LOGN>(a, phases, 0, a.C, st);
}

template <int LOGN>
cudaError_t launch_step_channel(const StepArgs& a, int phases, int c, cudaStream_t st) {
    return launch_step_range<LOGN>(a, phases, c, c + 1, st);
}

template <int LOGN>
int twiddle_count() {
    return Geo<LOGN>::TW_TOTAL;
}

template <int LOGN>
cudaError_t launch_pack(const float2* full, float2* out, cudaStream_t st) {
    using G = Geo<LOGN>;
    const int total = G::M * G::N;
    k_pack_kernel<LOGN><<<(total + 255) / 256, 256, 0, st>>>(full, out);
    return cudaGetLastError();
}

}  // namespace cg

// Per-size operation table (needs builder.cuh included before expansion).
#define CG_DEFINE_SIZE_OPS(LOGN)                                                          \
    namespace cg {                                                                        \
    extern const SizeOps size_ops_l##LOGN;                                                \
    const SizeOps size_ops_l##LOGN = {launch_step<LOGN>,      launch_pack<LOGN>,          \
                                      prepare_size<LOGN>,     twiddle_count<LOGN>,        \
                                      launch_backward<LOGN>,  launch_kgrad_final<LOGN>,   \
                                      prepare_backward<LOGN>, launch_step_channel<LOGN>,  \
                                      prepare_builder<LOGN>,  launch_kspec_cols<LOGN>};   \
    }
