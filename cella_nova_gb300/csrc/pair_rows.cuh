// pair_rows.cuh — row passes that transform two real rows as one complex
// sequence of length n (the plan variants 3 and 4 of the row phases).
//
// The reference transforms every row of every channel and kernel as a full
// complex FFT (ml-rs/shaders/compute_1024.wgsl:112-218).  Variants 0-2 of
// this library run an n/2-point complex FFT per real row and split even and
// odd samples with a twiddle per output (k_row_r2c, k_row_c2r_growth).
// These variants use the other classic real-input scheme: rows r0 and r1 of
// a CTA form z = x_r0 + i x_r1, one n-point FFT transforms both, and the
// two half spectra separate with additions only:
//   X_r0[k] = (Z[k] + conj Z[n-k]),  X_r1[k] = -i (Z[k] - conj Z[n-k])
// (both twice the true spectra, the scale of variants 0-2), and the inverse
// forms Y[k] = X_r0[k] + i X_r1[k] over the whole circle from the half
// spectra (Y[n-k] = conj X_r0[k] + i conj X_r1[k]) so that the inverse
// n-point FFT returns x_r0 + i x_r1.  No twiddle is applied outside the FFT
// passes, and the inverse's first pass reads both rows of a kx with one
// 16-byte load from the kx-major landing tile.
//
// PairGeo<LOGN, T, MR>: T threads, plans of maximum radix MR (16: the column
// pass's greedy table; 8: its own table), and as many sequences per CTA (S,
// 2S rows) as give every thread one butterfly of a radix-MR pass.
#pragma once

namespace cg {

template <int LOGN, int T, int MR>
struct PairGeo {
    static constexpr int N = 1 << LOGN;
    static constexpr int M = N / 2;
    static constexpr int S = (T * MR / N) < 1 ? 1 : T * MR / N;
    static constexpr int PS = S;          // sequences per CTA
    static constexpr int RB = 2 * S;      // rows per CTA
    static constexpr int RT = T;
    static constexpr int ROW_MR = MR;
    // pitch of the padded work sequences: 16/S mod 16 float2, which keeps
    // the sequence-fastest accesses of a half-warp (16/S butterflies of each
    // of the S sequences) conflict-free
    static constexpr int WP = padded_len(N) + (S > 1 ? 16 / S : 0);
    static_assert(S <= 16, "sequences per CTA");
    // the inverse pass's landing tile (RB rows x M kx, kx-major) after the
    // work sequences, 128-byte aligned, filled by 2-D tensor copies of boxes
    // of UBOX kx
    static constexpr int LAND = (S * WP + 15) & ~15;
    static constexpr int TILE = RB * M;
    static constexpr int UBOX = M < 256 ? M : 256;
    static constexpr size_t R2C_SMEM = size_t(S) * WP * sizeof(float2);
    static constexpr size_t C2R_SMEM = (size_t(LAND) + TILE) * sizeof(float2);
    static_assert(C2R_SMEM <= 227 * 1024, "paired inverse row pass shared memory");
    static_assert((TILE * sizeof(float2)) % 128 == 0 && (RB * UBOX * sizeof(float2)) % 128 == 0,
                  "tensor-copy destination alignment");
    static_assert(N / MR >= 2 && (S * (N / MR)) % 32 == 0, "whole warps per pass");
    // the plan's twiddle table in the size's buffer
    static constexpr int TWOFF = MR == 16 ? Geo<LOGN>::TW_COL_FWD : Geo<LOGN>::TW_PAIR8;
    static constexpr bool SF = S > 1;     // sequence index fastest over the threads
};

// Row phases' shapes per variant: 0-2 are Geo's half-length row kernels,
// 3 and 4 the paired ones.
// The forward row pass of variants 0 and 1 is bound by the latency of its
// first pass's global loads: a register cap of 64 (MINB = 1024 / RT, no
// spills) lets a third more warps share an SM.  Variant 2 (STREAM) runs
// variant 1's tile in a persistent grid whose CTAs bring each block's rows
// into a staging tile with one bulk copy, the next block's while the
// current one is transformed (row_r2c_stream); STG is the staging tile's
// offset in float2 (128-byte aligned, after the work rows).
template <int LOGN, int V>
struct R2CShape {
    static constexpr bool PAIR = false, STREAM = false;
    using G = Geo<LOGN, V>;
    static constexpr int RT = G::RT, RB = G::RB, MINB = 1024 / G::RT;
    static constexpr size_t SMEM = G::R2C_SMEM;
};
template <int LOGN>
struct R2CShape<LOGN, 2> {
    static constexpr bool PAIR = false, STREAM = true;
    using G = Geo<LOGN, 1>;
    static constexpr int RT = G::RT, RB = G::RB, MINB = 3;
    static constexpr int STG = int((G::R2C_SMEM / sizeof(float2) + 15) & ~size_t(15));
    static constexpr uint32_t kBlockBytes = uint32_t(RB) * G::N * sizeof(float);
    static constexpr size_t SMEM = size_t(STG) * sizeof(float2) + kBlockBytes;
    static_assert(kBlockBytes % 16 == 0, "bulk-copy size");
};
template <int LOGN>
struct R2CShape<LOGN, 3> {
    static constexpr bool PAIR = true, STREAM = false;
    using P = PairGeo<LOGN, 256, 16>;
    static constexpr int RT = P::RT, RB = P::RB, MINB = 2;
    static constexpr size_t SMEM = P::R2C_SMEM;
};
template <int LOGN>
struct R2CShape<LOGN, 4> {
    static constexpr bool PAIR = true, STREAM = false;
    using P = PairGeo<LOGN, 512, 8>;
    static constexpr int RT = P::RT, RB = P::RB, MINB = 2;
    static constexpr size_t SMEM = P::R2C_SMEM;
};

template <int LOGN, int V>
struct C2RShape {
    static constexpr bool PAIR = false;
    using G = Geo<LOGN, V>;
    static constexpr int RT = G::RT, RB = G::RB, MINB = 512 / G::RT;
    static constexpr size_t SMEM = G::C2R_SMEM;
};
template <int LOGN>
struct C2RShape<LOGN, 3> {
    static constexpr bool PAIR = true;
    using P = PairGeo<LOGN, 128, 16>;
    static constexpr int RT = P::RT, RB = P::RB, MINB = 5;
    static constexpr size_t SMEM = P::C2R_SMEM;
};
template <int LOGN>
struct C2RShape<LOGN, 4> {
    static constexpr bool PAIR = true;
    using P = PairGeo<LOGN, 256, 8>;
    static constexpr int RT = P::RT, RB = P::RB, MINB = 4;
    static constexpr size_t SMEM = P::C2R_SMEM;
};

// ---------------------------------------------------------------------------
// Forward: RB = 2S state rows from y0 -> their packed half spectra, kx-major
// (the layout of r2c_finish: X[0] and X[M] real, packed in slot 0).
// ---------------------------------------------------------------------------
template <class P>
__device__ __forceinline__ void pair_r2c_body(const float* __restrict__ state,
                                              float2* __restrict__ rowspec,
                                              const float2* __restrict__ tw, int c, int y0,
                                              float2* sm) {
    constexpr int N = P::N, M = P::M, S = P::PS;
    const float* src = state + (size_t(c) * N + y0) * N;
    // z_s[i] = x_{2s}[i] + i x_{2s+1}[i]
    auto ld0 = [&](int s, int i, int, int) {
        const float* r = src + size_t(2 * s) * N + i;
        return make_float2(__ldg(r), __ldg(r + N));
    };
    SmemRows rows{sm, P::WP};
    // the first pass reads global memory: no load-store barrier; the last
    // pass writes the work sequences, read below after its barrier
    FftPasses<N, 1, false, P::RT, S, false, P::ROW_MR, P::SF, false, true>::run(
        ld0, rows, rows, rows, tw + P::TWOFF);
    // split: item (s, k), s fastest, so the S sequences' 16-byte stores of
    // one kx are adjacent (rows y0 .. y0 + 2S - 1 of that kx)
    float2* dst = rowspec + size_t(c) * M * N + y0;
    for (int item = threadIdx.x; item < S * M; item += P::RT) {
        const int s = item % S, k = item / S;
        const float2* z = sm + s * P::WP;
        float4 o;
        if (k == 0) {
            const float2 z0 = z[0], zm = z[pidx(M)];
            o = make_float4(2.f * z0.x, 2.f * zm.x, 2.f * z0.y, 2.f * zm.y);
        } else {
            const float2 a = z[pidx(k)], b = z[pidx(N - k)];
            o = make_float4(a.x + b.x, a.y - b.y, a.y + b.y, b.x - a.x);
        }
        *reinterpret_cast<float4*>(dst + size_t(k) * N + 2 * s) = o;
    }
}

// ---------------------------------------------------------------------------
// Inverse + growth: the rows y0 .. y0 + 2S - 1 of output channel c, for
// every kernel k with c1[k] == c in increasing k: the n-point inverse FFT of
// Y = X_r0 + i X_r1 gives u on both rows at once, then the bump, the
// weighted sum and A = exp(temp * .), as row_c2r_growth_body does.  The U
// tiles arrive by 2-D tensor copies into the landing tile (element (kx, row)
// at kx * RB + row), the next kernel's tile is issued as soon as the first
// pass has read the current one.  Returns false if a bounded wait timed out.
// ---------------------------------------------------------------------------
template <class P, bool DBG = false>
__device__ __forceinline__ bool pair_c2r_growth_body(const CUtensorMap* umap, bool umap_global,
                                                     float* __restrict__ A,
                                                     const float2* __restrict__ tw,
                                                     const KernelGroups& groups,
                                                     const GrowthParams& gp, float temp,
                                                     float* __restrict__ udbg, float udbg_scale,
                                                     int c, int y0, float2* sm, uint64_t* barp,
                                                     uint32_t& phase, int* err) {
    constexpr int N = P::N, M = P::M, S = P::PS, RB = P::RB, T = P::RT;
    constexpr int R1 = PassRadix<N, 1, false, P::ROW_MR>::R;
    constexpr int RL = last_radix(N, P::ROW_MR);
    constexpr int JL = N / RL;
    constexpr int ITEMS = S * JL;
    constexpr int IPT = (ITEMS + T - 1) / T;
    constexpr uint32_t kTileBytes = uint32_t(P::TILE) * sizeof(float2);
    static_assert(R1 >= 2 && N / R1 * (R1 / 2) == M, "the first pass splits at k = M");
    const int cnt = groups.out_count[c], base = groups.out_start[c];
    float2* land = sm + P::LAND;
    uint64_t& bar = *barp;
    if (umap_global && threadIdx.x == 0) tensormap_acquire(umap);

    auto issue = [&](int gi) {   // all threads call; thread 0 copies
        const int k = groups.out_idx[base + gi];
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(&bar, kTileBytes);
#pragma unroll
            for (int q = 0; q < M / P::UBOX; ++q)
                tensor2d_g2s(land + q * P::UBOX * RB, umap, 2 * y0, k * M + q * P::UBOX, &bar);
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

    SmemRows rows{sm, P::WP};
    const float4* lt = reinterpret_cast<const float4*>(land);   // (X_r0, X_r1) of sequence s at kx: lt[kx * S + s]
    if (cnt > 0) issue(0);
    for (int gi = 0; gi < cnt; ++gi) {
        if (!wait_tile()) return false;
        // Y[k], k = j + q (n / R1): q < R1/2 <=> k < M; k = 0 and k = M need
        // j = 0 and the slots q = 0 and q = R1/2 (compile-time after
        // unrolling), so only those two slots test j
        auto ld0 = [&](int s, int k, int, int q) -> float2 {
            if (q < R1 / 2) {
                const float4 t = lt[k * S + s];
                if (q == 0 && k == 0) return make_float2(t.x, t.z);   // X_r0[0], X_r1[0] real
                return make_float2(t.x - t.w, t.y + t.z);             // X_r0 + i X_r1
            }
            if (q == R1 / 2 && k == M) {
                const float4 t = lt[s];
                return make_float2(t.y, t.w);                       // X_r0[M], X_r1[M] real
            }
            const float4 t = lt[(N - k) * S + s];
            return make_float2(t.x + t.w, t.z - t.y);               // conj X_r0 + i conj X_r1
        };
        const int k = groups.out_idx[base + gi];
        const float mu = gp.mu[k], c2 = gp.c2[k], w2 = gp.w2[k];
        float* ud = DBG ? udbg + (size_t(k) * N + y0) * N : nullptr;
        auto gst = [&](int s, int i, float2 v, int it, int r) {
            const float dx = v.x - mu, dy = v.y - mu;
            acc[it][r].x = fmaf(w2, ex2_approx(dx * dx * c2), acc[it][r].x);
            acc[it][r].y = fmaf(w2, ex2_approx(dy * dy * c2), acc[it][r].y);
            if constexpr (DBG) {
                ud[size_t(2 * s) * N + i] = v.x * udbg_scale;
                ud[size_t(2 * s + 1) * N + i] = v.y * udbg_scale;
            }
        };
        // the first pass reads the landing tile and the last one keeps its
        // values in registers: neither needs its load-store barrier
        fft_with_hook<N, true, T, S, false, P::ROW_MR, P::SF, false, false>(
            ld0, rows, rows, gst, tw + P::TWOFF, [&]() {
                if (gi + 1 < cnt) issue(gi + 1);   // the first pass has read the tile
            });
    }

    float* Ac = A + (size_t(c) * N + y0) * N;
    const float tl = temp * 1.44269504088896341f;   // temp log2(e)
    const float toff = -tl * gp.wsum[c];
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        const int item = threadIdx.x + it * T;
        if (ITEMS % T == 0 || item < ITEMS) {
            int s, j;
            item_pos<S, JL, P::SF>(item, s, j);
#pragma unroll
            for (int r = 0; r < RL; ++r) {
                const int i = j + r * JL;
                Ac[size_t(2 * s) * N + i] = ex2_approx(fmaf(tl, acc[it][r].x, toff));
                Ac[size_t(2 * s + 1) * N + i] = ex2_approx(fmaf(tl, acc[it][r].y, toff));
            }
        }
    }
    return true;
}

}  // namespace cg
