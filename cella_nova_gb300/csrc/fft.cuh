// fft.cuh — shared-memory batched FFT building blocks for sm_103a.
//
// The reference transforms each row or column of the grid with a radix-2 DIT
// FFT in WGSL (ml-rs/shaders/compute_1024.wgsl:38-218): a bit-reversal LUT
// on load, eight radix-2 stages in workgroup memory and two or three in
// registers, twiddles from an f32-angle host table (convolution.rs:19-30).
// This file does the same transform differently: a mixed-radix Stockham
// auto-sort FFT (radix 16 passes, then one radix 2/4/8 pass), natural order
// in and out, every pass a register-resident DFT-R between two shared-memory
// exchanges, twiddles from a table of W_N^m rounded once from double.
//
// A CTA transforms S independent sequences of length L at once.  Each pass
// is written against load / store functors so that the first pass can read
// global memory (or pre-process while loading) and the last pass can write
// global memory (or feed an epilogue) without an extra shared-memory trip.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

namespace cg {

// Shared-memory index padding: one spare float2 per 16, which keeps the
// strided stores of every pass free of bank conflicts within a half-warp.
__host__ __device__ constexpr int pidx(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int n) { return n + n / 16; }

// S padded sequences in shared memory, sequence s at buf + s * pitch.  A pass
// that reads or writes one of these addresses element j + c (c = r * J or
// r * NS, a compile-time constant after unrolling) as pidx(j) + pidx(c): the
// low four bits of j and c never carry into each other in any Stockham pass
// of a power-of-two plan, so this equals pidx(j + c), and the per-element
// offsets become immediates.
struct SmemRows {
    float2* buf;
    int pitch;
};
template <class F>
struct is_smem_rows : std::is_same<std::remove_cv_t<std::remove_reference_t<F>>, SmemRows> {};

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// cos(2*pi*q/16) and sin(2*pi*q/16), q = 0..15 (exact constants to float).
__device__ __forceinline__ constexpr float cos16(int q) {
    return q == 0 ? 1.0f : q == 1 ? 0.92387953251128674f : q == 2 ? 0.70710678118654752f
         : q == 3 ? 0.38268343236508977f : q == 4 ? 0.0f : q == 5 ? -0.38268343236508977f
         : q == 6 ? -0.70710678118654752f : q == 7 ? -0.92387953251128674f : q == 8 ? -1.0f
         : q == 9 ? -0.92387953251128674f : q == 10 ? -0.70710678118654752f
         : q == 11 ? -0.38268343236508977f : q == 12 ? 0.0f : q == 13 ? 0.38268343236508977f
         : q == 14 ? 0.70710678118654752f : 0.92387953251128674f;
}
__device__ __forceinline__ constexpr float sin16(int q) { return cos16((q + 12) & 15); }

// a * exp(-+2*pi*i*q16/16): forward uses the minus sign, inverse the plus.
// Called with compile-time q16 after unrolling, so the branches fold.
template <bool INV>
__device__ __forceinline__ float2 rot16(float2 a, int q16) {
    if (q16 == 0) return a;
    if (q16 == 4) return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    if (q16 == 8) return make_float2(-a.x, -a.y);
    if (q16 == 12) return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    const float c = cos16(q16), s = sin16(q16);
    return INV ? make_float2(a.x * c - a.y * s, a.y * c + a.x * s)
               : make_float2(a.x * c + a.y * s, a.y * c - a.x * s);
}

// In-register DFT of size R (1, 2, 4, 8, 16), natural order in and out.
template <int R, bool INV>
struct Dft {
    __device__ __forceinline__ static void run(float2* v) {
        float2 e[R / 2], o[R / 2];
#pragma unroll
        for (int i = 0; i < R / 2; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
        Dft<R / 2, INV>::run(e);
        Dft<R / 2, INV>::run(o);
#pragma unroll
        for (int q = 0; q < R / 2; ++q) {
            const float2 t = rot16<INV>(o[q], q * (16 / R));
            v[q] = cadd(e[q], t);
            v[q + R / 2] = csub(e[q], t);
        }
    }
};
template <bool INV>
struct Dft<2, INV> {
    __device__ __forceinline__ static void run(float2* v) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};
template <bool INV>
struct Dft<1, INV> {
    __device__ __forceinline__ static void run(float2*) {}
};

// Radix of the pass that starts at sub-transform size NS, for plans of
// maximum radix MR (16 or 8).  Greedy plans use radix MR until fewer than MR
// remain (MR,MR,...,rem); REMFIRST plans put the remainder first
// (rem,MR,MR,...), so the first pass of a REMFIRST inverse sees exactly the
// index sets the last pass of a greedy forward transform left in each
// thread's registers.
__host__ __device__ constexpr int log2_of(int v) {
    int b = 0;
    while ((1 << b) < v) ++b;
    return b;
}
__host__ __device__ constexpr int rem_radix(int L, int MR = 16) {
    const int b = log2_of(L), g = log2_of(MR);
    return (b % g) == 0 ? (L >= MR ? MR : L) : (1 << (b % g));
}
__host__ __device__ constexpr int plan_radix(int L, int ns, bool remfirst, int MR = 16) {
    return (remfirst && ns == 1) ? rem_radix(L, MR) : ((L / ns >= MR) ? MR : (L / ns));
}
template <int L, int NS, bool REMFIRST = false, int MR = 16>
struct PassRadix {
    static constexpr int R = plan_radix(L, NS, REMFIRST, MR);
};

// Per-pass twiddle tables.  The pass starting at sub-transform size NS > 1
// with radix R reads W_{NS*R}^{r*k} for r in [1, R), k in [0, NS), stored at
// tw_offset(L, plan, NS) + (r-1)*NS + k: consecutive butterflies read
// consecutive entries (one or two L1 wavefronts per warp).
__host__ __device__ constexpr int tw_offset(int L, bool remfirst, int NS, int MR = 16) {
    int off = 0, ns = 1;
    while (ns < NS) {
        const int R = plan_radix(L, ns, remfirst, MR);
        if (ns > 1) off += (R - 1) * ns;
        ns *= R;
    }
    return off;
}
__host__ __device__ constexpr int tw_size(int L, bool remfirst, int MR = 16) {
    return tw_offset(L, remfirst, L, MR);
}

// Radix of the last pass of a greedy length-L transform.
__host__ __device__ constexpr int last_radix(int L, int MR = 16) {
    int ns = 1, r = 1;
    while (ns < L) {
        r = (L / ns >= MR) ? MR : L / ns;
        ns *= r;
    }
    return r;
}

// Radix of the last pass of a greedy or remainder-first plan.
__host__ __device__ constexpr int plan_last_radix(int L, bool remfirst, int MR = 16) {
    int ns = 1, r = 1;
    while (ns < L) {
        r = plan_radix(L, ns, remfirst, MR);
        ns *= r;
    }
    return r;
}

// One Stockham pass (radix R, sub-transform size NS) over S sequences of
// length L, with T threads.  Work item `item` = (sequence s, butterfly j):
// s = item / J, j = item % J, or with SFAST the sequence index runs fastest,
// s = item % S, j = item / S (a warp then spans S sequences at the same few
// butterflies, which suits inputs stored element-major, x[j][s]); thread t
// owns items t, t+T, ...  It loads v[r] = x[j + r*L/R], applies
// W_{NS*R}^{r*(j mod NS)}, runs DFT-R and stores v[q] at
// (j div NS)*NS*R + (j mod NS) + q*NS.  All loads finish (barrier) before any
// store, so in-place passes are safe; a second barrier closes the pass.  A
// caller whose loads and stores of this pass cannot touch the same shared
// memory (loads from global memory or another buffer, or stores to registers
// or global memory) passes MIDBAR = false and skips the first barrier.
//   twp : this pass's table (tw_offset layout).
//   ld(s, i, it, q)         -> float2
//   st(s, i, v, it, q)      (it, q) name the register slot of the value.
template <int S, int J, bool SFAST>
__device__ __forceinline__ void item_pos(int item, int& s, int& j) {
    if constexpr (SFAST) {
        s = item % S;
        j = item / S;
    } else {
        s = item / J;
        j = item % J;
    }
}

template <int L, int R, int NS, bool INV, int T, int S, bool SFAST = false, bool MIDBAR = true,
          class LD, class ST>
__device__ __forceinline__ void stockham_pass(LD& ld, ST& st, const float2* __restrict__ twp) {
    constexpr int J = L / R;
    constexpr int ITEMS = S * J;
    constexpr int IPT = (ITEMS + T - 1) / T;
    float2 v[IPT][R];
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        const int item = threadIdx.x + it * T;
        if (ITEMS % T == 0 || item < ITEMS) {
            int s, j;
            item_pos<S, J, SFAST>(item, s, j);
            if constexpr (is_smem_rows<LD>::value) {
                const float2* b = ld.buf + s * ld.pitch + pidx(j);
#pragma unroll
                for (int r = 0; r < R; ++r) v[it][r] = b[pidx(r * J)];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) v[it][r] = ld(s, j + r * J, it, r);
            }
        }
    }
    if constexpr (MIDBAR) __syncthreads();
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        const int item = threadIdx.x + it * T;
        if (ITEMS % T == 0 || item < ITEMS) {
            int s, j;
            item_pos<S, J, SFAST>(item, s, j);
            const int k = j % NS;
            if (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    float2 w = __ldg(&twp[(r - 1) * NS + k]);
                    if (INV) w.y = -w.y;
                    v[it][r] = cmul(v[it][r], w);
                }
            }
            Dft<R, INV>::run(v[it]);
            const int d = (j / NS) * NS * R + k;
            if constexpr (is_smem_rows<ST>::value) {
                float2* b = st.buf + s * st.pitch + pidx(d);
#pragma unroll
                for (int r = 0; r < R; ++r) b[pidx(r * NS)] = v[it][r];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) st(s, d + r * NS, v[it][r], it, r);
            }
        }
    }
    __syncthreads();
}

// Full length-L transform: first pass reads through `ld`, middle passes use
// shared memory through smld/smst, the last pass writes through `stl`.
// `tab` is the plan's twiddle table (tw_offset layout); SFAST selects the
// item order of every pass (stockham_pass).  FIRSTBAR / LASTBAR = false
// drop the load-store barrier of the first / last pass (stockham_pass's
// MIDBAR): for a first pass whose `ld` reads no shared memory that smst
// writes, and a last pass whose `stl` writes no shared memory smld reads.
template <int L, int NS, bool INV, int T, int S, bool REMFIRST = false, int MR = 16,
          bool SFAST = false, bool FIRSTBAR = true, bool LASTBAR = true>
struct FftPasses {
    template <class LD, class SMLD, class SMST, class STL>
    __device__ __forceinline__ static void run(LD& ld, SMLD& smld, SMST& smst, STL& stl,
                                               const float2* __restrict__ tab) {
        constexpr int R = PassRadix<L, NS, REMFIRST, MR>::R;
        constexpr bool FIRST = (NS == 1), LAST = (NS * R == L);
        constexpr bool BAR = FIRST && LAST ? (FIRSTBAR || LASTBAR)
                                           : (FIRST ? FIRSTBAR : (LAST ? LASTBAR : true));
        const float2* twp = tab + tw_offset(L, REMFIRST, NS, MR);
        if constexpr (LAST) {
            stockham_pass<L, R, NS, INV, T, S, SFAST, BAR>(ld, stl, twp);
        } else {
            stockham_pass<L, R, NS, INV, T, S, SFAST, BAR>(ld, smst, twp);
            FftPasses<L, NS * R, INV, T, S, REMFIRST, MR, SFAST, FIRSTBAR, LASTBAR>::run(
                smld, smld, smst, stl, tab);
        }
    }
};

// Run the first pass of a transform, then `hook()`, then the rest.
// FIRSTBAR / LASTBAR as in FftPasses.
template <int L, bool INV, int T, int S, bool REMFIRST, int MR = 16, bool SFAST = false,
          bool FIRSTBAR = true, bool LASTBAR = true, class LD, class SMLD, class SMST, class STL,
          class HOOK>
__device__ __forceinline__ void fft_with_hook(LD& ld, SMLD& smld, SMST& smst, STL& stl,
                                              const float2* __restrict__ tab, HOOK hook) {
    constexpr int R = PassRadix<L, 1, REMFIRST, MR>::R;
    if constexpr (R == L) {
        stockham_pass<L, R, 1, INV, T, S, SFAST, FIRSTBAR || LASTBAR>(ld, stl, tab);
        hook();
    } else {
        stockham_pass<L, R, 1, INV, T, S, SFAST, FIRSTBAR>(ld, smst, tab);
        hook();
        FftPasses<L, R, INV, T, S, REMFIRST, MR, SFAST, true, LASTBAR>::run(smld, smld, smst, stl,
                                                                             tab);
    }
}

}  // namespace cg
