/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * Generic body of the CPU oracle for one DiffusionLenia step, instantiated
 * twice by lenia_oracle.c: once with REAL=double (the FP64 oracle every parity
 * test is checked against) and once with REAL=float (the faithful FP32 CPU
 * baseline, same arithmetic as the reference's f32 CPU program).
 *
 * It restates ml-rs/example.rs of anima-zetta/cella-nova:
 *   fft_1d            example.rs:42-71   radix-2 DIT, bit-reversal first
 *   ifft_1d           example.rs:76-88   conjugate, forward FFT, conjugate, 1/n
 *   fft_2d / ifft_2d  example.rs:95-126  rows, then columns
 *   step_ml           example.rs:164-222 per-kernel FFT conv, growth, diffusion
 *   growth_phase      example.rs:228-266 bump G(u), weighted sum, exp(temp*sum)
 *   diffusion_phase   example.rs:272-303 toroidal 3x3 Z, then A*sum(state/Z)
 * generalised from compile-time N, C, K=C*C, TEMP to runtime values and to the
 * orchestrator's c0 (input channel) / c1 (output channel) meaning
 * (ml-rs/orchestrator/convolution.rs:689, shaders/compute_1024.wgsl:313-319).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
 * this code, and only to check results or to time the CPU baseline.
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SUF)
#define CPX FN(orc_cpx)

typedef struct { REAL re, im; } CPX;

static inline CPX FN(cmul_)(CPX a, CPX b) {  /* example.rs:24-26 */
    CPX r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}

/* In-place forward FFT of length n (power of two), example.rs:42-71. */
static void FN(fft_1d_)(CPX* d, int n) {
    int bits = 0;
    while ((1 << bits) < n) bits++;
    for (int i = 0; i < n; i++) {
        unsigned j = 0, v = (unsigned)i;
        for (int b = 0; b < bits; b++) { j = (j << 1) | (v & 1u); v >>= 1; }
        if ((unsigned)i < j) { CPX t = d[i]; d[i] = d[j]; d[j] = t; }
    }
    for (int len = 1; len < n;) {
        int half = len;
        len *= 2;
        /* example.rs:60,63: angle = -pi/half, w = e^{i*angle*j}.  The FP64
         * build evaluates the angle in double; the FP32 build keeps the
         * reference's f32 angle product. */
        REAL angle = -(REAL)ORC_PI / (REAL)half;
        for (int i = 0; i < n; i += len) {
            for (int j = 0; j < half; j++) {
                REAL a = angle * (REAL)j;
                CPX w = {COS(a), SIN(a)};
                CPX u = d[i + j];
                CPX v = FN(cmul_)(d[i + j + half], w);
                d[i + j].re = u.re + v.re;
                d[i + j].im = u.im + v.im;
                d[i + j + half].re = u.re - v.re;
                d[i + j + half].im = u.im - v.im;
            }
        }
    }
}

/* example.rs:76-88 */
static void FN(ifft_1d_)(CPX* d, int n) {
    for (int i = 0; i < n; i++) d[i].im = -d[i].im;
    FN(fft_1d_)(d, n);
    REAL fn = (REAL)n;
    for (int i = 0; i < n; i++) {
        d[i].im = -d[i].im;
        d[i].re /= fn;
        d[i].im /= fn;
    }
}

/* example.rs:95-126: rows first, then columns through a column buffer. */
static void FN(fft_2d_)(CPX* g, int n, int inverse, int nthreads) {
    #pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int r = 0; r < n; r++) {
        if (inverse) FN(ifft_1d_)(g + (size_t)r * n, n);
        else FN(fft_1d_)(g + (size_t)r * n, n);
    }
    #pragma omp parallel num_threads(nthreads)
    {
        CPX* col = (CPX*)malloc(sizeof(CPX) * (size_t)n);
        #pragma omp for schedule(static)
        for (int c = 0; c < n; c++) {
            for (int r = 0; r < n; r++) col[r] = g[(size_t)r * n + c];
            if (inverse) FN(ifft_1d_)(col, n);
            else FN(fft_1d_)(col, n);
            for (int r = 0; r < n; r++) g[(size_t)r * n + c] = col[r];
        }
        free(col);
    }
}

/*
 * One step, in place on `state` (C planes of n*n, row-major).
 *   kspec   : K full spectra, n*n complex interleaved (re, im), origin at [0,0]
 *   c0, c1  : kernel k reads channel c0[k] and feeds output channel c1[k]
 *   faithful: 1 = recompute FFT(state[c0[k]]) for every kernel, as
 *             example.rs:179-199 does; 0 = transform each channel once
 *             (identical arithmetic, fewer repeats)
 *   u_out   : optional, K*n*n — Re of the normalised convolution (the value
 *             the growth function reads, example.rs:251)
 *   aff_out : optional, C*n*n — A = exp(temp * weighted growth sum)
 * Returns 0, or -1 on allocation failure.
 */
int FN(orc_step)(int n, int C, int K, REAL* state, const REAL* kspec,
                 const uint32_t* c0, const uint32_t* c1, const REAL* mu,
                 const REAL* sigma, const REAL* weight, REAL temp,
                 int faithful, int nthreads, REAL* u_out, REAL* aff_out) {
    size_t px = (size_t)n * n;
    CPX* conv = (CPX*)malloc(sizeof(CPX) * px * (size_t)K);
    CPX* spec = (CPX*)malloc(sizeof(CPX) * px * (size_t)C);
    REAL* aff = (REAL*)malloc(sizeof(REAL) * px);
    REAL* wsum = (REAL*)malloc(sizeof(REAL) * px);
    REAL* zsum = (REAL*)malloc(sizeof(REAL) * px);
    REAL* chtmp = (REAL*)malloc(sizeof(REAL) * px);
    if (!conv || !spec || !aff || !wsum || !zsum || !chtmp) {
        free(conv); free(spec); free(aff); free(wsum); free(zsum); free(chtmp);
        return -1;
    }
    if (nthreads < 1) nthreads = 1;

    /* Phase 1, example.rs:179-199 */
    if (!faithful) {
        for (int c = 0; c < C; c++) {
            CPX* s = spec + (size_t)c * px;
            for (size_t i = 0; i < px; i++) { s[i].re = state[(size_t)c * px + i]; s[i].im = 0; }
            FN(fft_2d_)(s, n, 0, nthreads);
        }
    }
    for (int k = 0; k < K; k++) {
        int in_ch = (int)c0[k];
        CPX* g = conv + (size_t)k * px;
        if (faithful) {
            for (size_t i = 0; i < px; i++) { g[i].re = state[(size_t)in_ch * px + i]; g[i].im = 0; }
            FN(fft_2d_)(g, n, 0, nthreads);
        } else {
            memcpy(g, spec + (size_t)in_ch * px, sizeof(CPX) * px);
        }
        const CPX* kk = (const CPX*)(kspec + (size_t)k * px * 2);
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (long i = 0; i < (long)px; i++) g[i] = FN(cmul_)(g[i], kk[i]);
        FN(fft_2d_)(g, n, 1, nthreads);
        if (u_out) for (size_t i = 0; i < px; i++) u_out[(size_t)k * px + i] = g[i].re;
    }

    /* Phases 2-3 per output channel, example.rs:204-221 */
    for (int out_ch = 0; out_ch < C; out_ch++) {
        /* growth_phase, example.rs:237-265 */
        for (size_t i = 0; i < px; i++) wsum[i] = 0;
        for (int k = 0; k < K; k++) {
            if ((int)c1[k] != out_ch) continue;
            REAL m = mu[k], s = sigma[k], w = weight[k];
            REAL inv_s2 = (REAL)1 / (s * s);
            const CPX* g = conv + (size_t)k * px;
            #pragma omp parallel for num_threads(nthreads) schedule(static)
            for (long i = 0; i < (long)px; i++) {
                REAL d = g[i].re - m;
                REAL gr = (REAL)2 * EXP((REAL)-0.5 * d * d * inv_s2) - (REAL)1;
                wsum[i] += gr * w;
            }
        }
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (long i = 0; i < (long)px; i++) aff[i] = EXP(temp * wsum[i]);
        if (aff_out) memcpy(aff_out + (size_t)out_ch * px, aff, sizeof(REAL) * px);

        /* diffusion_phase, example.rs:272-303 */
        REAL* ch = state + (size_t)out_ch * px;
        memcpy(chtmp, ch, sizeof(REAL) * px);
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < n; j++) {
                REAL s = 0;
                for (int di = 0; di < 3; di++)
                    for (int dj = 0; dj < 3; dj++) {
                        int ni = (i + di + n - 1) % n, nj = (j + dj + n - 1) % n;
                        s += aff[(size_t)ni * n + nj];
                    }
                zsum[(size_t)i * n + j] = s;
            }
        }
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < n; j++) {
                REAL s = 0;
                for (int di = 0; di < 3; di++)
                    for (int dj = 0; dj < 3; dj++) {
                        int ni = (i + di + n - 1) % n, nj = (j + dj + n - 1) % n;
                        size_t q = (size_t)ni * n + nj;
                        s += chtmp[q] / zsum[q];
                    }
                ch[(size_t)i * n + j] = aff[(size_t)i * n + j] * s;
            }
        }
    }
    free(conv); free(spec); free(aff); free(wsum); free(zsum); free(chtmp);
    return 0;
}

/* Per-channel total mass, summed in double (example.rs:547-553 sums in f32;
 * the mass-drift bar is stated against an FP64 sum). */
void FN(orc_mass)(int n, int C, const REAL* state, double* out) {
    size_t px = (size_t)n * n;
    for (int c = 0; c < C; c++) {
        double s = 0;
        for (size_t i = 0; i < px; i++) s += (double)state[(size_t)c * px + i];
        out[c] = s;
    }
}

#undef CPX
#undef FN
#undef CAT
#undef CAT2
