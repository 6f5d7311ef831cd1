// host.cu — the GpuMaceLenia orchestrator (ml-rs/orchestrator/mod.rs) in C++
// behind the C ABI of include/cella_gpu.h.
//
// Buffers (mod.rs:109-122 allocates channel, new_channel, affinity, z,
// kernel, conv, render) become: two state planes used in turn (no
// new_channel -> channel copy, mod.rs:377-383), row spectra, packed kernel
// half spectra, column-inverted products and the affinity exponential.  The
// Z buffer does not exist (Z lives in shared memory); the render buffer is
// written only by the render calls.  A step is two CUDA graphs, one per
// ping-pong parity, captured once at creation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <errno.h>
#include <unistd.h>

#include "cella_gpu.h"
#include "cella_internal.h"
#include "fft.cuh"

namespace cg {
extern const SizeOps size_ops_l4, size_ops_l5, size_ops_l6, size_ops_l7, size_ops_l8, size_ops_l9, size_ops_l10,
    size_ops_l11;

const SizeOps* size_ops(int logn) {
    switch (logn) {
        case 4: return &size_ops_l4;
        case 5: return &size_ops_l5;
        case 6: return &size_ops_l6;
        case 7: return &size_ops_l7;
        case 8: return &size_ops_l8;
        case 9: return &size_ops_l9;
        case 10: return &size_ops_l10;
        case 11: return &size_ops_l11;
        default: return nullptr;
    }
}

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(CG_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(CG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Device buffers given to the library feed 16-byte vector loads and bulk
// copies (TMA), so each must start on a 16-byte boundary (every cudaMalloc
// and PyTorch allocation does; a view at an odd element offset may not).
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
int misaligned(const char* fn) {
    return fail(CG_ERR_ARG, "%s: device buffers must be 16-byte aligned", fn);
}

#define CG_CHECK(call, what)                                \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
    } while (0)

// W_n^m for m < n, then the Stockham pass tables (fft.cuh tw_offset layout)
// of the column forward plan (greedy), the column inverse plan (remainder
// first), the row plan (greedy, length n/2) and the radix-8 plan of length n
// (greedy).  Every entry is rounded once
// from double; the reference builds its table from an f32 angle
// (convolution.rs:19-30).
static void fill_plan(int L, bool remfirst, int MR, float2* out) {
    int ns = 1;
    while (ns < L) {
        const int R = plan_radix(L, ns, remfirst, MR);
        if (ns > 1) {
            float2* t = out + tw_offset(L, remfirst, ns, MR);
            for (int r = 1; r < R; ++r)
                for (int k = 0; k < ns; ++k) {
                    const double a = -2.0 * M_PI * double(r) * double(k) / double(ns * R);
                    t[(r - 1) * ns + k] = make_float2(float(std::cos(a)), float(std::sin(a)));
                }
        }
        ns *= R;
    }
}

void build_twiddle_tables(int n, float2* out) {
    for (int m = 0; m < n; ++m) {
        const double a = -2.0 * M_PI * double(m) / double(n);
        out[m] = make_float2(float(std::cos(a)), float(std::sin(a)));
    }
    float2* p = out + n;
    fill_plan(n, false, 16, p);
    p += tw_size(n, false);
    fill_plan(n, true, 16, p);
    p += tw_size(n, true);
    fill_plan(n / 2, false, 16, p);
    p += tw_size(n / 2, false);
    fill_plan(n, false, 8, p);
}

static bool finite(float v) { return std::isfinite(v); }

// The packed kernel spectrum is the Hermitian part (K(f) + conj K(-f)) / 2;
// it is real when Im K(f) = Im K(-f), i.e. the spatial kernel is
// point-symmetric (h(x) = h(-x)), as every radially symmetric Lenia ring
// is.  Real to rounding: max |Im K(f) - Im K(-f)| <= 1e-9 max |Re K(f) +
// Re K(-f)|; a spectrum computed in double from a symmetric kernel leaves
// ~1e-17 there, any genuinely complex one orders of magnitude more.
bool hermitian_part_is_real(const float* spec, int n) {
    double re = 0.0, im = 0.0;
    for (int fy = 0; fy < n; ++fy) {
        const int my = (n - fy) & (n - 1);
        for (int fx = 0; fx < n; ++fx) {
            const int mx = (n - fx) & (n - 1);
            const float* a = spec + 2 * (size_t(fy) * n + fx);
            const float* b = spec + 2 * (size_t(my) * n + mx);
            re = std::max(re, std::fabs(double(a[0]) + double(b[0])));
            im = std::max(im, std::fabs(double(a[1]) - double(b[1])));
        }
    }
    return im <= 1e-9 * re;
}

int validate_world(int n, int C, int K, const uint32_t* c0, const uint32_t* c1, const float* mu,
                   const float* sigma, const float* weights, float temp, int* logn_out) {
    int logn = 0;
    while ((1 << logn) < n && logn < 30) ++logn;
    if (n <= 0 || (1 << logn) != n)
        return fail(CG_ERR_ARG, "grid side %d is not a power of two", n);
    if (logn < kMinLogN || logn > kMaxLogN)
        return fail(CG_ERR_UNSUPPORTED, "grid side %d outside [%d, %d]", n, 1 << kMinLogN,
                    1 << kMaxLogN);
    if (C < 1 || C > kMaxC) return fail(CG_ERR_ARG, "channel count %d outside [1, %d]", C, kMaxC);
    if (K < 1 || K > kMaxK) return fail(CG_ERR_ARG, "kernel count %d outside [1, %d]", K, kMaxK);
    if (!c0 || !c1 || !mu || !sigma || !weights)
        return fail(CG_ERR_ARG, "NULL parameter array");
    for (int k = 0; k < K; ++k) {
        if (c0[k] >= uint32_t(C) || c1[k] >= uint32_t(C))
            return fail(CG_ERR_ARG, "kernel %d maps channel %u -> %u, but C = %d", k, c0[k],
                        c1[k], C);
        if (!finite(mu[k]) || !finite(sigma[k]) || !finite(weights[k]) || sigma[k] == 0.f)
            return fail(CG_ERR_ARG, "kernel %d has a non-finite or zero-sigma growth parameter",
                        k);
    }
    if (!finite(temp)) return fail(CG_ERR_ARG, "temp is not finite");
    *logn_out = logn;
    return CG_OK;
}

void build_groups(int C, int K, const uint32_t* c0, const uint32_t* c1, const float* mu,
                  const float* sigma, const float* weights, KernelGroups* g, GrowthParams* gp) {
    *g = KernelGroups{};
    *gp = GrowthParams{};
    int pos = 0;
    for (int c = 0; c < C; ++c) {   // in increasing k within each channel
        g->in_start[c] = pos;
        for (int k = 0; k < K; ++k)
            if (int(c0[k]) == c) g->in_idx[pos++] = k;
        g->in_count[c] = pos - g->in_start[c];
    }
    pos = 0;
    for (int c = 0; c < C; ++c) {
        g->out_start[c] = pos;
        for (int k = 0; k < K; ++k)
            if (int(c1[k]) == c) g->out_idx[pos++] = k;
        g->out_count[c] = pos - g->out_start[c];
    }
    for (int k = 0; k < K; ++k) {
        gp->mu[k] = mu[k];
        gp->c2[k] = float(-1.4426950408889634 / (2.0 * double(sigma[k]) * double(sigma[k])));
        gp->w2[k] = 2.0f * weights[k];
    }
    for (int c = 0; c < C; ++c) {
        float ws = 0.f;   // f32, increasing k: the reference's sum of w * (-1)
        for (int i = 0; i < g->out_count[c]; ++i) ws += weights[g->out_idx[g->out_start[c] + i]];
        gp->wsum[c] = ws;
    }
}

}  // namespace cg

using namespace cg;

// Host-buffer pipeline of cg_step_host_async: uploads on `up` into one of two
// staging buffers, conversion and steps on the sim's stream, downloads on
// `down`.
struct HostPipe {
    cudaStream_t up = nullptr, down = nullptr;
    double* stage[2] = {nullptr, nullptr};   // C * n * n f64 each
    cudaEvent_t up_done[2] = {nullptr, nullptr};
    cudaEvent_t conv_done[2] = {nullptr, nullptr};
    cudaEvent_t step_done = nullptr, down_done = nullptr;
    int slot = 0;
    bool ready = false;
};

struct cg_sim {
    int n = 0, logn = 0, C = 0, K = 0;
    float temp = 1.f;
    std::vector<uint32_t> c0, c1;
    std::vector<float> mu, sigma, w;
    const SizeOps* ops = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    float* state[2] = {nullptr, nullptr};
    int cur = 0;
    float2* rowspec = nullptr;
    float2* kspec = nullptr;
    // real parts of kspec, and which kernels cg_set_kernel found
    // point-symmetric: when all are, the column pass reads kspec_re
    float* kspec_re = nullptr;
    std::vector<uint8_t> kreal;
    bool kreal_all = false;
    float2* U = nullptr;       // two [K][n/2][n] buffers, one per ping-pong parity
    float* A = nullptr;
    float2* tw = nullptr;
    void* staging = nullptr;
    double* mass_partial = nullptr;
    double* mass_out = nullptr;
    int* err = nullptr;   // device error word written by bounded waits
    cudaGraphExec_t graph[2] = {nullptr, nullptr};     // one step, per parity
    cudaGraphExec_t graph8[2] = {nullptr, nullptr};    // kStepsPerGraph steps, per parity
    cudaGraphExec_t graphR[2] = {nullptr, nullptr};    // one step that also renders
    unsigned* render = nullptr;   // [n][n] packed 0x00RRGGBB
    unsigned char* levels = nullptr;   // [3][n][n] render levels of a rendering step
    unsigned char* frames[2] = {nullptr, nullptr};   // pinned RGB24 frames (frame streaming)
    cudaEvent_t frame_ev[2] = {nullptr, nullptr};
    double* ring_partial = nullptr;   // kernel builder: K * kRingBlocks * kMaxRings
    double* ring_s = nullptr;         // K * kMaxRings per-ring sums of the last build
    double* zsum = nullptr;           // K normalisers of the last build
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    HostPipe pipe;
    KernelGroups groups{};
    GrowthParams gp{};          // host copies of the folded parameters
    AdjointParams ap{};
    DeviceParams* dparams = nullptr;   // the copies the kernels read
    Variants var{};
    // graph layout: 0, each channel's launches on a forked stream of its own
    // (the channels' phases overlap); 1, one stream, one launch per phase
    // over all channels (fewer, larger launches); the tuner picks
    int layout = 0;
    float* abar = nullptr;          // backward scratch, allocated on first use
    float* utmp[2] = {nullptr, nullptr};   // cg_unroll scratch states
    // cg_unroll_backward: each segment step's row spectra, U and A, kept from
    // the segment's recompute for its backward step (cache_steps of them)
    void* seg_cache = nullptr;
    int cache_steps = 0;
    bool bwd_ready = false;

    size_t px() const { return size_t(n) * n; }

    StepArgs args(int from, float* udbg) const {
        StepArgs a{};
        a.C = C;
        a.K = K;
        a.temp = temp;
        a.x_in = state[from];
        a.x_out = state[from ^ 1];
        a.rowspec = rowspec;
        a.kspec = kspec;
        a.kre = kreal_all ? kspec_re : nullptr;
        a.U = U + size_t(from) * K * (size_t(n / 2) * n);
        a.A = A;
        a.tw = tw;
        a.udbg = udbg;
        a.err = err;
        a.groups = groups;
        a.gp = &dparams->gp;
        a.var = var;
        return a;
    }
};

namespace {

void release(cg_sim* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    for (auto& g : s->graph)
        if (g) cudaGraphExecDestroy(g);
    for (auto& g : s->graph8)
        if (g) cudaGraphExecDestroy(g);
    for (auto& g : s->graphR)
        if (g) cudaGraphExecDestroy(g);
    for (auto& e : s->ev)
        if (e) cudaEventDestroy(e);
    cudaFree(s->state[0]);
    cudaFree(s->state[1]);
    cudaFree(s->rowspec);
    cudaFree(s->kspec);
    cudaFree(s->kspec_re);
    cudaFree(s->U);
    cudaFree(s->A);
    cudaFree(s->tw);
    cudaFree(s->staging);
    cudaFree(s->mass_partial);
    cudaFree(s->mass_out);
    cudaFree(s->err);
    cudaFree(s->dparams);
    cudaFree(s->render);
    cudaFree(s->levels);
    for (auto& f : s->frames)
        if (f) cudaFreeHost(f);
    for (auto& e : s->frame_ev)
        if (e) cudaEventDestroy(e);
    cudaFree(s->ring_partial);
    cudaFree(s->ring_s);
    cudaFree(s->zsum);
    cudaFree(s->abar);
    cudaFree(s->seg_cache);
    cudaFree(s->utmp[0]);
    cudaFree(s->utmp[1]);
    HostPipe& p = s->pipe;
    for (auto* st : {p.up, p.down})
        if (st) cudaStreamDestroy(st);
    for (auto* b : p.stage) cudaFree(b);
    for (auto* e : {p.up_done[0], p.up_done[1], p.conv_done[0], p.conv_done[1], p.step_done,
                    p.down_done})
        if (e) cudaEventDestroy(e);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

constexpr int kStepsPerGraph = 8;

// Capture `nsteps` steps starting at ping-pong parity p0 as one graph whose
// launches are per channel, on one stream per channel, so that independent
// channels overlap (one channel's diffusion runs in another's tail).  Only
// two dependencies cross channels: the inverse row pass of step t needs every
// channel's column pass of step t (the products U of all input channels), and
// the column pass of step t overwrites the U buffer of its parity, which every
// inverse row pass of step t-2 read.  Everything else is per channel and in
// stream order.
// nsteps steps from parity p0 into one graph; with render, the last step's
// diffusion kernels also write the level planes, and after the channels have
// joined, k_pack_levels turns them into the render buffer's words.
// fixed_parity: every captured step reads the same state (p0) and writes the
// other buffer (U still alternates, so the dependencies are a real run's),
// so replaying the graph does not advance the world (the tuner's timing)
cudaError_t capture_steps(cg_sim* s, int p0, int nsteps, bool render, cudaGraphExec_t* out,
                          bool fixed_parity = false) {
    const int C = s->C;
    if (s->layout == 1) {   // one stream, one launch per phase over all channels
        cudaStream_t st0 = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&st0, cudaStreamNonBlocking);
        cudaGraph_t g = nullptr;
        if (e == cudaSuccess) e = cudaStreamBeginCapture(st0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t le = cudaSuccess;
            for (int t = 0; t < nsteps && le == cudaSuccess; ++t) {
                StepArgs a = s->args(p0 ^ (t & 1), nullptr);
                if (fixed_parity) {
                    a.x_in = s->state[p0];
                    a.x_out = s->state[p0 ^ 1];
                }
                if (render && t == nsteps - 1) a.levels = s->levels;
                le = s->ops->step(a, kPhaseAll, st0);
            }
            if (render && le == cudaSuccess)
                le = launch_pack_levels(s->levels, C, s->px(), s->render, st0);
            e = cudaStreamEndCapture(st0, &g);
            if (le != cudaSuccess) e = le;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
        if (g) cudaGraphDestroy(g);
        if (st0) cudaStreamDestroy(st0);
        return e;
    }
    std::vector<cudaStream_t> st(C, nullptr);
    std::vector<cudaEvent_t> ecol(C, nullptr);
    std::vector<cudaEvent_t> ec2r[2] = {std::vector<cudaEvent_t>(C, nullptr),
                                        std::vector<cudaEvent_t>(C, nullptr)};
    cudaEvent_t fork = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    for (int c = 0; c < C && e == cudaSuccess; ++c) {
        e = cudaStreamCreateWithFlags(&st[c], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ecol[c], cudaEventDisableTiming);
        for (int q = 0; q < 2 && e == cudaSuccess; ++q)
            e = cudaEventCreateWithFlags(&ec2r[q][c], cudaEventDisableTiming);
    }
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(st[0], cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t le = cudaEventRecord(fork, st[0]);
        for (int c = 1; c < C && le == cudaSuccess; ++c) le = cudaStreamWaitEvent(st[c], fork, 0);
        for (int t = 0; t < nsteps && le == cudaSuccess; ++t) {
            StepArgs a = s->args(p0 ^ (t & 1), nullptr);
            if (fixed_parity) {   // the state stays put; U alternates as in a real run
                a.x_in = s->state[p0];
                a.x_out = s->state[p0 ^ 1];
            }
            if (render && t == nsteps - 1) a.levels = s->levels;
            for (int c = 0; c < C && le == cudaSuccess; ++c) {
                le = s->ops->step_channel(a, kPhaseRowFwd, c, st[c]);
                // U alternates with the parity, so the column pass of step t
                // only has to wait for the inverse row passes of step t-2,
                // which read the same buffer
                for (int c2 = 0; t > 1 && c2 < C && le == cudaSuccess; ++c2)
                    le = cudaStreamWaitEvent(st[c], ec2r[t & 1][c2], 0);   // step t-2
                if (le == cudaSuccess) le = s->ops->step_channel(a, kPhaseColConv, c, st[c]);
                if (le == cudaSuccess) le = cudaEventRecord(ecol[c], st[c]);
            }
            for (int c = 0; c < C && le == cudaSuccess; ++c) {
                for (int c2 = 0; c2 < C && le == cudaSuccess; ++c2)
                    if (c2 != c) le = cudaStreamWaitEvent(st[c], ecol[c2], 0);
                if (le == cudaSuccess) le = s->ops->step_channel(a, kPhaseGrowth, c, st[c]);
                if (le == cudaSuccess) le = cudaEventRecord(ec2r[t & 1][c], st[c]);
                if (le == cudaSuccess) le = s->ops->step_channel(a, kPhaseDiffusion, c, st[c]);
            }
        }
        // join every channel stream back into the origin stream
        for (int c = 1; c < C && le == cudaSuccess; ++c) {
            le = cudaEventRecord(ecol[c], st[c]);
            if (le == cudaSuccess) le = cudaStreamWaitEvent(st[0], ecol[c], 0);
        }
        if (render && le == cudaSuccess)
            le = launch_pack_levels(s->levels, C, s->px(), s->render, st[0]);
        e = cudaStreamEndCapture(st[0], &g);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    if (g) cudaGraphDestroy(g);
    for (int c = 0; c < C; ++c) {
        if (st[c]) cudaStreamDestroy(st[c]);
        if (ecol[c]) cudaEventDestroy(ecol[c]);
        for (int q = 0; q < 2; ++q)
            if (ec2r[q][c]) cudaEventDestroy(ec2r[q][c]);
    }
    if (fork) cudaEventDestroy(fork);
    return e;
}

int capture_graphs(cg_sim* s) {
    for (int p = 0; p < 2; ++p) {
        cudaError_t e = capture_steps(s, p, 1, false, &s->graph[p]);
        if (e == cudaSuccess) e = capture_steps(s, p, kStepsPerGraph, false, &s->graph8[p]);
        if (e == cudaSuccess) e = capture_steps(s, p, 1, true, &s->graphR[p]);
        if (e != cudaSuccess) return cuda_fail(e, "capturing the step graph");
    }
    return CG_OK;
}

int build_twiddles(cg_sim* s) {
    std::vector<float2> h(size_t(s->ops->twiddle_count()));
    build_twiddle_tables(s->n, h.data());
    CG_CHECK(cudaMemcpy(s->tw, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice),
             "uploading twiddles");
    return CG_OK;
}


// After a synchronisation: report (and clear) a device-side wait timeout.
int check_device_error(cg_sim* s) {
    int h = 0;
    CG_CHECK(cudaMemcpy(&h, s->err, sizeof(int), cudaMemcpyDeviceToHost), "reading error word");
    if (h != 0) {
        cudaMemset(s->err, 0, sizeof(int));
        return fail(CG_ERR_TIMEOUT, "a device-side wait for an asynchronous copy timed out "
                                    "(error word %d); the last steps are invalid", h);
    }
    return CG_OK;
}

#define CG_SYNC_CHECK(s)                               \
    do {                                               \
        int rc_ = check_device_error(s);               \
        if (rc_ != CG_OK) return rc_;                  \
    } while (0)

void build_adjoint_params(cg_sim* s) {
    for (int k = 0; k < s->K; ++k) {
        const double sg = double(s->sigma[k]);
        s->ap.cout[k] = int(s->c1[k]);
        s->ap.mu[k] = s->mu[k];
        s->ap.w[k] = s->w[k];
        s->ap.inv_s2[k] = float(1.0 / (sg * sg));
        s->ap.inv_s3[k] = float(1.0 / (sg * sg * sg));
    }
}

// Enqueue the folded parameters (host copies) for the kernels, in stream
// order: steps already enqueued keep the old values.
int upload_params(cg_sim* s) {
    DeviceParams h;
    h.gp = s->gp;
    h.ap = s->ap;
    CG_CHECK(cudaMemcpyAsync(s->dparams, &h, sizeof(h), cudaMemcpyHostToDevice, s->stream),
             "uploading growth parameters");
    return CG_OK;
}

int recapture(cg_sim* s) {
    for (auto* set : {s->graph, s->graph8, s->graphR})
        for (int p = 0; p < 2; ++p)
            if (set[p]) {
                cudaGraphExecDestroy(set[p]);
                set[p] = nullptr;
            }
    return capture_graphs(s);
}

int ensure_backward(cg_sim* s) {
    if (s->bwd_ready) return CG_OK;
    CG_CHECK(s->ops->prepare_backward(), "configuring backward kernels");
    CG_CHECK(cudaMalloc(&s->abar, sizeof(float) * s->C * s->px()), "cudaMalloc(abar)");
    s->bwd_ready = true;
    return CG_OK;
}

BwdArgs bwd_args(cg_sim* s, const float* x, const float* ybar, float* xbar, double* pgrad,
                 float2* kgrad) {
    BwdArgs a{};
    a.C = s->C;
    a.K = s->K;
    a.temp = s->temp;
    a.x = x;
    a.ybar = ybar;
    a.xbar = xbar;
    a.abar = s->abar;
    a.rowspec = s->rowspec;
    a.kspec = s->kspec;
    a.kre = s->kreal_all ? s->kspec_re : nullptr;
    a.U = s->U;
    a.A = s->A;
    a.tw = s->tw;
    a.pgrad = pgrad;
    a.kgrad = kgrad;
    a.err = s->err;
    a.groups = s->groups;
    a.gp = &s->dparams->gp;
    a.ap = &s->dparams->ap;
    a.recompute = true;
    a.var = s->var;
    return a;
}

int ring_set(const cg_sim* s, const cg_ring_spec* specs, RingSet* rs, const char* who) {
    *rs = RingSet{};
    for (int k = 0; k < s->K; ++k) {
        const cg_ring_spec& r = specs[k];
        if (r.family != CG_RING_SHELL && r.family != CG_RING_GAUSS)
            return fail(CG_ERR_ARG, "%s: kernel %d: unknown ring family %d", who, k, r.family);
        if (r.family == CG_RING_SHELL && (r.rings < 1 || r.rings > CG_MAX_RINGS))
            return fail(CG_ERR_ARG, "%s: kernel %d: %d rings outside [1, %d]", who, k, r.rings,
                        CG_MAX_RINGS);
        if (!(r.radius > 0.f) || !std::isfinite(r.radius))
            return fail(CG_ERR_ARG, "%s: kernel %d: radius must be positive", who, k);
        if (r.family == CG_RING_GAUSS && (!(r.width > 0.f) || !std::isfinite(r.width)))
            return fail(CG_ERR_ARG, "%s: kernel %d: width must be positive", who, k);
        rs->family[k] = r.family;
        rs->rings[k] = r.family == CG_RING_SHELL ? r.rings : 1;
        rs->radius[k] = r.radius;
        rs->width[k] = r.width;
    }
    return CG_OK;
}

}  // namespace

extern "C" {

const char* cg_last_error(void) { return g_last_error.c_str(); }

const char* cg_version(void) { return "cella-gb300 0.1 (sm_103a)"; }

int cg_create(int n, int C, int K, const uint32_t* c0, const uint32_t* c1, const float* mu,
              const float* sigma, const float* weights, float temp, cg_stream_t stream,
              cg_sim** out) {
    if (!out) return fail(CG_ERR_ARG, "cg_create: out is NULL");
    *out = nullptr;
    int logn = 0;
    int rc0 = validate_world(n, C, K, c0, c1, mu, sigma, weights, temp, &logn);
    if (rc0 != CG_OK) return rc0;

    cg_sim* s = new (std::nothrow) cg_sim;
    if (!s) return fail(CG_ERR_OOM, "cg_create: host allocation failed");
    s->n = n;
    s->logn = logn;
    s->C = C;
    s->K = K;
    s->temp = temp;
    s->c0.assign(c0, c0 + K);
    s->c1.assign(c1, c1 + K);
    s->mu.assign(mu, mu + K);
    s->sigma.assign(sigma, sigma + K);
    s->w.assign(weights, weights + K);
    s->ops = size_ops(logn);

    build_groups(C, K, c0, c1, mu, sigma, weights, &s->groups, &s->gp);
    build_adjoint_params(s);

    int rc = CG_OK;
    auto chk = [&](cudaError_t e, const char* what) {
        if (rc == CG_OK && e != cudaSuccess) rc = cuda_fail(e, what);
        return rc == CG_OK;
    };
    chk(cudaGetDevice(&s->device), "cudaGetDevice");
    if (rc == CG_OK) {
        if (stream) {
            s->stream = static_cast<cudaStream_t>(stream);
        } else if (chk(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking),
                       "cudaStreamCreate")) {
            s->own_stream = true;
        }
    }
    const size_t px = s->px();
    const size_t half = size_t(n / 2) * n;
    if (rc == CG_OK) chk(s->ops->prepare(), "configuring kernels");
    if (rc == CG_OK) chk(cudaMalloc(&s->state[0], sizeof(float) * C * px), "cudaMalloc(state)");
    if (rc == CG_OK) chk(cudaMalloc(&s->state[1], sizeof(float) * C * px), "cudaMalloc(state)");
    if (rc == CG_OK) chk(cudaMalloc(&s->rowspec, sizeof(float2) * C * half), "cudaMalloc(rowspec)");
    if (rc == CG_OK)
        chk(cudaMalloc(&s->kspec, sizeof(float2) * K * (half + n)), "cudaMalloc(kspec)");
        chk(cudaMalloc(&s->kspec_re, sizeof(float) * K * (half + n)), "cudaMalloc(kspec_re)");
        s->kreal.assign(size_t(K), 0);
    if (rc == CG_OK) chk(cudaMalloc(&s->U, 2 * sizeof(float2) * K * half), "cudaMalloc(U)");
    if (rc == CG_OK) chk(cudaMalloc(&s->A, sizeof(float) * C * px), "cudaMalloc(A)");
    if (rc == CG_OK)
        chk(cudaMalloc(&s->tw, sizeof(float2) * s->ops->twiddle_count()), "cudaMalloc(twiddles)");
    if (rc == CG_OK) chk(cudaMalloc(&s->staging, sizeof(double) * px), "cudaMalloc(staging)");
    if (rc == CG_OK)
        chk(cudaMalloc(&s->mass_partial, sizeof(double) * C * kMassBlocks), "cudaMalloc(mass)");
    if (rc == CG_OK) chk(cudaMalloc(&s->mass_out, sizeof(double) * C), "cudaMalloc(mass)");
    if (rc == CG_OK) chk(cudaMalloc(&s->err, sizeof(int)), "cudaMalloc(err)");
    if (rc == CG_OK) chk(cudaMemset(s->err, 0, sizeof(int)), "memset(err)");
    if (rc == CG_OK) chk(cudaMalloc(&s->dparams, sizeof(DeviceParams)), "cudaMalloc(params)");
    if (rc == CG_OK) chk(cudaMalloc(&s->render, sizeof(unsigned) * px), "cudaMalloc(render)");
    if (rc == CG_OK) chk(cudaMalloc(&s->levels, 3 * px), "cudaMalloc(render levels)");
    if (rc == CG_OK) chk(cudaMemsetAsync(s->render, 0, sizeof(unsigned) * px, s->stream), "memset");
    if (rc == CG_OK)
        chk(cudaMalloc(&s->ring_partial, sizeof(double) * K * kRingBlocks * kMaxRings),
            "cudaMalloc(builder)");
    if (rc == CG_OK) chk(cudaMalloc(&s->ring_s, sizeof(double) * K * kMaxRings), "cudaMalloc(builder)");
    if (rc == CG_OK) chk(cudaMalloc(&s->zsum, sizeof(double) * K), "cudaMalloc(builder)");
    if (rc == CG_OK) chk(s->ops->prepare_builder(), "configuring builder kernels");
    if (rc == CG_OK) rc = upload_params(s);
    for (int i = 0; i < 4 && rc == CG_OK; ++i) chk(cudaEventCreate(&s->ev[i]), "cudaEventCreate");
    if (rc == CG_OK) chk(cudaMemsetAsync(s->state[0], 0, sizeof(float) * C * px, s->stream), "memset");
    if (rc == CG_OK) chk(cudaMemsetAsync(s->state[1], 0, sizeof(float) * C * px, s->stream), "memset");
    if (rc == CG_OK)
        chk(cudaMemsetAsync(s->kspec, 0, sizeof(float2) * K * (half + n), s->stream), "memset");
    if (rc == CG_OK) rc = build_twiddles(s);
    if (rc == CG_OK) rc = capture_graphs(s);
    if (rc == CG_OK) chk(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    if (rc != CG_OK) {
        release(s);
        return rc;
    }
    *out = s;
    return CG_OK;
}

int cg_destroy(cg_sim* s) {
    if (!s) return fail(CG_ERR_ARG, "cg_destroy: NULL handle");
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    release(s);
    return CG_OK;
}

}  // extern "C"

namespace {
// Record whether kernel k's spectrum is real (k < 0: every kernel not real);
// when the world's column pass changes between the real and the complex
// form, re-capture the step graphs.
int set_kernel_realness(cg_sim* s, int k, bool real) {
    if (k >= 0) s->kreal[size_t(k)] = real ? 1 : 0;
    else std::fill(s->kreal.begin(), s->kreal.end(), uint8_t(0));
    bool all = true;
    for (uint8_t r : s->kreal) all = all && r != 0;
    if (all == s->kreal_all) return CG_OK;
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    s->kreal_all = all;
    return recapture(s);
}
}  // namespace

extern "C" {

int cg_set_kernel(cg_sim* s, int k, const float* spec) {
    if (!s || !spec) return fail(CG_ERR_ARG, "cg_set_kernel: NULL argument");
    if (k < 0 || k >= s->K) return fail(CG_ERR_ARG, "kernel index %d outside [0, %d)", k, s->K);
    const size_t half = size_t(s->n / 2) * s->n;
    const bool real = hermitian_part_is_real(spec, s->n);
    CG_CHECK(cudaMemcpyAsync(s->staging, spec, sizeof(float2) * s->px(), cudaMemcpyHostToDevice,
                             s->stream),
             "uploading kernel spectrum");
    float2* packed = s->kspec + size_t(k) * (half + s->n);
    CG_CHECK(s->ops->pack(static_cast<const float2*>(s->staging), packed, s->stream),
             "packing kernel spectrum");
    if (real)
        CG_CHECK(launch_real_parts(packed, s->kspec_re + size_t(k) * (half + s->n), half + s->n,
                                   s->stream),
                 "keeping the real parts");
    return set_kernel_realness(s, k, real);
}

int cg_kernels_real(cg_sim* s, int* real) {
    if (!s || !real) return fail(CG_ERR_ARG, "cg_kernels_real: NULL argument");
    *real = s->kreal_all ? 1 : 0;
    return CG_OK;
}

int cg_set_kernel_device(cg_sim* s, int k, const float* dev_spec) {
    if (!s || !dev_spec) return fail(CG_ERR_ARG, "cg_set_kernel_device: NULL argument");
    if (!aligned16(dev_spec)) return misaligned("cg_set_kernel_device");
    if (k < 0 || k >= s->K) return fail(CG_ERR_ARG, "kernel index %d outside [0, %d)", k, s->K);
    const size_t half = size_t(s->n / 2) * s->n;
    CG_CHECK(s->ops->pack(reinterpret_cast<const float2*>(dev_spec),
                          s->kspec + size_t(k) * (half + s->n), s->stream),
             "packing kernel spectrum");
    // device spectra are not inspected: the column pass keeps the complex form
    return set_kernel_realness(s, k, false);
}

int cg_upload_channel(cg_sim* s, int c, const double* data) {
    if (!s || !data) return fail(CG_ERR_ARG, "cg_upload_channel: NULL argument");
    if (c < 0 || c >= s->C) return fail(CG_ERR_ARG, "channel index %d outside [0, %d)", c, s->C);
    CG_CHECK(cudaMemcpyAsync(s->staging, data, sizeof(double) * s->px(), cudaMemcpyHostToDevice,
                             s->stream),
             "uploading channel");
    CG_CHECK(launch_f64_to_f32(static_cast<const double*>(s->staging),
                               s->state[s->cur] + size_t(c) * s->px(), s->px(), s->stream),
             "converting channel");
    return CG_OK;
}

int cg_upload_channel_f32(cg_sim* s, int c, const float* data) {
    if (!s || !data) return fail(CG_ERR_ARG, "cg_upload_channel_f32: NULL argument");
    if (c < 0 || c >= s->C) return fail(CG_ERR_ARG, "channel index %d outside [0, %d)", c, s->C);
    CG_CHECK(cudaMemcpyAsync(s->state[s->cur] + size_t(c) * s->px(), data, sizeof(float) * s->px(),
                             cudaMemcpyHostToDevice, s->stream),
             "uploading channel");
    return CG_OK;
}

int cg_step(cg_sim* s, int nsteps) {
    if (!s) return fail(CG_ERR_ARG, "cg_step: NULL handle");
    if (nsteps < 0) return fail(CG_ERR_ARG, "negative step count %d", nsteps);
    int left = nsteps;
    while (left >= kStepsPerGraph) {   // an even count: the parity is unchanged
        CG_CHECK(cudaGraphLaunch(s->graph8[s->cur], s->stream), "cudaGraphLaunch");
        left -= kStepsPerGraph;
    }
    for (; left > 0; --left) {
        CG_CHECK(cudaGraphLaunch(s->graph[s->cur], s->stream), "cudaGraphLaunch");
        s->cur ^= 1;
    }
    return CG_OK;
}

int cg_iterate(cg_sim* s) { return cg_step(s, 1); }

int cg_iterate_and_render(cg_sim* s) {
    if (!s) return fail(CG_ERR_ARG, "cg_iterate_and_render: NULL handle");
    CG_CHECK(cudaGraphLaunch(s->graphR[s->cur], s->stream), "cudaGraphLaunch");
    s->cur ^= 1;
    return CG_OK;
}

int cg_render(cg_sim* s) {
    if (!s) return fail(CG_ERR_ARG, "cg_render: NULL handle");
    CG_CHECK(launch_render(s->state[s->cur], s->C, s->px(), s->render, s->stream),
             "launching render");
    return CG_OK;
}

// Write all of buf to fd (a file or a pipe), retrying short writes.
static bool write_all(int fd, const unsigned char* buf, size_t bytes) {
    while (bytes > 0) {
        const ssize_t w = ::write(fd, buf, bytes);
        if (w < 0) {
            if (errno == EINTR) continue;
            return false;
        }
        buf += w;
        bytes -= size_t(w);
    }
    return true;
}

int cg_stream_frames(cg_sim* s, int fd, int nframes, int steps_per_frame) {
    if (!s) return fail(CG_ERR_ARG, "cg_stream_frames: NULL handle");
    if (fd < 0 || nframes < 0 || steps_per_frame < 1)
        return fail(CG_ERR_ARG, "cg_stream_frames: fd %d, %d frames, %d steps per frame", fd,
                    nframes, steps_per_frame);
    const size_t bytes = 3 * s->px();
    for (int i = 0; i < 2; ++i) {
        if (!s->frames[i])
            CG_CHECK(cudaMallocHost(reinterpret_cast<void**>(&s->frames[i]), bytes),
                     "cudaMallocHost(frames)");
        if (!s->frame_ev[i])
            CG_CHECK(cudaEventCreateWithFlags(&s->frame_ev[i], cudaEventDisableTiming),
                     "cudaEventCreate");
    }
    auto* dev_rgb = static_cast<unsigned char*>(s->staging);   // 8 B per pixel, 3 used
    // Frame f is enqueued (its steps, the render levels and words, the RGB24
    // conversion and the copy into host buffer f % 2) before frame f - 1 is
    // written out, so the GPU computes while the host writes.
    for (int f = 0; f <= nframes; ++f) {
        if (f < nframes) {
            int rc = cg_step(s, steps_per_frame - 1);
            if (rc == CG_OK) rc = cg_iterate_and_render(s);
            if (rc != CG_OK) return rc;
            CG_CHECK(launch_rgb24(s->render, dev_rgb, s->px(), s->stream), "launching RGB24");
            CG_CHECK(cudaMemcpyAsync(s->frames[f & 1], dev_rgb, bytes, cudaMemcpyDeviceToHost,
                                     s->stream),
                     "downloading a frame");
            CG_CHECK(cudaEventRecord(s->frame_ev[f & 1], s->stream), "cudaEventRecord");
        }
        if (f > 0) {
            const int b = (f - 1) & 1;
            CG_CHECK(cudaEventSynchronize(s->frame_ev[b]), "cudaEventSynchronize");
            if (!write_all(fd, s->frames[b], bytes)) {
                cudaStreamSynchronize(s->stream);
                return fail(CG_ERR_IO, "writing frame %d to fd %d failed (errno %d)", f - 1, fd,
                            errno);
            }
        }
    }
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_download_render(cg_sim* s, uint8_t* rgb24) {
    if (!s || !rgb24) return fail(CG_ERR_ARG, "cg_download_render: NULL argument");
    auto* bytes = static_cast<unsigned char*>(s->staging);   // 8 B per pixel, 3 used
    CG_CHECK(launch_rgb24(s->render, bytes, s->px(), s->stream), "launching RGB24 conversion");
    CG_CHECK(cudaMemcpyAsync(rgb24, bytes, 3 * s->px(), cudaMemcpyDeviceToHost, s->stream),
             "downloading render");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_download_render_packed(cg_sim* s, uint32_t* out) {
    if (!s || !out) return fail(CG_ERR_ARG, "cg_download_render_packed: NULL argument");
    CG_CHECK(cudaMemcpyAsync(out, s->render, sizeof(uint32_t) * s->px(), cudaMemcpyDeviceToHost,
                             s->stream),
             "downloading render");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_render_ptr(cg_sim* s, const uint32_t** out) {
    if (!s || !out) return fail(CG_ERR_ARG, "cg_render_ptr: NULL argument");
    *out = s->render;
    return CG_OK;
}

int cg_iterate_on(cg_sim* s, cg_stream_t stream) {
    if (!s) return fail(CG_ERR_ARG, "cg_iterate_on: NULL handle");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->stream;
    CG_CHECK(cudaGraphLaunch(s->graph[s->cur], st), "cudaGraphLaunch");
    s->cur ^= 1;
    return CG_OK;
}

int cg_download_channels(cg_sim* s, float* out) {
    if (!s || !out) return fail(CG_ERR_ARG, "cg_download_channels: NULL argument");
    CG_CHECK(cudaMemcpyAsync(out, s->state[s->cur], sizeof(float) * s->C * s->px(),
                             cudaMemcpyDeviceToHost, s->stream),
             "downloading channels");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    CG_SYNC_CHECK(s);
    return CG_OK;
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister): the pipeline's
// copies must not block on a pageable staging copy.
static bool page_locked(const void* ptr) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

static int ensure_pipe(cg_sim* s) {
    HostPipe& p = s->pipe;
    if (p.ready) return CG_OK;
    const size_t bytes = sizeof(double) * s->C * s->px();
    if (!p.up) CG_CHECK(cudaStreamCreateWithFlags(&p.up, cudaStreamNonBlocking), "creating a stream");
    if (!p.down)
        CG_CHECK(cudaStreamCreateWithFlags(&p.down, cudaStreamNonBlocking), "creating a stream");
    for (auto& b : p.stage)
        if (!b) CG_CHECK(cudaMalloc(&b, bytes), "cudaMalloc(host pipeline staging)");
    for (auto* e : {&p.up_done[0], &p.up_done[1], &p.conv_done[0], &p.conv_done[1], &p.step_done,
                    &p.down_done})
        if (!*e) CG_CHECK(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "creating an event");
    p.ready = true;
    return CG_OK;
}

int cg_step_host_async(cg_sim* s, const double* in, float* out, int nsteps) {
    if (!s || !in || !out) return fail(CG_ERR_ARG, "cg_step_host_async: NULL argument");
    if (nsteps < 0) return fail(CG_ERR_ARG, "negative step count %d", nsteps);
    if (!page_locked(in) || !page_locked(out))
        return fail(CG_ERR_ARG, "cg_step_host_async: host buffers must be page-locked "
                                "(cudaHostAlloc or cudaHostRegister)");
    int rc = ensure_pipe(s);
    if (rc != CG_OK) return rc;
    HostPipe& p = s->pipe;
    const int b = p.slot;
    p.slot ^= 1;
    const size_t count = size_t(s->C) * s->px();
    // upload into staging slot b once the conversion of two calls ago has read it
    CG_CHECK(cudaStreamWaitEvent(p.up, p.conv_done[b], 0), "cudaStreamWaitEvent");
    CG_CHECK(cudaMemcpyAsync(p.stage[b], in, sizeof(double) * count, cudaMemcpyHostToDevice, p.up),
             "uploading channels");
    CG_CHECK(cudaEventRecord(p.up_done[b], p.up), "cudaEventRecord");
    // convert and step in the sim's stream (already ordered after the
    // previous call's download)
    CG_CHECK(cudaStreamWaitEvent(s->stream, p.up_done[b], 0), "cudaStreamWaitEvent");
    CG_CHECK(launch_f64_to_f32(p.stage[b], s->state[s->cur], count, s->stream),
             "converting channels");
    CG_CHECK(cudaEventRecord(p.conv_done[b], s->stream), "cudaEventRecord");
    rc = cg_step(s, nsteps);
    if (rc != CG_OK) return rc;
    CG_CHECK(cudaEventRecord(p.step_done, s->stream), "cudaEventRecord");
    // download, then order everything later in the sim's stream after it
    CG_CHECK(cudaStreamWaitEvent(p.down, p.step_done, 0), "cudaStreamWaitEvent");
    CG_CHECK(cudaMemcpyAsync(out, s->state[s->cur], sizeof(float) * count, cudaMemcpyDeviceToHost,
                             p.down),
             "downloading channels");
    CG_CHECK(cudaEventRecord(p.down_done, p.down), "cudaEventRecord");
    CG_CHECK(cudaStreamWaitEvent(s->stream, p.down_done, 0), "cudaStreamWaitEvent");
    return CG_OK;
}

int cg_host_wait(cg_sim* s) {
    if (!s) return fail(CG_ERR_ARG, "cg_host_wait: NULL handle");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    if (s->pipe.ready) {
        CG_CHECK(cudaStreamSynchronize(s->pipe.down), "cudaStreamSynchronize");
        CG_CHECK(cudaStreamSynchronize(s->pipe.up), "cudaStreamSynchronize");
    }
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_download_conv_real(cg_sim* s, float* out) {
    if (!s || !out) return fail(CG_ERR_ARG, "cg_download_conv_real: NULL argument");
    float* dbg = nullptr;
    CG_CHECK(cudaMallocAsync(reinterpret_cast<void**>(&dbg), sizeof(float) * s->K * s->px(), s->stream),
             "cudaMallocAsync(conv)");
    cudaError_t e = s->ops->step(s->args(s->cur, dbg), kPhaseRowFwd | kPhaseColConv | kPhaseGrowth,
                                 s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, dbg, sizeof(float) * s->K * s->px(), cudaMemcpyDeviceToHost,
                            s->stream);
    cudaFreeAsync(dbg, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "computing the convolution buffer");
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_download_affinity(cg_sim* s, float* out) {
    if (!s || !out) return fail(CG_ERR_ARG, "cg_download_affinity: NULL argument");
    CG_CHECK(s->ops->step(s->args(s->cur, nullptr), kPhaseRowFwd | kPhaseColConv | kPhaseGrowth,
                          s->stream),
             "computing the affinity");
    CG_CHECK(cudaMemcpyAsync(out, s->A, sizeof(float) * s->C * s->px(), cudaMemcpyDeviceToHost,
                             s->stream),
             "downloading the affinity");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_timed_iterate(cg_sim* s, double ms[4]) {
    if (!s || !ms) return fail(CG_ERR_ARG, "cg_timed_iterate: NULL argument");
    const StepArgs a = s->args(s->cur, nullptr);
    const int phases[3] = {kPhaseRowFwd | kPhaseColConv, kPhaseGrowth, kPhaseDiffusion};
    CG_CHECK(cudaEventRecord(s->ev[0], s->stream), "cudaEventRecord");
    for (int p = 0; p < 3; ++p) {
        CG_CHECK(s->ops->step(a, phases[p], s->stream), "launching a phase");
        CG_CHECK(cudaEventRecord(s->ev[p + 1], s->stream), "cudaEventRecord");
    }
    CG_CHECK(cudaEventSynchronize(s->ev[3]), "cudaEventSynchronize");
    for (int p = 0; p < 3; ++p) {
        float t = 0.f;
        CG_CHECK(cudaEventElapsedTime(&t, s->ev[p], s->ev[p + 1]), "cudaEventElapsedTime");
        ms[p] = t;
    }
    ms[3] = 0.0;
    s->cur ^= 1;
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_profile_kernels(cg_sim* s, int nsteps, double ms[4]) {
    if (!s || !ms) return fail(CG_ERR_ARG, "cg_profile_kernels: NULL argument");
    if (nsteps < 1 || nsteps > 1024)
        return fail(CG_ERR_ARG, "cg_profile_kernels: nsteps %d outside [1, 1024]", nsteps);
    const int phases[4] = {kPhaseRowFwd, kPhaseColConv, kPhaseGrowth, kPhaseDiffusion};
    std::vector<cudaEvent_t> ev(size_t(nsteps) * 5, nullptr);
    int rc = CG_OK;
    for (auto& e : ev) {
        cudaError_t ce = cudaEventCreate(&e);
        if (ce != cudaSuccess) {
            rc = cuda_fail(ce, "cudaEventCreate");
            break;
        }
    }
    for (int i = 0; i < nsteps && rc == CG_OK; ++i) {
        const StepArgs a = s->args(s->cur, nullptr);
        cudaError_t ce = cudaEventRecord(ev[i * 5], s->stream);
        for (int p = 0; p < 4 && ce == cudaSuccess; ++p) {
            ce = s->ops->step(a, phases[p], s->stream);
            if (ce == cudaSuccess) ce = cudaEventRecord(ev[i * 5 + p + 1], s->stream);
        }
        if (ce != cudaSuccess) rc = cuda_fail(ce, "profiling a step");
        s->cur ^= 1;
    }
    if (rc == CG_OK) {
        cudaError_t ce = cudaEventSynchronize(ev.back());
        if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaEventSynchronize");
    }
    double acc[4] = {0, 0, 0, 0};
    for (int i = 0; i < nsteps && rc == CG_OK; ++i)
        for (int p = 0; p < 4; ++p) {
            float t = 0.f;
            cudaError_t ce = cudaEventElapsedTime(&t, ev[i * 5 + p], ev[i * 5 + p + 1]);
            if (ce != cudaSuccess) {
                rc = cuda_fail(ce, "cudaEventElapsedTime");
                break;
            }
            acc[p] += t;
        }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    if (rc == CG_OK)
        for (int p = 0; p < 4; ++p) ms[p] = acc[p] / nsteps;
    if (rc == CG_OK) rc = check_device_error(s);
    return rc;
}

int cg_mass_f64(cg_sim* s, double* out) {
    if (!s || !out) return fail(CG_ERR_ARG, "cg_mass_f64: NULL argument");
    CG_CHECK(launch_mass_f64(s->state[s->cur], s->C, s->px(), s->mass_partial, kMassBlocks,
                             s->mass_out, s->stream),
             "mass reduction");
    CG_CHECK(cudaMemcpyAsync(out, s->mass_out, sizeof(double) * s->C, cudaMemcpyDeviceToHost,
                             s->stream),
             "downloading masses");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    CG_SYNC_CHECK(s);
    return CG_OK;
}

int cg_channel_ptr(cg_sim* s, float** p) {
    if (!s || !p) return fail(CG_ERR_ARG, "cg_channel_ptr: NULL argument");
    *p = s->state[s->cur];
    return CG_OK;
}

int cg_stream(cg_sim* s, cg_stream_t* out) {
    if (!s || !out) return fail(CG_ERR_ARG, "cg_stream: NULL argument");
    *out = s->stream;
    return CG_OK;
}

int cg_set_params(cg_sim* s, const float* mu, const float* sigma, const float* weights,
                  float temp) {
    if (!s) return fail(CG_ERR_ARG, "cg_set_params: NULL handle");
    int logn = 0;
    int rc = validate_world(s->n, s->C, s->K, s->c0.data(), s->c1.data(), mu, sigma, weights,
                            temp, &logn);
    if (rc != CG_OK) return rc;
    s->mu.assign(mu, mu + s->K);
    s->sigma.assign(sigma, sigma + s->K);
    s->w.assign(weights, weights + s->K);
    build_groups(s->C, s->K, s->c0.data(), s->c1.data(), mu, sigma, weights, &s->groups, &s->gp);
    build_adjoint_params(s);
    rc = upload_params(s);
    if (rc != CG_OK || temp == s->temp) return rc;
    // temp is a launch argument of the captured graphs
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    s->temp = temp;
    return recapture(s);
}

int cg_build_ring_kernels(cg_sim* s, const cg_ring_spec* specs, const float* dev_ring_weights) {
    if (!s || !specs) return fail(CG_ERR_ARG, "cg_build_ring_kernels: NULL argument");
    RingSet rs;
    int rc = ring_set(s, specs, &rs, "cg_build_ring_kernels");
    if (rc != CG_OK) return rc;
    // scratch: the two halves of U (free between steps, in stream order)
    const size_t half = size_t(s->n / 2) * s->n;
    float2* rows = s->U;
    float* h = reinterpret_cast<float*>(s->U + size_t(s->K) * half);
    CG_CHECK(launch_ring_build(s->n, s->K, rs, dev_ring_weights, h, s->ring_partial, s->ring_s,
                               s->zsum, s->stream),
             "launching the ring builder");
    StepArgs a = s->args(s->cur, nullptr);
    a.C = s->K;   // the kernels pass through the row transform as channels
    a.x_in = h;
    a.rowspec = rows;
    CG_CHECK(s->ops->step(a, kPhaseRowFwd, s->stream), "launching the builder's row transform");
    CG_CHECK(s->ops->kspec_cols(rows, s->kspec, s->tw, s->zsum, s->K, s->stream),
             "launching the builder's column transform");
    // spectra built on the device keep the complex column pass
    return set_kernel_realness(s, -1, false);
}

int cg_set_kernels_spatial_device(cg_sim* s, const float* dev_h) {
    if (!s || !dev_h) return fail(CG_ERR_ARG, "cg_set_kernels_spatial_device: NULL argument");
    // the builder's scratch (the second half of U) holds an aligned copy for
    // the row transform, as cg_build_ring_kernels' builder output does
    const size_t half = size_t(s->n / 2) * s->n;
    float2* rows = s->U;
    float* h = reinterpret_cast<float*>(s->U + size_t(s->K) * half);
    CG_CHECK(cudaMemcpyAsync(h, dev_h, sizeof(float) * size_t(s->K) * s->px(),
                             cudaMemcpyDeviceToDevice, s->stream),
             "copying the spatial kernels");
    StepArgs a = s->args(s->cur, nullptr);
    a.C = s->K;   // the kernels pass through the row transform as channels
    a.x_in = h;
    a.rowspec = rows;
    CG_CHECK(s->ops->step(a, kPhaseRowFwd, s->stream), "launching the builder's row transform");
    CG_CHECK(s->ops->kspec_cols(rows, s->kspec, s->tw, nullptr, s->K, s->stream),
             "launching the builder's column transform");
    return set_kernel_realness(s, -1, false);
}

int cg_ring_weight_grad(cg_sim* s, const cg_ring_spec* specs, const float* dev_ring_weights,
                        const float* dev_hbar, float* dev_grad) {
    if (!s || !specs || !dev_hbar || !dev_grad)
        return fail(CG_ERR_ARG, "cg_ring_weight_grad: NULL argument");
    if (!aligned16(dev_hbar)) return misaligned("cg_ring_weight_grad");
    RingSet rs;
    int rc = ring_set(s, specs, &rs, "cg_ring_weight_grad");
    if (rc != CG_OK) return rc;
    CG_CHECK(launch_ring_grad(s->n, s->K, rs, dev_ring_weights, dev_hbar, s->ring_partial,
                              s->ring_s, s->zsum, dev_grad, s->stream),
             "launching the ring-weight gradient");
    return CG_OK;
}

int cg_set_params_device(cg_sim* s, const float* dev_mu, const float* dev_sigma,
                         const float* dev_weights) {
    if (!s || !dev_mu || !dev_sigma || !dev_weights)
        return fail(CG_ERR_ARG, "cg_set_params_device: NULL argument");
    CG_CHECK(launch_fold_params(dev_mu, dev_sigma, dev_weights, s->C, s->K, s->groups, s->dparams,
                                s->stream),
             "launching parameter folding");
    return CG_OK;
}

int cg_step_from(cg_sim* s, const float* x_in, float* x_out) {
    if (!s || !x_in || !x_out) return fail(CG_ERR_ARG, "cg_step_from: NULL argument");
    if (x_in == x_out) return fail(CG_ERR_ARG, "cg_step_from: input and output must differ");
    if (!aligned16(x_in) || !aligned16(x_out)) return misaligned("cg_step_from");
    StepArgs a = s->args(s->cur, nullptr);
    a.x_in = x_in;
    a.x_out = x_out;
    CG_CHECK(s->ops->step(a, kPhaseAll, s->stream), "launching a step");
    return CG_OK;
}

int cg_step_backward(cg_sim* s, const float* x, const float* ybar, float* xbar, double* pgrad,
                     float* kgrad) {
    if (!s || !x || !ybar || !xbar || !pgrad)
        return fail(CG_ERR_ARG, "cg_step_backward: NULL argument");
    if (xbar == ybar || xbar == x)
        return fail(CG_ERR_ARG, "cg_step_backward: xbar must not alias x or ybar");
    if (!aligned16(x) || !aligned16(ybar) || !aligned16(xbar) || !aligned16(kgrad))
        return misaligned("cg_step_backward");
    int rc = ensure_backward(s);
    if (rc != CG_OK) return rc;
    CG_CHECK(s->ops->backward(bwd_args(s, x, ybar, xbar, pgrad, reinterpret_cast<float2*>(kgrad)),
                              s->stream),
             "launching a backward step");
    return CG_OK;
}

int cg_check_bounded_wait(cg_sim* s, int timeout_ms) {
    if (!s) return fail(CG_ERR_ARG, "cg_check_bounded_wait: NULL handle");
    if (timeout_ms < 1 || timeout_ms > 2000)
        return fail(CG_ERR_ARG, "cg_check_bounded_wait: timeout %d ms outside [1, 2000]", timeout_ms);
    CG_CHECK(launch_wait_check(s->err, timeout_ms, s->stream), "launching the wait check");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    return check_device_error(s);   // CG_ERR_TIMEOUT, and the word is cleared
}

int cg_zero_grads(cg_sim* s, double* pgrad, float* kgrad) {
    if (!s || !pgrad) return fail(CG_ERR_ARG, "cg_zero_grads: NULL argument");
    CG_CHECK(cudaMemsetAsync(pgrad, 0, sizeof(double) * 3 * s->K, s->stream), "zeroing pgrad");
    if (kgrad)
        CG_CHECK(cudaMemsetAsync(kgrad, 0, sizeof(float2) * s->K * (size_t(s->n / 2) * s->n),
                                 s->stream),
                 "zeroing kgrad");
    return CG_OK;
}

int cg_kernel_grad_spatial(cg_sim* s, float* kgrad, float* hbar) {
    if (!s || !kgrad || !hbar) return fail(CG_ERR_ARG, "cg_kernel_grad_spatial: NULL argument");
    if (!aligned16(kgrad) || !aligned16(hbar)) return misaligned("cg_kernel_grad_spatial");
    int rc = ensure_backward(s);
    if (rc != CG_OK) return rc;
    CG_CHECK(s->ops->kgrad_final(reinterpret_cast<float2*>(kgrad), hbar, s->K, s->tw, s->stream),
             "finishing the kernel gradient");
    return CG_OK;
}

int cg_unroll(cg_sim* s, const float* x0, int T, int every, float* ckpt, float* xT) {
    if (!s || !x0 || !ckpt || !xT) return fail(CG_ERR_ARG, "cg_unroll: NULL argument");
    if (T < 1 || every < 1) return fail(CG_ERR_ARG, "cg_unroll: T=%d, every=%d", T, every);
    if (!aligned16(x0) || !aligned16(ckpt) || !aligned16(xT)) return misaligned("cg_unroll");
    const size_t bytes = sizeof(float) * s->C * s->px();
    const size_t plane = size_t(s->C) * s->px();
    for (auto& p : s->utmp)
        if (!p) CG_CHECK(cudaMalloc(&p, bytes), "cudaMalloc(unroll scratch)");
    // checkpoint j holds x_{j*every}, j = 0 .. (T-1)/every
    CG_CHECK(cudaMemcpyAsync(ckpt, x0, bytes, cudaMemcpyDeviceToDevice, s->stream), "checkpoint");
    const float* cur = x0;
    for (int t = 0; t < T; ++t) {
        float* nxt;
        if (t + 1 == T) nxt = xT;
        else if ((t + 1) % every == 0) nxt = ckpt + plane * size_t((t + 1) / every);
        else nxt = s->utmp[(t + 1) & 1];
        int rc = cg_step_from(s, cur, nxt);
        if (rc != CG_OK) return rc;
        cur = nxt;
    }
    return CG_OK;
}

int cg_unroll_backward(cg_sim* s, const float* ckpt, int T, int every, const float* gT, float* g0,
                       double* pgrad, float* kgrad, float* seg, float* gtmp) {
    if (!s || !ckpt || !gT || !g0 || !pgrad || !seg || !gtmp)
        return fail(CG_ERR_ARG, "cg_unroll_backward: NULL argument");
    if (T < 1 || every < 1) return fail(CG_ERR_ARG, "cg_unroll_backward: T=%d, every=%d", T, every);
    if (!aligned16(ckpt) || !aligned16(gT) || !aligned16(g0) || !aligned16(kgrad) ||
        !aligned16(seg) || !aligned16(gtmp))
        return misaligned("cg_unroll_backward");
    int rc = ensure_backward(s);
    if (rc != CG_OK) return rc;
    const size_t bytes = sizeof(float) * s->C * s->px();
    const size_t plane = size_t(s->C) * s->px();
    const size_t half = size_t(s->n / 2) * s->n;
    // per cached step: row spectra (C half planes), U (K half planes), A
    const size_t spec_elems = size_t(s->C) * half, u_elems = size_t(s->K) * half;
    const size_t step_bytes = sizeof(float2) * (spec_elems + u_elems) + bytes;
    const int span = std::min(every, T);
    if (s->cache_steps < span) {
        cudaFree(s->seg_cache);
        s->seg_cache = nullptr;
        s->cache_steps = 0;
        CG_CHECK(cudaMalloc(&s->seg_cache, step_bytes * size_t(span)),
                 "cudaMalloc(segment cache)");
        s->cache_steps = span;
    }
    auto slot = [&](int i, float2** rowspec, float2** U, float** A) {
        char* base = static_cast<char*>(s->seg_cache) + step_bytes * size_t(i);
        *rowspec = reinterpret_cast<float2*>(base);
        *U = *rowspec + spec_elems;
        *A = reinterpret_cast<float*>(*U + u_elems);
    };
    // gradient ping-pong between g0 and gtmp, arranged to end in g0
    float* gb[2] = {(T % 2 == 0) ? g0 : gtmp, (T % 2 == 0) ? gtmp : g0};
    CG_CHECK(cudaMemcpyAsync(gb[0], gT, bytes, cudaMemcpyDeviceToDevice, s->stream), "gradient");
    int which = 0;
    const int nseg = (T + every - 1) / every;
    for (int j = nseg - 1; j >= 0; --j) {
        const int t0 = j * every, t1 = std::min(T, t0 + every);
        // recompute x_{t0} .. x_{t1-1} into seg, keeping each step's row
        // spectra, U and A for its backward step (the last step needs no
        // diffusion)
        CG_CHECK(cudaMemcpyAsync(seg, ckpt + plane * size_t(j), bytes, cudaMemcpyDeviceToDevice,
                                 s->stream),
                 "segment");
        for (int t = t0; t < t1; ++t) {
            StepArgs a = s->args(s->cur, nullptr);
            slot(t - t0, &a.rowspec, &a.U, &a.A);
            a.x_in = seg + plane * size_t(t - t0);
            const bool last = t + 1 == t1;
            a.x_out = last ? nullptr : seg + plane * size_t(t - t0 + 1);
            CG_CHECK(s->ops->step(a, last ? (kPhaseRowFwd | kPhaseColConv | kPhaseGrowth) : kPhaseAll,
                                  s->stream),
                     "recomputing a segment");
        }
        for (int t = t1 - 1; t >= t0; --t) {
            BwdArgs b = bwd_args(s, seg + plane * size_t(t - t0), gb[which], gb[which ^ 1], pgrad,
                                 reinterpret_cast<float2*>(kgrad));
            slot(t - t0, &b.rowspec, &b.U, &b.A);
            b.recompute = false;
            CG_CHECK(s->ops->backward(b, s->stream), "launching a backward step");
            which ^= 1;
        }
    }
    return CG_OK;
}

int cg_set_variants(cg_sim* s, const int v[4]) {
    if (!s || !v) return fail(CG_ERR_ARG, "cg_set_variants: NULL argument");
    for (int p = 0; p < 4; ++p)
        if (v[p] < 0 || v[p] >= phase_variant_count(s->logn, p))
            return fail(CG_ERR_ARG, "variant %d of phase %d outside [0, %d] at grid side %d", v[p],
                        p, phase_variant_count(s->logn, p) - 1, s->n);
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    s->var.r2c = v[0];
    s->var.col = v[1];
    s->var.c2r = v[2];
    s->var.diff = v[3];
    return recapture(s);
}

int cg_get_variants(cg_sim* s, int v[4]) {
    if (!s || !v) return fail(CG_ERR_ARG, "cg_get_variants: NULL argument");
    v[0] = s->var.r2c;
    v[1] = s->var.col;
    v[2] = s->var.c2r;
    v[3] = s->var.diff;
    return CG_OK;
}

int cg_autotune(cg_sim* s, int reps, double ms_out[4 * CG_MAX_VARIANTS], int chosen[4]) {
    static_assert(CG_MAX_VARIANTS == kMaxVariants, "variant count");
    if (!s) return fail(CG_ERR_ARG, "cg_autotune: NULL handle");
    if (reps < 1 || reps > 1000) return fail(CG_ERR_ARG, "cg_autotune: reps %d outside [1, 1000]", reps);
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    const int phases[4] = {kPhaseRowFwd, kPhaseColConv, kPhaseGrowth, kPhaseDiffusion};
    double ms[4][kMaxVariants];
    int best[4];
    // Every phase reads the current state or the scratch the previous phase
    // wrote; running them in order on the live handle leaves the state
    // untouched (diffusion writes the spare ping-pong buffer only).
    for (int p = 0; p < 4; ++p) {
        best[p] = 0;
        for (int v = 0; v < kMaxVariants; ++v) ms[p][v] = -1.0;
        for (int v = 0; v < phase_variant_count(s->logn, p); ++v) {
            Variants var = s->var;
            int* slot[4] = {&var.r2c, &var.col, &var.c2r, &var.diff};
            *slot[p] = v;
            StepArgs a = s->args(s->cur, nullptr);
            a.var = var;
            for (int q = 0; q < p; ++q)   // inputs of phase p
                CG_CHECK(s->ops->step(a, phases[q], s->stream), "autotune prologue");
            CG_CHECK(s->ops->step(a, phases[p], s->stream), "autotune warm-up");
            CG_CHECK(cudaEventRecord(s->ev[0], s->stream), "cudaEventRecord");
            for (int r = 0; r < reps; ++r)
                CG_CHECK(s->ops->step(a, phases[p], s->stream), "autotune launch");
            CG_CHECK(cudaEventRecord(s->ev[1], s->stream), "cudaEventRecord");
            CG_CHECK(cudaEventSynchronize(s->ev[1]), "cudaEventSynchronize");
            float t = 0.f;
            CG_CHECK(cudaEventElapsedTime(&t, s->ev[0], s->ev[1]), "cudaEventElapsedTime");
            ms[p][v] = double(t) / reps;
            if (ms[p][v] < ms[p][best[p]]) best[p] = v;
        }
    }
    int rc = check_device_error(s);
    if (rc != CG_OK) return rc;
    if (ms_out)
        for (int p = 0; p < 4; ++p)
            for (int v = 0; v < kMaxVariants; ++v) ms_out[p * kMaxVariants + v] = ms[p][v];
    if (chosen)
        for (int p = 0; p < 4; ++p) chosen[p] = best[p];
    s->var.r2c = best[0];
    s->var.col = best[1];
    s->var.c2r = best[2];
    s->var.diff = best[3];
    // then the graph layout: each layout's graph of kStepsPerGraph steps,
    // all reading the current state (nothing steps), replayed reps times
    double lay_ms[2] = {0.0, 0.0};
    for (int l = 0; l < 2; ++l) {
        s->layout = l;
        cudaGraphExec_t ge = nullptr;
        cudaError_t e = capture_steps(s, s->cur, kStepsPerGraph, false, &ge, true);
        if (e == cudaSuccess) e = cudaGraphLaunch(ge, s->stream);   // warm-up
        if (e == cudaSuccess) e = cudaEventRecord(s->ev[0], s->stream);
        for (int r = 0; r < reps && e == cudaSuccess; ++r) e = cudaGraphLaunch(ge, s->stream);
        if (e == cudaSuccess) e = cudaEventRecord(s->ev[1], s->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(s->ev[1]);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, s->ev[0], s->ev[1]);
        if (ge) cudaGraphExecDestroy(ge);
        if (e != cudaSuccess) return cuda_fail(e, "timing a graph layout");
        lay_ms[l] = double(t) / reps / kStepsPerGraph;
    }
    s->layout = lay_ms[1] < lay_ms[0] ? 1 : 0;
    rc = check_device_error(s);
    if (rc != CG_OK) return rc;
    return recapture(s);
}

int cg_set_graph_layout(cg_sim* s, int layout) {
    if (!s) return fail(CG_ERR_ARG, "cg_set_graph_layout: NULL handle");
    if (layout < 0 || layout > 1) return fail(CG_ERR_ARG, "graph layout %d outside [0, 1]", layout);
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    s->layout = layout;
    return recapture(s);
}

int cg_get_graph_layout(cg_sim* s, int* layout) {
    if (!s || !layout) return fail(CG_ERR_ARG, "cg_get_graph_layout: NULL argument");
    *layout = s->layout;
    return CG_OK;
}

int cg_synchronize(cg_sim* s) {
    if (!s) return fail(CG_ERR_ARG, "cg_synchronize: NULL handle");
    CG_CHECK(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    CG_SYNC_CHECK(s);
    return CG_OK;
}

}  // extern "C"
