// batch.cu — many DiffusionLenia worlds of uneven size, channel and kernel
// count, advanced together: one persistent launch per phase, the whole step
// captured in one CUDA graph per ping-pong parity.
//
// The reference runs one world per GpuMaceLenia (ml-rs/orchestrator/mod.rs)
// and batches only in its PyTorch model, where every world shares one shape
// (train/lenia_org.py:47, state (B,C,H,W)).  Here each phase's work (row
// blocks, column tiles, diffusion tiles of every world and channel) is a list
// of items; each phase is one persistent launch per grid size present, whose
// resident CTAs stride through that size's items and run the same per-size
// device bodies as the single-world kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "cella_gpu.h"
#include "cella_internal.h"
#include "step_kernels.cuh"

namespace cg {

constexpr int kBatchMinLogN = 6;   // 64^2 .. 2048^2 in one batch
constexpr int kBatchMaxLogN = 11;

constexpr int kVariants = 5;   // per phase at most (phase_variant_count)

struct WorldDesc {
    // tensor maps of U for the inverse row pass's tile copies, one per
    // variant (rows per tile)
    CUtensorMap umap[kVariants];
    int logn, C, K;
    float temp;
    float* state[2];
    float2* rowspec;
    const float2* kspec;
    const float* kre;   // real parts of kspec (read when every world's kernels are real)
    float2* U;
    float* A;
    const float2* tw;
    KernelGroups groups;
    GrowthParams gp;
};

// Rows per inverse-row-pass tile of a size and variant (C2RShape::RB).
template <int LOGN>
int row_tile_rows(int v) {
    if constexpr (LOGN >= kMinPairLogN) {
        if (v == 3) return C2RShape<LOGN, 3>::RB;
        if (v == 4) return C2RShape<LOGN, 4>::RB;
    }
    return v == 1 ? Geo<LOGN, 1>::RB : (v == 2 ? Geo<LOGN, 2>::RB : Geo<LOGN, 0>::RB);
}
int row_tile_rows(int logn, int v) {
    switch (logn) {
        case 6: return row_tile_rows<6>(v);
        case 7: return row_tile_rows<7>(v);
        case 8: return row_tile_rows<8>(v);
        case 9: return row_tile_rows<9>(v);
        case 10: return row_tile_rows<10>(v);
        default: return row_tile_rows<11>(v);
    }
}

struct WorkItem {
    int world, c, a, b;   // a, b: row/column offsets of the unit
};


// One persistent kernel per phase, grid size and CTA-shape variant: a kernel
// that served several sizes made the compiler spill the column pass's
// register-resident spectrum, so each size gets its own instantiation.
// Within one size the items cost about the same (sorted by cost, largest
// first), so each resident CTA takes items blockIdx.x, blockIdx.x + gridDim.x,
// ...  The variants are the single-world kernels' (Geo<LOGN, V>), with the same
// bits.
template <int LOGN, int V>
__global__ void __launch_bounds__(R2CShape<LOGN, V>::RT, R2CShape<LOGN, V>::MINB)
    kb_row_r2c(const WorldDesc* __restrict__ worlds, const WorkItem* __restrict__ items, int count,
               int parity, int* err) {
    extern __shared__ __align__(128) float2 smb_r2c[];
    using Sh = R2CShape<LOGN, V>;
    pdl_wait();
    pdl_launch_dependents();
    if constexpr (Sh::STREAM) {
        constexpr int N = 1 << LOGN;
        __shared__ __align__(8) uint64_t bar;
        init_tile_barrier(&bar);
        uint32_t phase = 0;
        auto item = [&](int i, const float*& src, float2*& dst) {
            const WorkItem it = items[i];
            const WorldDesc& w = worlds[it.world];
            src = w.state[parity] + (size_t(it.c) * N + it.a) * N;
            dst = w.rowspec + size_t(it.c) * (N / 2) * N + it.a;
        };
        // every world of this size class shares the size's twiddle table
        const float2* tw = int(blockIdx.x) < count ? worlds[items[blockIdx.x].world].tw : nullptr;
        row_r2c_stream<LOGN>(item, count, tw, smb_r2c, &bar, phase, err);
    } else {
        for (int i = blockIdx.x; i < count; i += gridDim.x) {
            __syncthreads();
            const WorkItem it = items[i];
            const WorldDesc& w = worlds[it.world];
            row_r2c_variant<LOGN, V>(w.state[parity], w.rowspec, w.tw, it.c, it.a, smb_r2c);
        }
    }
}

template <int LOGN, int V, bool KRE = false>
__global__ void __launch_bounds__(Geo<LOGN, V>::CT, 512 / Geo<LOGN, V>::CT)
    kb_col_conv(const WorldDesc* __restrict__ worlds, const WorkItem* __restrict__ items, int count,
                int* err) {
    extern __shared__ __align__(128) float2 smb_col[];
    __shared__ __align__(8) uint64_t bar;
    pdl_wait();
    pdl_launch_dependents();
    init_tile_barrier(&bar);
    uint32_t phase = 0;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        __syncthreads();
        const WorkItem it = items[i];
        const WorldDesc& w = worlds[it.world];
        if (!col_conv_body<LOGN, V, KRE>(w.rowspec, w.kspec, w.kre, w.U, w.tw, w.groups, it.c,
                                         it.a, smb_col, &bar, phase, err))
            return;   // a bounded wait timed out (uniform across the block)
    }
}

template <int LOGN, int V>
__global__ void __launch_bounds__(C2RShape<LOGN, V>::RT, C2RShape<LOGN, V>::MINB)
    kb_row_c2r_growth(const WorldDesc* __restrict__ worlds, const WorkItem* __restrict__ items,
                      int count, int* err) {
    extern __shared__ __align__(128) float2 smb_c2r[];
    __shared__ __align__(8) uint64_t bar;
    pdl_wait();
    pdl_launch_dependents();
    init_tile_barrier(&bar);
    uint32_t phase = 0;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        __syncthreads();
        const WorkItem it = items[i];
        const WorldDesc& w = worlds[it.world];
        if (!row_c2r_growth_variant<LOGN, V>(&w.umap[V], true, w.A, w.tw, w.groups, w.gp,
                                             w.temp, nullptr, 0.f, it.c, it.a, smb_c2r, &bar,
                                             phase, err))
            return;   // a bounded wait timed out (uniform across the block)
    }
}

template <int LOGN, int V>
__global__ void __launch_bounds__(DiffTile<LOGN, V>::THREADS)
    kb_diffusion(const WorldDesc* __restrict__ worlds, const WorkItem* __restrict__ items,
                 int count, int parity) {
    extern __shared__ __align__(128) float smb_diff[];
    pdl_wait();
    pdl_launch_dependents();
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        __syncthreads();
        const WorkItem it = items[i];
        const WorldDesc& w = worlds[it.world];
        diffusion_tile<LOGN, V>(w.A, w.state[parity], w.state[parity ^ 1], it.c, it.a, it.b,
                                smb_diff, nullptr);
    }
}

// Per size and variant: the four kernels, their block sizes, shared memory
// and the unit each work item covers.
struct PhaseVariant {
    const void* fn;
    const void* fn_real;   // column phase: the real-spectrum form (else nullptr)
    int threads;
    size_t smem;
    int unit_a, unit_b;   // rows per item (row phases), columns per item (column
                          // phase), tile width and height (diffusion)
};
// pv[p][v].fn == nullptr: phase p has no variant v at this size.
template <int LOGN, int V>
void fill_variant(PhaseVariant (&pv)[4][kVariants]) {
    using G = Geo<LOGN, V>;
    using R = R2CShape<LOGN, V>;
    using Q = C2RShape<LOGN, V>;
    pv[0][V] = {reinterpret_cast<const void*>(kb_row_r2c<LOGN, V>), nullptr, R::RT, R::SMEM, R::RB,
                0};
    pv[1][V] = {reinterpret_cast<const void*>(kb_col_conv<LOGN, V>),
                reinterpret_cast<const void*>(kb_col_conv<LOGN, V, true>), G::CT, G::COL_SMEM, G::TW,
                0};
    pv[2][V] = {reinterpret_cast<const void*>(kb_row_c2r_growth<LOGN, V>), nullptr, Q::RT, Q::SMEM,
                Q::RB, 0};
}
template <int LOGN, int V>
void fill_diffusion(PhaseVariant (&pv)[4][kVariants]) {
    using D = DiffTile<LOGN, V>;
    pv[3][V] = {reinterpret_cast<const void*>(kb_diffusion<LOGN, V>), nullptr, D::THREADS, D::SMEM,
                D::TX, D::TY};
}
template <int LOGN>
void fill_size(PhaseVariant (&pv)[4][kVariants]) {
    fill_variant<LOGN, 0>(pv);
    fill_variant<LOGN, 1>(pv);
    fill_variant<LOGN, 2>(pv);
    if constexpr (LOGN >= kMinPairLogN) {
        fill_variant<LOGN, 3>(pv);
        fill_variant<LOGN, 4>(pv);
    }
    fill_diffusion<LOGN, 0>(pv);
    fill_diffusion<LOGN, 1>(pv);
    fill_diffusion<LOGN, 2>(pv);
    fill_diffusion<LOGN, 3>(pv);
}
static void phase_variants_for(int logn, PhaseVariant (&pv)[4][kVariants]) {
    switch (logn) {
        case 6: fill_size<6>(pv); break;
        case 7: fill_size<7>(pv); break;
        case 8: fill_size<8>(pv); break;
        case 9: fill_size<9>(pv); break;
        case 10: fill_size<10>(pv); break;
        default: fill_size<11>(pv); break;
    }
}

}  // namespace cg

using namespace cg;

struct cg_batch {
    struct World {
        int n = 0, logn = 0, C = 0, K = 0;
        float temp = 1.f;
        float* state[2] = {nullptr, nullptr};
        float2* rowspec = nullptr;
        float2* kspec = nullptr;
        float* kspec_re = nullptr;
        std::vector<uint8_t> kreal;   // per kernel: point-symmetric (cg_batch_set_kernel)
        float2* U = nullptr;
        float* A = nullptr;
        KernelGroups groups{};
        GrowthParams gp{};
    };
    // All worlds of one grid side: per phase and CTA-shape variant a work
    // list and a persistent grid; var[] names the variant in use.  mode 0
    // steps the side with one persistent launch per phase over all its
    // worlds; mode 1 runs each world's own step kernels (the single-world
    // kernels, per channel, as in a single world's step graph) with the
    // worlds as parallel branches of the step graph.  The tuner picks the
    // faster; both compute the same bits.
    struct SizeClass {
        int logn = 0;
        int mode = 0;
        PhaseVariant pv[4][kVariants]{};
        WorkItem* d_items[4][kVariants] = {};
        int count[4][kVariants] = {};
        int grid[4][kVariants] = {};
        int var[4] = {0, 0, 0, 0};
    };
    std::vector<World> worlds;
    std::vector<SizeClass> classes;   // largest grid side first
    std::vector<float2*> tw_by_logn = std::vector<float2*>(kMaxLogN + 1, nullptr);
    WorldDesc* d_worlds = nullptr;
    int* err = nullptr;
    void* staging = nullptr;
    double* mass_partial = nullptr;
    double* mass_out = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool kreal_all = false;   // every world's kernels point-symmetric: real column pass
    int cur = 0;
    int device = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    size_t max_px = 0;
};

namespace {

void batch_release(cg_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    for (auto& g : b->graph)
        if (g) cudaGraphExecDestroy(g);
    for (auto& e : b->ev)
        if (e) cudaEventDestroy(e);
    for (auto& w : b->worlds) {
        cudaFree(w.state[0]);
        cudaFree(w.state[1]);
        cudaFree(w.rowspec);
        cudaFree(w.kspec);
        cudaFree(w.kspec_re);
        cudaFree(w.U);
        cudaFree(w.A);
    }
    for (auto p : b->tw_by_logn) cudaFree(p);
    for (auto& sc : b->classes)
        for (auto& per_phase : sc.d_items)
            for (auto p : per_phase) cudaFree(p);
    cudaFree(b->d_worlds);
    cudaFree(b->err);
    cudaFree(b->staging);
    cudaFree(b->mass_partial);
    cudaFree(b->mass_out);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// One phase of one size class in variant v: a persistent launch.
cudaError_t launch_class_phase(cg_batch* b, const cg_batch::SizeClass& sc, int phase, int v,
                               int parity, cudaStream_t st) {
    if (sc.count[phase][v] == 0) return cudaSuccess;
    const PhaseVariant& pv = sc.pv[phase][v];
    const WorldDesc* worlds = b->d_worlds;
    const WorkItem* items = sc.d_items[phase][v];
    int count = sc.count[phase][v];
    void* args[5];
    args[0] = &worlds;
    args[1] = &items;
    args[2] = &count;
    if (phase == 1 || phase == 2) {   // the bulk-copy phases
        args[3] = &b->err;
    } else {
        args[3] = &parity;
        args[4] = &b->err;   // the forward row pass (its streaming variant copies)
    }
    const void* fn = (b->kreal_all && pv.fn_real) ? pv.fn_real : pv.fn;
    // programmatic stream serialization, as the single-world kernels: the
    // next phase's CTAs are dispatched while this one drains
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(sc.grid[phase][v]);
    cfg.blockDim = dim3(pv.threads);
    cfg.dynamicSmemBytes = pv.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

// One phase: a persistent launch per size class (largest first).
cudaError_t launch_phase(cg_batch* b, int phase, int parity, cudaStream_t st) {
    for (const auto& sc : b->classes) {
        cudaError_t e = launch_class_phase(b, sc, phase, sc.var[phase], parity, st);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// Arguments of the single-world step kernels for batched world w (mode 1).
StepArgs world_step_args(const cg_batch* b, int w, int parity, const Variants& var) {
    const auto& W = b->worlds[size_t(w)];
    StepArgs a{};
    a.C = W.C;
    a.K = W.K;
    a.temp = W.temp;
    a.x_in = W.state[parity];
    a.x_out = W.state[parity ^ 1];
    a.rowspec = W.rowspec;
    a.kspec = W.kspec;
    bool real = true;
    for (uint8_t r : W.kreal) real = real && r != 0;
    a.kre = real ? W.kspec_re : nullptr;
    a.U = W.U;
    a.A = W.A;
    a.tw = b->tw_by_logn[W.logn];
    a.udbg = nullptr;
    a.err = b->err;
    a.levels = nullptr;
    a.groups = W.groups;
    a.gp = &b->d_worlds[w].gp;   // the descriptor's copy, in device memory
    a.var = var;
    return a;
}

// Streams and events one class step in mode 1 uses: kLanes lane groups of
// C_max streams (world i of the class runs on lane group i % kLanes, channel
// c on its stream c), a join event per lane stream and, per world and
// channel, the event after its column pass.
constexpr int kLanes = 8;
struct LanePool {
    std::vector<cudaStream_t> streams;   // [kLanes][cmax]
    std::vector<cudaEvent_t> events;
    int cmax = 0;
    LanePool() = default;
    LanePool(const LanePool&) = delete;
    LanePool& operator=(const LanePool&) = delete;
    cudaError_t make(int cmax_, int nevents) {
        cmax = cmax_;
        streams.assign(size_t(kLanes) * cmax, nullptr);
        events.assign(size_t(nevents), nullptr);
        cudaError_t e = cudaSuccess;
        for (auto& st : streams)
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        for (auto& ev : events)
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        return e;
    }
    ~LanePool() {
        for (auto st : streams)
            if (st) cudaStreamDestroy(st);
        for (auto ev : events)
            if (ev) cudaEventDestroy(ev);
    }
};

int class_cmax(const cg_batch* b, const cg_batch::SizeClass& sc) {
    int c = 1;
    for (const auto& W : b->worlds)
        if (W.logn == sc.logn) c = std::max(c, W.C);
    return c;
}
int class_events(const cg_batch* b, const cg_batch::SizeClass& sc) {
    int n = 1 + kLanes * class_cmax(b, sc);
    for (const auto& W : b->worlds)
        if (W.logn == sc.logn) n += W.C;
    return n;
}

// One step of one class on stream st, after what st holds and before what
// it gets next (the lanes fork from st and join back into it).
cudaError_t enqueue_class_step(cg_batch* b, const cg_batch::SizeClass& sc, int parity,
                               cudaStream_t st, LanePool* pool) {
    if (sc.mode == 0) {
        for (int ph = 0; ph < 4; ++ph) {
            cudaError_t e = launch_class_phase(b, sc, ph, sc.var[ph], parity, st);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    Variants var;
    var.r2c = sc.var[0];
    var.col = sc.var[1];
    var.c2r = sc.var[2];
    var.diff = sc.var[3];
    const SizeOps* ops = size_ops(sc.logn);
    size_t ev = 0;
    cudaEvent_t fork = pool->events[ev++];
    cudaError_t e = cudaEventRecord(fork, st);
    for (auto lane : pool->streams)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(lane, fork, 0);
    int i = 0;
    for (int w = 0; w < int(b->worlds.size()) && e == cudaSuccess; ++w) {
        const auto& W = b->worlds[size_t(w)];
        if (W.logn != sc.logn) continue;
        const StepArgs a = world_step_args(b, w, parity, var);
        cudaStream_t* ls = &pool->streams[size_t(i % kLanes) * pool->cmax];
        ++i;
        const size_t ev0 = ev;
        for (int c = 0; c < W.C && e == cudaSuccess; ++c) {
            e = ops->step_channel(a, kPhaseRowFwd | kPhaseColConv, c, ls[c]);
            if (e == cudaSuccess) e = cudaEventRecord(pool->events[ev0 + c], ls[c]);
        }
        ev += size_t(W.C);
        // a channel's inverse row pass reads U of every input channel
        for (int c = 0; c < W.C && e == cudaSuccess; ++c) {
            for (int o = 0; o < W.C && e == cudaSuccess; ++o)
                if (o != c) e = cudaStreamWaitEvent(ls[c], pool->events[ev0 + o], 0);
            if (e == cudaSuccess) e = ops->step_channel(a, kPhaseGrowth | kPhaseDiffusion, c, ls[c]);
        }
    }
    for (auto lane : pool->streams) {
        if (e != cudaSuccess) break;
        cudaEvent_t j = pool->events[ev++];
        e = cudaEventRecord(j, lane);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, j, 0);
    }
    return e;
}

// One graph per ping-pong parity, (re)captured from the current variants.
// The size classes share no data, so each runs its four phases on a forked
// stream of its own: one class's phase tails overlap the other's work.
cudaError_t capture_batch_graphs(cg_batch* b) {
    for (auto& g : b->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    const size_t nc = b->classes.size();
    std::vector<cudaStream_t> st(nc, nullptr);
    std::vector<cudaEvent_t> done(nc, nullptr);
    std::vector<LanePool> pools(nc);
    cudaEvent_t fork = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    for (size_t i = 0; i < nc && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&st[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
        if (e == cudaSuccess && b->classes[i].mode == 1)
            e = pools[i].make(class_cmax(b, b->classes[i]), class_events(b, b->classes[i]));
    }
    for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(st[0], cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t le = cudaEventRecord(fork, st[0]);
            for (size_t i = 1; i < nc && le == cudaSuccess; ++i)
                le = cudaStreamWaitEvent(st[i], fork, 0);
            for (size_t i = 0; i < nc && le == cudaSuccess; ++i)
                le = enqueue_class_step(b, b->classes[i], p, st[i], &pools[i]);
            for (size_t i = 1; i < nc && le == cudaSuccess; ++i) {
                le = cudaEventRecord(done[i], st[i]);
                if (le == cudaSuccess) le = cudaStreamWaitEvent(st[0], done[i], 0);
            }
            if (le == cudaSuccess) le = cudaGetLastError();
            e = cudaStreamEndCapture(st[0], &g);
            if (le != cudaSuccess) e = le;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph[p], g, 0);
        if (g) cudaGraphDestroy(g);
    }
    for (size_t i = 0; i < nc; ++i) {
        if (st[i]) cudaStreamDestroy(st[i]);
        if (done[i]) cudaEventDestroy(done[i]);
    }
    if (fork) cudaEventDestroy(fork);
    return e;
}

// Device ms of one whole batched step (every side, as captured), averaged
// over reps launches of the step graph of the current parity: each launch
// reads the current state and writes the spare buffer, so nothing steps.
int time_batch_step(cg_batch* b, int reps, double* ms) {
    cudaError_t e = cudaGraphLaunch(b->graph[b->cur], b->stream);   // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(b->ev[0], b->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r)
        e = cudaGraphLaunch(b->graph[b->cur], b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev[1], b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->ev[1]);
    float f = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, b->ev[0], b->ev[1]);
    if (e != cudaSuccess) return cuda_fail(e, "timing the batched step");
    *ms = double(f) / reps;
    return CG_OK;
}

// Device ms of one step of class sc alone (its current mode and variants),
// averaged over reps launches of a captured one-step graph.
int time_class_step(cg_batch* b, const cg_batch::SizeClass& sc, int reps, double* ms) {
    cudaStream_t ts = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    LanePool pool;
    cudaError_t e = cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking);
    if (e == cudaSuccess && sc.mode == 1) e = pool.make(class_cmax(b, sc), class_events(b, sc));
    if (e == cudaSuccess) e = cudaStreamBeginCapture(ts, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t le = enqueue_class_step(b, sc, b->cur, ts, &pool);
        e = cudaStreamEndCapture(ts, &g);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(ge, ts);   // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(b->ev[0], ts);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = cudaGraphLaunch(ge, ts);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev[1], ts);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->ev[1]);
    float f = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, b->ev[0], b->ev[1]);
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    if (ts) cudaStreamDestroy(ts);
    if (e != cudaSuccess) return cuda_fail(e, "timing a batched step");
    *ms = double(f) / reps;
    return CG_OK;
}

int batch_sync_check(cg_batch* b) {
    int h = 0;
    cudaError_t e = cudaMemcpy(&h, b->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "reading error word");
    if (h != 0) {
        cudaMemset(b->err, 0, sizeof(int));
        return fail(CG_ERR_TIMEOUT, "a device-side wait for an asynchronous copy timed out");
    }
    return CG_OK;
}

}  // namespace

#define BCHECK(call, what)                                   \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);   \
    } while (0)

extern "C" {

int cg_batch_create(int n_worlds, const int* n, const int* C, const int* K, const uint32_t* c0,
                    const uint32_t* c1, const float* mu, const float* sigma, const float* weights,
                    const float* temp, cg_stream_t stream, cg_batch** out) {
    if (!out) return fail(CG_ERR_ARG, "cg_batch_create: out is NULL");
    *out = nullptr;
    if (n_worlds < 1 || n_worlds > 4096)
        return fail(CG_ERR_ARG, "world count %d outside [1, 4096]", n_worlds);
    if (!n || !C || !K || !c0 || !c1 || !mu || !sigma || !weights || !temp)
        return fail(CG_ERR_ARG, "cg_batch_create: NULL array");
    cg_batch* b = new (std::nothrow) cg_batch;
    if (!b) return fail(CG_ERR_OOM, "cg_batch_create: host allocation failed");
    b->worlds.resize(n_worlds);
    size_t koff = 0;
    for (int w = 0; w < n_worlds; ++w) {
        int logn = 0;
        int rc = validate_world(n[w], C[w], K[w], c0 + koff, c1 + koff, mu + koff, sigma + koff,
                                weights + koff, temp[w], &logn);
        if (rc == CG_OK && logn < kBatchMinLogN) {
            rc = fail(CG_ERR_UNSUPPORTED, "batched worlds need a grid side of at least %d",
                      1 << kBatchMinLogN);
        }
        if (rc != CG_OK) {
            char buf[600];
            snprintf(buf, sizeof buf, "world %d: %s", w, cg_last_error());
            delete b;
            return fail(rc, "%s", buf);
        }
        auto& W = b->worlds[w];
        W.n = n[w];
        W.logn = logn;
        W.C = C[w];
        W.K = K[w];
        W.temp = temp[w];
        build_groups(W.C, W.K, c0 + koff, c1 + koff, mu + koff, sigma + koff, weights + koff,
                     &W.groups, &W.gp);
        koff += size_t(K[w]);
        b->max_px = std::max(b->max_px, size_t(W.n) * W.n);
    }

    int rc = CG_OK;
    auto chk = [&](cudaError_t e, const char* what) {
        if (rc == CG_OK && e != cudaSuccess) rc = cuda_fail(e, what);
        return rc == CG_OK;
    };
    chk(cudaGetDevice(&b->device), "cudaGetDevice");
    if (rc == CG_OK) {
        if (stream) {
            b->stream = static_cast<cudaStream_t>(stream);
        } else if (chk(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking),
                       "cudaStreamCreate")) {
            b->own_stream = true;
        }
    }
    // per-world buffers and per-size twiddles
    for (auto& W : b->worlds) {
        if (rc != CG_OK) break;
        const size_t px = size_t(W.n) * W.n, half = size_t(W.n / 2) * W.n;
        chk(cudaMalloc(&W.state[0], sizeof(float) * W.C * px), "cudaMalloc(state)");
        chk(cudaMalloc(&W.state[1], sizeof(float) * W.C * px), "cudaMalloc(state)");
        chk(cudaMalloc(&W.rowspec, sizeof(float2) * W.C * half), "cudaMalloc(rowspec)");
        chk(cudaMalloc(&W.kspec, sizeof(float2) * W.K * (half + W.n)), "cudaMalloc(kspec)");
        chk(cudaMalloc(&W.kspec_re, sizeof(float) * W.K * (half + W.n)), "cudaMalloc(kspec_re)");
        W.kreal.assign(size_t(W.K), 0);
        chk(cudaMalloc(&W.U, sizeof(float2) * W.K * half), "cudaMalloc(U)");
        chk(cudaMalloc(&W.A, sizeof(float) * W.C * px), "cudaMalloc(A)");
        if (rc == CG_OK) {
            chk(cudaMemsetAsync(W.state[0], 0, sizeof(float) * W.C * px, b->stream), "memset");
            chk(cudaMemsetAsync(W.state[1], 0, sizeof(float) * W.C * px, b->stream), "memset");
            chk(cudaMemsetAsync(W.kspec, 0, sizeof(float2) * W.K * (half + W.n), b->stream),
                "memset");
        }
        if (rc == CG_OK && !b->tw_by_logn[W.logn]) {
            const SizeOps* ops = size_ops(W.logn);
            std::vector<float2> h(size_t(ops->twiddle_count()));
            build_twiddle_tables(W.n, h.data());
            if (chk(cudaMalloc(&b->tw_by_logn[W.logn], sizeof(float2) * h.size()),
                    "cudaMalloc(twiddles)"))
                chk(cudaMemcpy(b->tw_by_logn[W.logn], h.data(), sizeof(float2) * h.size(),
                               cudaMemcpyHostToDevice),
                    "uploading twiddles");
            chk(ops->prepare(), "configuring kernels");
        }
    }
    // descriptors
    std::vector<WorldDesc> descs(n_worlds);
    for (int w = 0; w < n_worlds && rc == CG_OK; ++w) {
        const auto& W = b->worlds[w];
        WorldDesc& d = descs[w];
        d.logn = W.logn;
        d.C = W.C;
        d.K = W.K;
        d.temp = W.temp;
        d.state[0] = W.state[0];
        d.state[1] = W.state[1];
        d.rowspec = W.rowspec;
        d.kspec = W.kspec;
        d.kre = W.kspec_re;
        d.U = W.U;
        d.A = W.A;
        d.tw = b->tw_by_logn[W.logn];
        d.groups = W.groups;
        d.gp = W.gp;
        for (int m = 0; m < phase_variant_count(W.logn, 2) && rc == CG_OK; ++m)
            chk(encode_u_map(&d.umap[m], W.U, W.n, W.K, row_tile_rows(W.logn, m)),
                "encoding a tensor map of U");
    }
    if (rc == CG_OK && chk(cudaMalloc(&b->d_worlds, sizeof(WorldDesc) * n_worlds), "cudaMalloc"))
        chk(cudaMemcpy(b->d_worlds, descs.data(), sizeof(WorldDesc) * n_worlds,
                       cudaMemcpyHostToDevice),
            "uploading world descriptors");
    // size classes, largest first; per class and phase a work list
    int sms = 0;
    if (rc == CG_OK)
        chk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device), "attr");
    for (int logn = kBatchMaxLogN; logn >= kBatchMinLogN && rc == CG_OK; --logn) {
        bool present = false;
        for (const auto& W : b->worlds) present = present || W.logn == logn;
        if (!present) continue;
        cg_batch::SizeClass sc;
        sc.logn = logn;
        phase_variants_for(logn, sc.pv);
        for (int p = 0; p < 4 && rc == CG_OK; ++p)
            for (int v = 0; v < phase_variant_count(logn, p) && rc == CG_OK; ++v) {
                const PhaseVariant& pv = sc.pv[p][v];
                std::vector<WorkItem> list;
                for (int w = 0; w < n_worlds; ++w) {
                    const auto& W = b->worlds[w];
                    if (W.logn != logn) continue;
                    for (int c = 0; c < W.C; ++c) {
                        if (p == 0 || p == 2) {
                            for (int y0 = 0; y0 < W.n; y0 += pv.unit_a) list.push_back({w, c, y0, 0});
                        } else if (p == 1) {
                            if (W.groups.in_count[c] > 0)
                                for (int x0 = 0; x0 < W.n / 2; x0 += pv.unit_a)
                                    list.push_back({w, c, x0, 0});
                        } else {
                            for (int y0 = 0; y0 < W.n; y0 += pv.unit_b)
                                for (int x0 = 0; x0 < W.n; x0 += pv.unit_a)
                                    list.push_back({w, c, x0, y0});
                        }
                    }
                }
                sc.count[p][v] = int(list.size());
                if (chk(cudaMalloc(&sc.d_items[p][v],
                                   sizeof(WorkItem) * std::max<size_t>(1, list.size())),
                        "cudaMalloc(items)"))
                    chk(cudaMemcpy(sc.d_items[p][v], list.data(), sizeof(WorkItem) * list.size(),
                                   cudaMemcpyHostToDevice),
                        "uploading work lists");
                chk(cudaFuncSetAttribute(pv.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(pv.smem)),
                    "cudaFuncSetAttribute");
                if (pv.fn_real)
                    chk(cudaFuncSetAttribute(pv.fn_real,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(pv.smem)),
                        "cudaFuncSetAttribute");
                int per_sm = 0;
                chk(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pv.fn, pv.threads,
                                                                  pv.smem),
                    "occupancy");
                sc.grid[p][v] = std::max(1, std::min(per_sm * sms, std::max(1, sc.count[p][v])));
            }
        b->classes.push_back(sc);
    }
    if (rc == CG_OK) chk(cudaMalloc(&b->err, sizeof(int)), "cudaMalloc(err)");
    if (rc == CG_OK) chk(cudaMemset(b->err, 0, sizeof(int)), "memset(err)");
    if (rc == CG_OK) chk(cudaMalloc(&b->staging, sizeof(double) * b->max_px), "cudaMalloc(staging)");
    if (rc == CG_OK)
        chk(cudaMalloc(&b->mass_partial, sizeof(double) * kMaxC * kMassBlocks), "cudaMalloc(mass)");
    if (rc == CG_OK) chk(cudaMalloc(&b->mass_out, sizeof(double) * kMaxC), "cudaMalloc(mass)");
    for (int i = 0; i < 5 && rc == CG_OK; ++i) chk(cudaEventCreate(&b->ev[i]), "cudaEventCreate");
    if (rc == CG_OK) chk(capture_batch_graphs(b), "capturing the batched step graph");
    if (rc == CG_OK) chk(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    if (rc != CG_OK) {
        batch_release(b);
        return rc;
    }
    *out = b;
    return CG_OK;
}

int cg_batch_destroy(cg_batch* b) {
    if (!b) return fail(CG_ERR_ARG, "cg_batch_destroy: NULL handle");
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    batch_release(b);
    return CG_OK;
}

static int world_check(cg_batch* b, int w) {
    if (!b) return fail(CG_ERR_ARG, "NULL batch handle");
    if (w < 0 || w >= int(b->worlds.size()))
        return fail(CG_ERR_ARG, "world index %d outside [0, %zu)", w, b->worlds.size());
    return CG_OK;
}

int cg_batch_set_kernel(cg_batch* b, int world, int k, const float* spec) {
    int rc = world_check(b, world);
    if (rc != CG_OK) return rc;
    auto& W = b->worlds[world];
    if (!spec) return fail(CG_ERR_ARG, "cg_batch_set_kernel: NULL spectrum");
    if (k < 0 || k >= W.K) return fail(CG_ERR_ARG, "kernel index %d outside [0, %d)", k, W.K);
    const size_t px = size_t(W.n) * W.n, half = size_t(W.n / 2) * W.n;
    BCHECK(cudaMemcpyAsync(b->staging, spec, sizeof(float2) * px, cudaMemcpyHostToDevice,
                           b->stream),
           "uploading kernel spectrum");
    float2* packed = W.kspec + size_t(k) * (half + W.n);
    BCHECK(size_ops(W.logn)->pack(static_cast<const float2*>(b->staging), packed, b->stream),
           "packing kernel spectrum");
    // point-symmetric kernels: keep the real parts (see cg_set_kernel)
    const bool real = hermitian_part_is_real(spec, W.n);
    if (real)
        BCHECK(launch_real_parts(packed, W.kspec_re + size_t(k) * (half + W.n), half + W.n,
                                 b->stream),
               "keeping the real parts");
    W.kreal[size_t(k)] = real ? 1 : 0;
    bool all = true;
    for (const auto& w : b->worlds)
        for (uint8_t r : w.kreal) all = all && r != 0;
    if (all != b->kreal_all) {
        BCHECK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        b->kreal_all = all;
        BCHECK(capture_batch_graphs(b), "re-capturing the batched step graph");
    }
    return CG_OK;
}

int cg_batch_upload_channel(cg_batch* b, int world, int c, const double* data) {
    int rc = world_check(b, world);
    if (rc != CG_OK) return rc;
    auto& W = b->worlds[world];
    if (!data) return fail(CG_ERR_ARG, "cg_batch_upload_channel: NULL data");
    if (c < 0 || c >= W.C) return fail(CG_ERR_ARG, "channel index %d outside [0, %d)", c, W.C);
    const size_t px = size_t(W.n) * W.n;
    BCHECK(cudaMemcpyAsync(b->staging, data, sizeof(double) * px, cudaMemcpyHostToDevice,
                           b->stream),
           "uploading channel");
    BCHECK(launch_f64_to_f32(static_cast<const double*>(b->staging),
                             W.state[b->cur] + size_t(c) * px, px, b->stream),
           "converting channel");
    return CG_OK;
}

int cg_batch_step(cg_batch* b, int nsteps) {
    if (!b) return fail(CG_ERR_ARG, "cg_batch_step: NULL handle");
    if (nsteps < 0) return fail(CG_ERR_ARG, "negative step count %d", nsteps);
    for (int i = 0; i < nsteps; ++i) {
        BCHECK(cudaGraphLaunch(b->graph[b->cur], b->stream), "cudaGraphLaunch");
        b->cur ^= 1;
    }
    return CG_OK;
}

int cg_batch_download_channels(cg_batch* b, int world, float* out) {
    int rc = world_check(b, world);
    if (rc != CG_OK) return rc;
    if (!out) return fail(CG_ERR_ARG, "cg_batch_download_channels: NULL output");
    auto& W = b->worlds[world];
    BCHECK(cudaMemcpyAsync(out, W.state[b->cur], sizeof(float) * W.C * size_t(W.n) * W.n,
                           cudaMemcpyDeviceToHost, b->stream),
           "downloading channels");
    BCHECK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    return batch_sync_check(b);
}

int cg_batch_mass_f64(cg_batch* b, int world, double* out) {
    int rc = world_check(b, world);
    if (rc != CG_OK) return rc;
    if (!out) return fail(CG_ERR_ARG, "cg_batch_mass_f64: NULL output");
    auto& W = b->worlds[world];
    BCHECK(launch_mass_f64(W.state[b->cur], W.C, size_t(W.n) * W.n, b->mass_partial, kMassBlocks,
                           b->mass_out, b->stream),
           "mass reduction");
    BCHECK(cudaMemcpyAsync(out, b->mass_out, sizeof(double) * W.C, cudaMemcpyDeviceToHost,
                           b->stream),
           "downloading masses");
    BCHECK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    return batch_sync_check(b);
}

int cg_batch_synchronize(cg_batch* b) {
    if (!b) return fail(CG_ERR_ARG, "cg_batch_synchronize: NULL handle");
    BCHECK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    return batch_sync_check(b);
}

int cg_batch_profile(cg_batch* b, int nsteps, double ms[4]) {
    if (!b || !ms) return fail(CG_ERR_ARG, "cg_batch_profile: NULL argument");
    if (nsteps < 1 || nsteps > 1024) return fail(CG_ERR_ARG, "nsteps %d outside [1, 1024]", nsteps);
    double acc[4] = {0, 0, 0, 0};
    for (int i = 0; i < nsteps; ++i) {
        BCHECK(cudaEventRecord(b->ev[0], b->stream), "cudaEventRecord");
        for (int p = 0; p < 4; ++p) {
            BCHECK(launch_phase(b, p, b->cur, b->stream), "launching a phase");
            BCHECK(cudaEventRecord(b->ev[p + 1], b->stream), "cudaEventRecord");
        }
        BCHECK(cudaEventSynchronize(b->ev[4]), "cudaEventSynchronize");
        for (int p = 0; p < 4; ++p) {
            float t = 0.f;
            BCHECK(cudaEventElapsedTime(&t, b->ev[p], b->ev[p + 1]), "cudaEventElapsedTime");
            acc[p] += t;
        }
        b->cur ^= 1;
    }
    for (int p = 0; p < 4; ++p) ms[p] = acc[p] / nsteps;
    return batch_sync_check(b);
}

int cg_batch_stream(cg_batch* b, cg_stream_t* out) {
    if (!b || !out) return fail(CG_ERR_ARG, "cg_batch_stream: NULL argument");
    *out = b->stream;
    return CG_OK;
}

int cg_batch_info(cg_batch* b, int* items4, int* grid4) {
    if (!b) return fail(CG_ERR_ARG, "cg_batch_info: NULL handle");
    for (int p = 0; p < 4; ++p) {
        int items = 0, grid = 0;
        for (auto& sc : b->classes) {
            items += sc.count[p][sc.var[p]];
            grid = std::max(grid, sc.grid[p][sc.var[p]]);
        }
        if (items4) items4[p] = items;
        if (grid4) grid4[p] = grid;
    }
    return CG_OK;
}

int cg_batch_set_variants(cg_batch* b, int n, const int v[4]) {
    if (!b || !v) return fail(CG_ERR_ARG, "cg_batch_set_variants: NULL argument");
    for (auto& sc : b->classes) {
        if ((1 << sc.logn) != n) continue;
        for (int p = 0; p < 4; ++p)
            if (v[p] < 0 || v[p] >= phase_variant_count(sc.logn, p))
                return fail(CG_ERR_ARG, "variant %d of phase %d outside [0, %d] at grid side %d",
                            v[p], p, phase_variant_count(sc.logn, p) - 1, n);
        BCHECK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        for (int p = 0; p < 4; ++p) sc.var[p] = v[p];
        BCHECK(capture_batch_graphs(b), "re-capturing the batched step graph");
        return CG_OK;
    }
    return fail(CG_ERR_ARG, "the batch has no world of grid side %d", n);
}

int cg_batch_set_mode(cg_batch* b, int n, int mode) {
    if (!b) return fail(CG_ERR_ARG, "cg_batch_set_mode: NULL handle");
    if (mode < 0 || mode > 1) return fail(CG_ERR_ARG, "batch mode %d outside [0, 1]", mode);
    for (auto& sc : b->classes) {
        if ((1 << sc.logn) != n) continue;
        BCHECK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        sc.mode = mode;
        BCHECK(capture_batch_graphs(b), "re-capturing the batched step graph");
        return CG_OK;
    }
    return fail(CG_ERR_ARG, "the batch has no world of grid side %d", n);
}

int cg_batch_get_mode(cg_batch* b, int n, int* mode) {
    if (!b || !mode) return fail(CG_ERR_ARG, "cg_batch_get_mode: NULL argument");
    for (const auto& sc : b->classes)
        if ((1 << sc.logn) == n) {
            *mode = sc.mode;
            return CG_OK;
        }
    return fail(CG_ERR_ARG, "the batch has no world of grid side %d", n);
}

int cg_batch_autotune(cg_batch* b, int reps, int* chosen, double* ms_out) {
    if (!b) return fail(CG_ERR_ARG, "cg_batch_autotune: NULL handle");
    if (reps < 1 || reps > 1000)
        return fail(CG_ERR_ARG, "cg_batch_autotune: reps %d outside [1, 1000]", reps);
    BCHECK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    constexpr int kSizes = kBatchMaxLogN - kBatchMinLogN + 1;
    if (chosen)
        for (int i = 0; i < kSizes * 4; ++i) chosen[i] = -1;
    if (ms_out)
        for (int i = 0; i < kSizes * 4 * kVariants; ++i) ms_out[i] = -1.0;
    // Each phase of a size class reads the state or the scratch the previous
    // phases wrote; run in order on the live batch, the state is untouched
    // (diffusion writes the spare ping-pong buffer only).
    for (auto& sc : b->classes) {
        const int slot = sc.logn - kBatchMinLogN;
        for (int p = 0; p < 4; ++p) {
            double t[kVariants];
            int best = 0;
            for (int v = 0; v < phase_variant_count(sc.logn, p); ++v) {
                for (int q = 0; q < p; ++q)
                    BCHECK(launch_class_phase(b, sc, q, sc.var[q], b->cur, b->stream),
                           "autotune prologue");
                BCHECK(launch_class_phase(b, sc, p, v, b->cur, b->stream), "autotune warm-up");
                BCHECK(cudaEventRecord(b->ev[0], b->stream), "cudaEventRecord");
                for (int r = 0; r < reps; ++r)
                    BCHECK(launch_class_phase(b, sc, p, v, b->cur, b->stream), "autotune launch");
                BCHECK(cudaEventRecord(b->ev[1], b->stream), "cudaEventRecord");
                BCHECK(cudaEventSynchronize(b->ev[1]), "cudaEventSynchronize");
                float f = 0.f;
                BCHECK(cudaEventElapsedTime(&f, b->ev[0], b->ev[1]), "cudaEventElapsedTime");
                t[v] = double(f) / reps;
                if (t[v] < t[best]) best = v;
                if (ms_out) ms_out[(slot * 4 + p) * kVariants + v] = t[v];
            }
            sc.var[p] = best;
            if (chosen) chosen[slot * 4 + p] = best;
        }
        // then the two ways of stepping the side (mode 0 and 1), each as a
        // captured one-step graph of this side alone, in the parity of the
        // current state (diffusion writes the spare buffer: nothing steps)
        double best_t = 0.0;
        int best_mode = 0;
        for (int m = 0; m < 2; ++m) {
            sc.mode = m;
            double t = 0.0;
            const int rc = time_class_step(b, sc, reps, &t);
            if (rc != CG_OK) return rc;
            if (m == 0 || t < best_t) {
                best_t = t;
                best_mode = m;
            }
        }
        sc.mode = best_mode;
    }
    // The sides run concurrently in the step graph, so a mode that wins for
    // a side alone can lose in the whole step (two sides' world branches
    // competing for the SMs).  With at most three sides, every combination
    // of modes is timed on the whole step and the fastest kept.
    const int nsides = int(b->classes.size());
    if (nsides >= 2 && nsides <= 3) {
        int best_mask = 0;
        for (int i = 0; i < nsides; ++i) best_mask |= b->classes[size_t(i)].mode << i;
        double best_t = -1.0;
        for (int mask = 0; mask < (1 << nsides); ++mask) {
            for (int i = 0; i < nsides; ++i) b->classes[size_t(i)].mode = (mask >> i) & 1;
            BCHECK(capture_batch_graphs(b), "capturing a batched step graph to time");
            double t = 0.0;
            const int rc = time_batch_step(b, reps, &t);
            if (rc != CG_OK) return rc;
            if (best_t < 0.0 || t < best_t) {
                best_t = t;
                best_mask = mask;
            }
        }
        for (int i = 0; i < nsides; ++i) b->classes[size_t(i)].mode = (best_mask >> i) & 1;
    }
    int rc = batch_sync_check(b);
    if (rc != CG_OK) return rc;
    BCHECK(capture_batch_graphs(b), "re-capturing the batched step graph");
    return CG_OK;
}

}  // extern "C"
