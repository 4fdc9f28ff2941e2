// ss_batch.cu — many grids per launch sequence: batches under a CUDA graph
// (with an autotuner for the ring-kernel CTA size), RL multi-patch chains
// (PatchChain / multiGridTransform!, src/multipatch.jl), and radial tiles
// with halo sums (sumSpectralTile!, src/tiling.jl:1048-1136).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ss_df64.cuh"
#include "ss_grid.h"
#include "ss_kernels.h"

using namespace ss;

#define CUDA_TRY(expr)                                                                      \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) {                                                            \
            set_error("%s failed: %s", #expr, cudaGetErrorString(_e));                      \
            return (_e == cudaErrorMemoryAllocation) ? SS_OUT_OF_MEMORY : SS_CUDA_ERROR;   \
        }                                                                                   \
    } while (0)

// ====================================================================== batch
// One launch of a fused batch: the CTAs of many grids' records of one stage
// (one shared-memory class), each CTA running the record its work entry names.
enum { FK_RING_FWD = 0, FK_SB = 1, FK_SA = 2, FK_SA_F32 = 3, FK_RING_INV = 4 };
struct FusedLaunch {
    int kind, tl;
    size_t smem;
    int threads, nwork;
    const void *recs;       // RingLaunch / SbLaunch / SaLaunch records (device)
    const BatchWork *work;  // one entry per CTA (device)
};

struct ss_batch {
    std::vector<ss_grid *> grids;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> side;  // fork-join branches of the captured graph
    std::vector<cudaEvent_t> ev;
    cudaGraph_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaGraphExec_t exec[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<uint64_t> gen[4];  // each grid's generation when graph[what] was captured
    // fused mode: every RL grid's stages as a few launches over work lists
    bool fused = false;
    int ib_scale = 1;                   // items per ring CTA × this (autotuned)
    std::vector<FusedLaunch> fwd, inv;  // in launch order
    std::vector<ss_grid *> unfused;     // RLZ grids: their own launch sequences
    std::vector<void *> fused_mem;
    std::vector<uint64_t> fused_gen;    // generations the records were built from
};

// The grids' generation counters; a graph whose grids have changed since (ahat registered or cleared, filter set) is captured again,
// because its launches hold the old pointers and flags.
static std::vector<uint64_t> generations(const ss_batch *bt) {
    std::vector<uint64_t> out;
    for (const ss_grid *g : bt->grids) out.push_back(g->generation);
    return out;
}

static int32_t run_direction(ss_grid *g, int what, cudaStream_t st) {
    int32_t r = SS_OK;
    if (what & 1) r = grid_forward(g, st);
    if (r == SS_OK && (what & 2)) r = grid_inverse(g, st);
    return r;
}

// Autotuner: time each candidate CTA size of the ring kernels on the grid's
// own data and keep the fastest per direction.
static int32_t autotune_grid(ss_grid *g, cudaStream_t st) {
    const int cand[3] = {64, 128, 256};
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    for (int dir = 1; dir <= 2; dir++) {
        float best = 1e30f;
        int best_t = 256;
        for (int c = 0; c < 3; c++) {
            if (dir == 1) g->ring_threads_fwd = cand[c];
            else g->ring_threads_inv = cand[c];
            int32_t r = run_direction(g, dir, st);  // warm-up
            if (r) { cudaEventDestroy(a); cudaEventDestroy(b); return r; }
            CUDA_TRY(cudaEventRecord(a, st));
            for (int rep = 0; rep < 2; rep++) {
                r = run_direction(g, dir, st);
                if (r) { cudaEventDestroy(a); cudaEventDestroy(b); return r; }
            }
            CUDA_TRY(cudaEventRecord(b, st));
            CUDA_TRY(cudaEventSynchronize(b));
            float ms = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
            if (ms < best) { best = ms; best_t = cand[c]; }
        }
        if (dir == 1) g->ring_threads_fwd = best_t;
        else g->ring_threads_inv = best_t;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return SS_OK;
}

// ---- fused plan
// shared-memory classes of the fused ring and SA launches: a CTA's dynamic
// shared memory is its class's largest, so records of similar size share a launch.
// The top class leaves 1 KB of the 227 KB per-block limit to the kernels' static
// shared memory (the staged launch record, per-item offsets).
static const size_t kSmemClass[] = {12 << 10, 24 << 10, 48 << 10, 72 << 10, 100 << 10, 140 << 10, 226 << 10};
static int smem_class(size_t b) {
    for (int c = 0; c < (int)(sizeof kSmemClass / sizeof kSmemClass[0]); c++)
        if (b <= kSmemClass[c]) return c;
    return -1;
}

static void free_fused(ss_batch *bt) {
    for (void *p : bt->fused_mem) cudaFree(p);
    bt->fused_mem.clear();
    bt->fwd.clear();
    bt->inv.clear();
    bt->unfused.clear();
}

template <typename R>
static int32_t upload(ss_batch *bt, const std::vector<R> &v, const void **out) {
    void *p = nullptr;
    CUDA_TRY(cudaMalloc(&p, std::max<size_t>(v.size(), 1) * sizeof(R)));
    bt->fused_mem.push_back(p);
    CUDA_TRY(cudaMemcpy(p, v.data(), v.size() * sizeof(R), cudaMemcpyHostToDevice));
    *out = p;
    return SS_OK;
}

// ring stage of every grid of one compute layout: one record per (grid, bucket),
// CTAs grouped by (shared-memory class, CTA size), largest rings first
static int32_t plan_rings(ss_batch *bt, const std::vector<ss_grid *> &gs, int tl, bool inverse,
                          std::vector<FusedLaunch> &out) {
    struct Rec { RingLaunch L; size_t smem; int threads, nrings, nb, buf; };
    std::vector<Rec> recs;
    for (ss_grid *g : gs)
        for (const RingBucket &bkt : g->buckets) {
            Rec r;
            r.L = ring_record(g, inverse);
            r.L.ring_list = g->d_ring_list + bkt.offset;
            r.threads = inverse ? g->ring_threads_inv : g->ring_threads_fwd;
            const size_t per = ring_item_smem(g, bkt, inverse);
            int ib = ring_batch(per, g->nitems, bkt.count, 1, r.threads, bkt.max_buf, true) * bt->ib_scale;
            ib = std::max(1, std::min({ib, kRingBatchMax, g->nitems}));
            while (ib > 1 && per * ib > kSmemClass[6]) ib--;
            r.L.ib = ib;
            r.smem = per * ib;
            r.nrings = bkt.count;
            r.nb = (g->nitems + ib - 1) / ib;
            r.buf = bkt.max_buf;
            if (smem_class(r.smem) < 0) {
                set_error("a ring of the batch needs %zu bytes of shared memory", r.smem);
                return SS_BAD_SHAPE;
            }
            recs.push_back(r);
        }
    std::vector<RingLaunch> L;
    for (const Rec &r : recs) L.push_back(r.L);
    const void *d_recs = nullptr;
    int32_t rc = upload(bt, L, &d_recs);
    if (rc) return rc;
    std::vector<int> order(recs.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return recs[a].buf > recs[b].buf; });
    for (int c = 0; c < 7; c++)
        for (int threads : {64, 128, 256}) {
            std::vector<BatchWork> work;
            size_t smem = 0;
            for (int i : order) {
                const Rec &r = recs[i];
                if (smem_class(r.smem) != c || r.threads != threads) continue;
                smem = std::max(smem, r.smem);
                for (int ring = 0; ring < r.nrings; ring++)
                    for (int bx = 0; bx < r.nb; bx++) work.push_back({i, bx, ring, 0});
            }
            if (work.empty()) continue;
            FusedLaunch f{inverse ? FK_RING_INV : FK_RING_FWD, tl, smem, threads, (int)work.size(), d_recs, nullptr};
            const void *w = nullptr;
            if ((rc = upload(bt, work, &w))) return rc;
            f.work = (const BatchWork *)w;
            out.push_back(f);
        }
    return SS_OK;
}

static int32_t plan_sb(ss_batch *bt, const std::vector<ss_grid *> &gs, int tl, std::vector<FusedLaunch> &out) {
    std::vector<SbLaunch> L;
    std::vector<BatchWork> work;
    for (ss_grid *g : gs) {
        const int i = (int)L.size();
        L.push_back(sb_record(g));
        const SbLaunch &S = L.back();
        for (int bz = 0; bz < g->nitems; bz++)
            for (int by = 0; by < (S.b + kSbOut - 1) / kSbOut; by++)
                for (int bx = 0; bx < (S.nslots_z + 31) / 32; bx++) work.push_back({i, bx, by, bz});
    }
    const void *d_recs = nullptr, *w = nullptr;
    int32_t rc = upload(bt, L, &d_recs);
    if (!rc) rc = upload(bt, work, &w);
    if (rc) return rc;
    out.push_back({FK_SB, tl, 0, 256, (int)work.size(), d_recs, (const BatchWork *)w});
    return SS_OK;
}

static int32_t plan_sa(ss_batch *bt, const std::vector<ss_grid *> &gs, int tl, std::vector<FusedLaunch> &out) {
    std::vector<SaLaunch> L;
    std::vector<size_t> smem;
    for (ss_grid *g : gs) {
        size_t sm = 0;
        L.push_back(sa_record(g, 0, &sm));
        smem.push_back(sm);
    }
    const void *d_recs = nullptr;
    int32_t rc = upload(bt, L, &d_recs);
    if (rc) return rc;
    // binary32 grids: the slot-parallel solve (no dynamic shared memory), except
    // grids with a periodic spline, whose dense-tail solve runs on the tiled kernel
    auto periodic = [&](int i) {
        for (auto &sh : gs[i]->spl_host)
            if (sh.periodic) return true;
        return false;
    };
    if (tl == TL_F32) {
        std::vector<BatchWork> work;
        for (int i = 0; i < (int)gs.size(); i++)
            if (!periodic(i))
                for (int by = 0; by < gs[i]->nitems; by++)
                    for (int bx = 0; bx < (L[i].nslots_z + 127) / 128; bx++) work.push_back({i, bx, by, 0});
        if (!work.empty()) {
            const void *w = nullptr;
            if ((rc = upload(bt, work, &w))) return rc;
            out.push_back({FK_SA_F32, tl, 0, 128, (int)work.size(), d_recs, (const BatchWork *)w});
        }
    }
    for (int c = 0; c < 7; c++) {
        std::vector<BatchWork> work;
        size_t sm = 0;
        for (int i = 0; i < (int)gs.size(); i++) {
            if (tl == TL_F32 && !periodic(i)) continue;
            if (smem_class(smem[i]) != c) continue;
            sm = std::max(sm, smem[i]);
            for (int by = 0; by < gs[i]->nitems; by++)
                for (int bx = 0; bx < (L[i].nslots_z + 31) / 32; bx++) work.push_back({i, bx, by, 0});
        }
        if (work.empty()) continue;
        const void *w = nullptr;
        if ((rc = upload(bt, work, &w))) return rc;
        out.push_back({FK_SA, tl, sm, 128, (int)work.size(), d_recs, (const BatchWork *)w});
    }
    for (size_t i = 0; i < smem.size(); i++)
        if (smem_class(smem[i]) < 0) {
            set_error("a spline solve of the batch needs %zu bytes of shared memory", smem[i]);
            return SS_BAD_SHAPE;
        }
    return SS_OK;
}

static std::vector<uint64_t> generations(const ss_batch *bt);
static int32_t build_fused(ss_batch *bt) {
    free_fused(bt);
    for (int tl : {TL_F64, TL_DF64, TL_F32}) {
        std::vector<ss_grid *> gs;
        for (ss_grid *g : bt->grids)
            if (!g->rlz && g->tl == tl) gs.push_back(g);
        if (gs.empty()) continue;
        int32_t rc = plan_rings(bt, gs, tl, false, bt->fwd);
        if (!rc) rc = plan_sb(bt, gs, tl, bt->fwd);
        if (!rc) rc = plan_sa(bt, gs, tl, bt->inv);
        if (!rc) rc = plan_rings(bt, gs, tl, true, bt->inv);
        if (rc) { free_fused(bt); return rc; }
    }
    for (ss_grid *g : bt->grids)
        if (g->rlz) bt->unfused.push_back(g);
    bt->fused_gen = generations(bt);
    return SS_OK;
}

template <typename P, typename T>
static cudaError_t fused_launch(const FusedLaunch &f, cudaStream_t st) {
    switch (f.kind) {
    case FK_RING_FWD:
        return launch_ring_forward_fused<P, T>((const RingLaunch *)f.recs, f.work, f.nwork, f.smem, f.threads, st);
    case FK_RING_INV:
        return launch_ring_inverse_fused<P, T>((const RingLaunch *)f.recs, f.work, f.nwork, f.smem, f.threads, st);
    case FK_SB: return launch_sb_project_fused<P, T>((const SbLaunch *)f.recs, f.work, f.nwork, st);
    case FK_SA: return launch_sa_si_fused<P, T>((const SaLaunch *)f.recs, f.work, f.nwork, f.smem, st);
    default:
        if constexpr (std::is_same<P, float>::value)
            return launch_sa_si_f32_fused<P>((const SaLaunch *)f.recs, f.work, f.nwork, st);
        return cudaErrorInvalidValue;
    }
}

static int32_t enqueue_fused(ss_batch *bt, int what, cudaStream_t st) {
    for (int dir = 1; dir <= 2; dir++) {
        if (!(what & dir)) continue;
        for (const FusedLaunch &f : dir == 1 ? bt->fwd : bt->inv) {
            cudaError_t e = f.tl == TL_F64 ? fused_launch<double, double>(f, st)
                            : f.tl == TL_DF64 ? fused_launch<double, df64>(f, st)
                                              : fused_launch<float, float>(f, st);
            CUDA_TRY(e);
        }
        for (ss_grid *g : bt->unfused) {
            int32_t r = run_direction(g, dir, st);
            if (r) return r;
        }
    }
    return SS_OK;
}

// Autotuner of the fused plan: CTA size of the ring kernels and items per ring
// CTA, timed on the batch's own data (both directions); the fastest is kept.
static int32_t autotune_fused(ss_batch *bt, cudaStream_t st) {
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    float best = 1e30f;
    int best_t = -1, best_s = 1;
    for (int threads : {128, 256})
        for (int scale : {1, 2}) {
            for (ss_grid *g : bt->grids) g->ring_threads_fwd = g->ring_threads_inv = threads;
            bt->ib_scale = scale;
            int32_t r = build_fused(bt);
            if (!r) r = enqueue_fused(bt, 3, st);  // warm-up
            if (r) { cudaEventDestroy(a); cudaEventDestroy(b); return r; }
            CUDA_TRY(cudaEventRecord(a, st));
            for (int rep = 0; rep < 2 && !r; rep++) r = enqueue_fused(bt, 3, st);
            CUDA_TRY(cudaEventRecord(b, st));
            CUDA_TRY(cudaEventSynchronize(b));
            if (r) { cudaEventDestroy(a); cudaEventDestroy(b); return r; }
            float ms = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
            if (ms < best) { best = ms; best_t = threads; best_s = scale; }
        }
    for (ss_grid *g : bt->grids) g->ring_threads_fwd = g->ring_threads_inv = best_t;
    bt->ib_scale = best_s;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return build_fused(bt);
}

extern "C" int32_t ss_batch_destroy(ss_batch *bt);
extern "C" int32_t ss_batch_create(ss_grid *const *grids, int32_t n, int32_t flags, ss_batch **out) {
    if (!out || !grids || n < 1) { set_error("bad batch arguments"); return SS_BAD_ARG; }
    *out = nullptr;
    ss_batch *bt = new ss_batch();
    for (int i = 0; i < n; i++) {
        if (!grids[i]) { delete bt; set_error("null grid in batch"); return SS_BAD_ARG; }
        bt->grids.push_back(grids[i]);
    }
    bt->device = grids[0]->device;
    cudaSetDevice(bt->device);
    if (cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete bt;
        set_error("cudaStreamCreate failed");
        return SS_CUDA_ERROR;
    }
    const int nside = std::min(n, 8);
    for (int i = 0; i < nside; i++) {
        cudaStream_t s;
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        bt->side.push_back(s);
    }
    for (int i = 0; i < nside + 1; i++) {
        cudaEvent_t e;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        bt->ev.push_back(e);
    }
    bt->fused = (flags & SS_BATCH_FUSED) != 0;
    if (bt->fused) {
        for (ss_grid *g : bt->grids)
            if (g->profiling) { ss_batch_destroy(bt); set_error("disable stage profiling on batched grids"); return SS_BAD_ARG; }
        int32_t r = (flags & SS_BATCH_AUTOTUNE) ? autotune_fused(bt, bt->stream) : build_fused(bt);
        if (r) { ss_batch_destroy(bt); return r; }
    } else if (flags & SS_BATCH_AUTOTUNE) {
        for (ss_grid *g : bt->grids) {
            int32_t r = autotune_grid(g, bt->stream);
            if (r) { ss_batch_destroy(bt); return r; }
        }
    }
    *out = bt;
    return SS_OK;
}

extern "C" int32_t ss_batch_destroy(ss_batch *bt) {
    if (!bt) return SS_OK;
    cudaSetDevice(bt->device);
    cudaStreamSynchronize(bt->stream);
    for (int i = 0; i < 4; i++) {
        if (bt->exec[i]) cudaGraphExecDestroy(bt->exec[i]);
        if (bt->graph[i]) cudaGraphDestroy(bt->graph[i]);
    }
    for (cudaStream_t s : bt->side) cudaStreamDestroy(s);
    for (cudaEvent_t e : bt->ev) cudaEventDestroy(e);
    free_fused(bt);
    cudaStreamDestroy(bt->stream);
    delete bt;
    return SS_OK;
}

// Enqueue every grid's transforms: grids round-robin over the side streams,
// forked from and joined back into `st` (the graph gets parallel branches).
static int32_t enqueue_batch(ss_batch *bt, int what, cudaStream_t st) {
    const int nside = (int)bt->side.size();
    CUDA_TRY(cudaEventRecord(bt->ev[0], st));
    for (int i = 0; i < nside; i++) CUDA_TRY(cudaStreamWaitEvent(bt->side[i], bt->ev[0], 0));
    for (size_t i = 0; i < bt->grids.size(); i++) {
        int32_t r = run_direction(bt->grids[i], what, bt->side[i % nside]);
        if (r) return r;
    }
    for (int i = 0; i < nside; i++) {
        CUDA_TRY(cudaEventRecord(bt->ev[1 + i], bt->side[i]));
        CUDA_TRY(cudaStreamWaitEvent(st, bt->ev[1 + i], 0));
    }
    return SS_OK;
}

extern "C" int32_t ss_batch_run(ss_batch *bt, int32_t what, int32_t use_graph, void *stream) {
    if (!bt || what < 1 || what > 3) { set_error("bad batch run arguments"); return SS_BAD_ARG; }
    cudaSetDevice(bt->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : bt->stream;
    for (ss_grid *g : bt->grids)
        if (g->profiling) { set_error("disable stage profiling on batched grids"); return SS_BAD_ARG; }
    if (bt->fused && bt->fused_gen != generations(bt)) {  // records hold the old ahat pointer / filter flag
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaStreamSynchronize(bt->stream));
        int32_t r = build_fused(bt);
        if (r) return r;
    }
    if (!use_graph) return bt->fused ? enqueue_fused(bt, what, st) : enqueue_batch(bt, what, st);
    if (bt->exec[what] && bt->gen[what] != generations(bt)) {
        CUDA_TRY(cudaStreamSynchronize(st));  // a replay in flight still uses the old graph
        cudaGraphExecDestroy(bt->exec[what]);
        cudaGraphDestroy(bt->graph[what]);
        bt->exec[what] = nullptr;
        bt->graph[what] = nullptr;
    }
    if (!bt->exec[what]) {
        // capture on the batch's own stream, then launch the graph on `st`
        CUDA_TRY(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeRelaxed));
        int32_t r = bt->fused ? enqueue_fused(bt, what, bt->stream) : enqueue_batch(bt, what, bt->stream);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(bt->stream, &graph);
        if (r) { if (graph) cudaGraphDestroy(graph); return r; }
        if (e != cudaSuccess) { set_error("graph capture failed: %s", cudaGetErrorString(e)); return SS_CUDA_ERROR; }
        bt->graph[what] = graph;
        CUDA_TRY(cudaGraphInstantiate(&bt->exec[what], graph, 0));
        bt->gen[what] = generations(bt);
    }
    CUDA_TRY(cudaGraphLaunch(bt->exec[what], st));
    return SS_OK;
}

extern "C" int32_t ss_batch_synchronize(ss_batch *bt) {
    if (!bt) { set_error("null batch"); return SS_BAD_ARG; }
    cudaSetDevice(bt->device);
    CUDA_TRY(cudaStreamSynchronize(bt->stream));
    return SS_OK;
}

extern "C" int32_t ss_batch_fused_launches(const ss_batch *bt, int32_t what, int32_t *launches) {
    if (!bt || !launches || what < 1 || what > 3) { set_error("bad batch query"); return SS_BAD_ARG; }
    *launches = (int32_t)(((what & 1) ? bt->fwd.size() : 0) + ((what & 2) ? bt->inv.size() : 0));
    return SS_OK;
}

extern "C" int32_t ss_batch_ring_threads(const ss_batch *bt, int32_t i, int32_t *fwd, int32_t *inv) {
    if (!bt || i < 0 || i >= (int)bt->grids.size()) { set_error("bad batch index"); return SS_BAD_ARG; }
    if (fwd) *fwd = bt->grids[i]->ring_threads_fwd;
    if (inv) *inv = bt->grids[i]->ring_threads_inv;
    return SS_OK;
}

// ====================================================================== chain
struct IfaceDev {
    int primary, secondary, pside, sside;
    int node[3];
    double C[9];
};

struct ss_chain {
    std::vector<ss_grid *> g;
    std::vector<IfaceDev> ifs;
    std::vector<int> layer_of;
    int nlayers = 0;
    std::vector<double *> state;  // per patch: [v][3][b] spline-object ahat (device)
    double *coupled = nullptr;
    size_t coupled_len = 0;
    int device = 0;
    std::vector<cudaEvent_t> ev;  // ordering between the patches' streams and the chain's stream
};

static double grid_DX(const ss_grid *g) { return (g->p.iMax - g->p.iMin) / g->p.num_cells; }

// PatchChain (embedded = false) or PatchEmbedded (embedded = true)
static int32_t chain_build(ss_grid *const *grids, int32_t n, bool embedded, ss_chain **out) {
    if (!out || !grids || n < 2) {
        set_error("%s requires at least 2 grids, got %d", embedded ? "PatchEmbedded" : "PatchChain", n);
        return SS_BAD_ARG;
    }
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        if (!grids[i] || grids[i]->rlz != grids[0]->rlz || grids[i]->d.nvars != grids[0]->d.nvars ||
            grids[i]->d.b_kDim != grids[0]->d.b_kDim) {
            set_error("the chain supports RL or RLZ patches with equal variable counts (and Chebyshev modes)");
            return SS_BAD_ARG;
        }
        for (auto &sh : grids[i]->spl_host)
            if (sh.periodic) {
                set_error("a patch of a chain cannot have a PERIODIC spline (patches couple at their ends)");
                return SS_UNSUPPORTED_BC;
            }
    }
    ss_chain *c = new ss_chain();
    c->device = grids[0]->device;
    cudaSetDevice(c->device);
    for (int i = 0; i < n; i++) c->g.push_back(grids[i]);
    const int nv = (int)grids[0]->d.nvars;
    for (int k = 0; embedded && k < n - 1; k++) {
        // PatchEmbedded (src/multipatch.jl:891-925): the inner grid k+1 takes R3X data
        // from grid k at both ends through stacked interfaces whose primary nodes sit
        // at the inner boundary (_compute_primary_node_index, :190-207, 270-276)
        const ss_grid *P = grids[k], *S = grids[k + 1];
        const double pDX = grid_DX(P), sDX = grid_DX(S), ratio = pDX / sDX;
        if (std::fabs(ratio - 1.0) < 1e-12 * std::max(pDX, sDX)) {
            delete c;
            set_error("PatchEmbedded requires refinement at each level (grids %d and %d have DX=%g)", k + 1, k + 2, pDX);
            return SS_BAD_ARG;
        }
        if (std::fabs(ratio - 2.0) >= 1e-12 * std::max(pDX, sDX)) {
            delete c;
            set_error("Only 1:1 and 2:1 coarse-to-fine ratios are supported, got %g:1", ratio);
            return SS_BAD_ARG;
        }
        for (int v = 0; v < nv; v++)
            if (!S->spl_host[v].r3x) {
                delete c;
                set_error("embedded grid %d needs R3X (FixedBC) at both ends", k + 2);
                return SS_UNSUPPORTED_BC;
            }
        for (int side = 0; side < 2; side++) {  // (outer, inner, :right, :left), then (:left, :right)
            IfaceDev f{};
            f.primary = k;
            f.secondary = k + 1;
            f.pside = side == 0 ? 1 : 0;
            f.sside = side == 0 ? 0 : 1;
            static const double M2[9] = {0.5, 0.5, 0.0, 0.125, 0.75, 0.125, 0.0, 0.5, 0.5};
            std::memcpy(f.C, M2, sizeof M2);
            const double xb = f.sside == 0 ? S->p.iMin : S->p.iMax;
            const long m = std::lround((xb - P->p.iMin) / pDX);
            const double xn = P->p.iMin + (double)m * pDX;
            if (std::fabs(xn - xb) > 1e-12 * pDX || m < 0 || m + 2 > (long)P->d.b_iDim - 1) {
                delete c;
                set_error("inner boundary %g does not align with a node of its parent", xb);
                return SS_BAD_ARG;
            }
            f.node[0] = (int)m; f.node[1] = (int)m + 1; f.node[2] = (int)m + 2;
            c->ifs.push_back(f);
        }
    }
    for (int k = 0; !embedded && k < n - 1; k++) {
        IfaceDev f{};
        // PatchChain (src/multipatch.jl:825-848): the coarser side is primary
        if (grid_DX(grids[k]) >= grid_DX(grids[k + 1])) { f.primary = k; f.secondary = k + 1; f.pside = 1; f.sside = 0; }
        else { f.primary = k + 1; f.secondary = k; f.pside = 0; f.sside = 1; }
        const ss_grid *P = grids[f.primary], *S = grids[f.secondary];
        const double pDX = grid_DX(P), sDX = grid_DX(S), ratio = pDX / sDX;
        const double tol = 1e-12 * std::max(pDX, sDX);
        static const double M1[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        static const double M2[9] = {0.5, 0.5, 0.0, 0.125, 0.75, 0.125, 0.0, 0.5, 0.5};
        if (std::fabs(ratio - 1.0) < tol) std::memcpy(f.C, M1, sizeof M1);
        else if (std::fabs(ratio - 2.0) < tol) std::memcpy(f.C, M2, sizeof M2);
        else { delete c; set_error("Only 1:1 and 2:1 coarse-to-fine ratios are supported, got %g:1", ratio); return SS_BAD_ARG; }
        for (int v = 0; v < nv; v++) {
            if (!S->spl_host[v].r3x || P->spl_host[v].r3x) {
                delete c;
                set_error("chain interface %d: the secondary needs R3X (FixedBC) and the primary must not be R3X", k);
                return SS_UNSUPPORTED_BC;
            }
        }
        const int b = (int)P->d.b_iDim;
        if (f.pside == 1) { f.node[0] = b - 3; f.node[1] = b - 2; f.node[2] = b - 1; }
        else { f.node[0] = 0; f.node[1] = 1; f.node[2] = 2; }
        c->ifs.push_back(f);
    }
    c->layer_of.assign(n, 0);
    for (int it = 0; it < n + 2; it++) {
        bool changed = false;
        for (auto &f : c->ifs) {
            int need = c->layer_of[f.primary] + 1;
            if (c->layer_of[f.secondary] < need) { c->layer_of[f.secondary] = need; changed = true; }
        }
        if (!changed) break;
    }
    for (int v : c->layer_of) c->nlayers = std::max(c->nlayers, v + 1);
    size_t maxq = 0;
    for (auto &f : c->ifs) {
        const ss_grid *P = grids[f.primary], *S = grids[f.secondary];
        size_t nq = 1 + 2 * (size_t)std::min(P->d.kDim_wn, S->d.kDim_wn);
        maxq = std::max(maxq, nq);
    }
    c->state.assign(n, nullptr);
    for (int i = 0; i < n; i++) {
        size_t bytes = (size_t)nv * 3 * grids[i]->d.b_iDim * sizeof(double);
        if (cudaMalloc(&c->state[i], bytes) != cudaSuccess) { cudaGetLastError(); set_error("out of device memory"); return SS_OUT_OF_MEMORY; }
        cudaMemset(c->state[i], 0, bytes);
    }
    c->coupled_len = (size_t)nv * grids[0]->d.b_kDim * maxq * 3;
    if (cudaMalloc(&c->coupled, c->coupled_len * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        set_error("out of device memory");
        return SS_OUT_OF_MEMORY;
    }
    // secondaries keep their per-wavenumber registry resident
    for (auto &f : c->ifs) {
        ss_grid *S = grids[f.secondary];
        if (!S->d_ahat) {
            size_t bytes = (size_t)S->d.nvars * S->d.n_blocks * S->d.b_iDim * sizeof(double);
            if (cudaMalloc((void **)&S->d_ahat, bytes) != cudaSuccess) { cudaGetLastError(); set_error("out of device memory"); return SS_OUT_OF_MEMORY; }
            cudaMemset(S->d_ahat, 0, bytes);
            S->allocs.push_back(S->d_ahat);
        }
    }
    for (int i = 0; i < n + 1; i++) {
        cudaEvent_t e;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        c->ev.push_back(e);
    }
    cudaDeviceSynchronize();
    *out = c;
    return SS_OK;
}

extern "C" int32_t ss_chain_create(ss_grid *const *grids, int32_t n, ss_chain **out) {
    return chain_build(grids, n, false, out);
}

extern "C" int32_t ss_chain_create_embedded(ss_grid *const *grids, int32_t n, ss_chain **out) {
    return chain_build(grids, n, true, out);
}

extern "C" int32_t ss_chain_destroy(ss_chain *c) {
    if (!c) return SS_OK;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (double *p : c->state) cudaFree(p);
    for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
    cudaFree(c->coupled);
    delete c;
    return SS_OK;
}

// update_interface! for an RL secondary (_rl_kernel!, src/multipatch.jl:417-478)
// or an RLZ one (_rlz_kernel!, :496-571: every Chebyshev level z_b, primary
// blocks z_b·(1+2K_p) + q, registry blocks z_b·(1+2K_s) + q)
static int32_t update_interface(ss_chain *c, const IfaceDev &f, cudaStream_t st) {
    ss_grid *P = c->g[f.primary], *S = c->g[f.secondary];
    ChainLaunch L{};
    L.spec = P->spec;
    L.spl = P->d_spl;
    L.coupled = c->coupled;
    L.state = c->state[f.secondary];
    L.reg = S->d_ahat;
    L.nspec_p = P->d.n_spectral;
    L.nblocks_s = S->d.n_blocks;
    L.b_p = (int)P->d.b_iDim;
    L.b_s = (int)S->d.b_iDim;
    L.ld = (L.b_p % 2) ? L.b_p : L.b_p + 1;
    L.nq = 1 + 2 * (int)std::min(P->d.kDim_wn, S->d.kDim_wn);
    L.nvars = (int)P->d.nvars;
    L.bk = (int)P->d.b_kDim;  // 1 for RL
    L.zblk_p = 1 + 2 * (int)P->d.kDim_wn;
    L.zblk_s = 1 + 2 * (int)S->d.kDim_wn;
    L.side = f.sside;
    L.pstate = c->state[f.primary];
    for (int i = 0; i < 3; i++) L.node[i] = f.node[i];
    std::memcpy(L.C, f.C, sizeof L.C);
    int nmax = 0;
    for (auto &sh : P->spl_host) nmax = std::max(nmax, sh.Min);
    size_t smem = (size_t(32) * L.ld + size_t(5) * nmax) * sizeof(double);
    if (P->esz == 8) CUDA_TRY(launch_chain_couple<double>(L, smem, st));
    else CUDA_TRY(launch_chain_couple<float>(L, smem, st));
    CUDA_TRY(launch_chain_assemble(L, st));
    return SS_OK;
}

extern "C" int32_t ss_multi_grid_transform(ss_chain *c, void *stream) {
    if (!c) { set_error("null chain"); return SS_BAD_ARG; }
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : c->g[0]->stream;
    // earlier work on every patch's own stream comes first
    for (size_t i = 0; i < c->g.size(); i++) {
        CUDA_TRY(cudaEventRecord(c->ev[i], c->g[i]->stream));
        CUDA_TRY(cudaStreamWaitEvent(st, c->ev[i], 0));
    }
    // patches run on `st` in topological order (multiGridTransform!, src/multipatch.jl:769-786)
    for (int L = 0; L < c->nlayers; L++) {
        for (size_t i = 0; i < c->g.size(); i++)
            if (c->layer_of[i] == L) {
                int32_t r = grid_inverse(c->g[i], st);
                if (r) return r;
            }
        for (auto &f : c->ifs)
            if (c->layer_of[f.primary] == L) {
                int32_t r = update_interface(c, f, st);
                if (r) return r;
            }
    }
    // and later work on each patch's own stream (downloads) comes after
    CUDA_TRY(cudaEventRecord(c->ev[c->g.size()], st));
    for (size_t i = 0; i < c->g.size(); i++) CUDA_TRY(cudaStreamWaitEvent(c->g[i]->stream, c->ev[c->g.size()], 0));
    return SS_OK;
}

// ====================================================================== tiles
// sumSpectralTile! (set = 0) / setSpectralTile!'s write (set = 1)
extern "C" int32_t ss_tile_sum_spectral(ss_grid *patch, const ss_grid *tile, int32_t set, void *stream) {
    if (!patch || !tile) { set_error("null grid"); return SS_BAD_ARG; }
    if (patch->rlz != tile->rlz || patch->esz != tile->esz || patch->d.nvars != tile->d.nvars ||
        patch->d.b_kDim != tile->d.b_kDim || patch->p.mubar != tile->p.mubar) {
        set_error("tile and patch disagree in geometry, precision, variables or Chebyshev modes");
        return SS_BAD_SHAPE;
    }
    const int offset = (tile->pOL - patch->pOL) / patch->p.mubar;  // spectralIndexL - 1
    if (offset < 0 || offset + tile->d.b_iDim > patch->d.b_iDim || tile->d.kDim_wn > patch->d.kDim_wn) {
        set_error("tile does not lie inside the patch");
        return SS_BAD_SHAPE;
    }
    cudaSetDevice(patch->device);
    TileLaunch T{};
    T.patch = patch->spec;
    T.tile = tile->spec;
    T.nspec_p = patch->d.n_spectral;
    T.nspec_t = tile->d.n_spectral;
    T.b_p = (int)patch->d.b_iDim;
    T.b_t = (int)tile->d.b_iDim;
    T.blocks_p = 1 + 2 * (int)patch->d.kDim_wn;
    T.blocks_t = 1 + 2 * (int)tile->d.kDim_wn;
    T.bk = (int)patch->d.b_kDim;
    T.nvars = (int)patch->d.nvars;
    T.offset = offset;
    T.set = set ? 1 : 0;
    cudaStream_t st = stream ? (cudaStream_t)stream : patch->stream;
    if (patch->esz == 8) CUDA_TRY(launch_tile_sum<double>(T, st));
    else CUDA_TRY(launch_tile_sum<float>(T, st));
    return SS_OK;
}

// Copy the tile's rings of one physical slot between patch and tile
// (direction 0: patch → tile, 1: tile → patch); slot 0 = every slot.
extern "C" int32_t ss_tile_copy_physical(ss_grid *patch, ss_grid *tile, int32_t slot, int32_t direction,
                                         void *stream) {
    if (!patch || !tile) { set_error("null grid"); return SS_BAD_ARG; }
    if (patch->rlz != tile->rlz || patch->esz != tile->esz || patch->d.nvars != tile->d.nvars ||
        patch->d.kDim != tile->d.kDim || slot < 0 || slot > patch->d.nslots) {
        set_error("tile and patch disagree in geometry, precision, variables or levels");
        return SS_BAD_SHAPE;
    }
    // rings of the tile start after the patch rings below the tile's offset
    int64_t row0 = 0;
    for (int ri = patch->pOL + 1; ri <= tile->pOL; ri++) row0 += 4 + 4 * ri;
    row0 *= patch->d.kDim;
    if (row0 + tile->d.n_physical > patch->d.n_physical) { set_error("tile does not lie inside the patch"); return SS_BAD_SHAPE; }
    cudaSetDevice(patch->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : patch->stream;
    const size_t es = patch->esz;
    const int s0 = slot ? slot - 1 : 0, s1 = slot ? slot : (int)patch->d.nslots;
    for (int s = s0; s < s1; s++)
        for (int v = 0; v < patch->d.nvars; v++) {
            char *pp = (char *)patch->phys + ((size_t)s * patch->d.nvars + v) * patch->d.n_physical * es + row0 * es;
            char *tp = (char *)tile->phys + ((size_t)s * tile->d.nvars + v) * tile->d.n_physical * es;
            if (direction == 0) CUDA_TRY(cudaMemcpyAsync(tp, pp, tile->d.n_physical * es, cudaMemcpyDeviceToDevice, st));
            else CUDA_TRY(cudaMemcpyAsync(pp, tp, tile->d.n_physical * es, cudaMemcpyDeviceToDevice, st));
        }
    return SS_OK;
}

extern "C" int32_t ss_grid_zero_spectral(ss_grid *g, void *stream) {
    if (!g) { set_error("null grid"); return SS_BAD_ARG; }
    cudaSetDevice(g->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    CUDA_TRY(cudaMemsetAsync(g->spec, 0, (size_t)g->d.n_spectral * g->d.nvars * g->esz, st));
    return SS_OK;
}
