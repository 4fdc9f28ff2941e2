// ss_grid.h — the device-resident grid object behind ss_grid* (internal).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "ss_internal.h"

using namespace ss;

// radial chunks of the host-overlapped transforms (copies of one chunk run
// while the next one computes)
constexpr int kHostChunks = 4;

struct RingBucket {
    int offset;   // into the ring list
    int count;
    size_t smem_fwd_f64, smem_inv_f64;
    int max_buf, max_kmax;
};

struct ss_grid {
    ss_grid_params p{};
    std::vector<double> l_q;
    std::vector<ss_spline_bc> bcl, bcr;
    std::vector<int32_t> bcb, bct, kmaxv;
    int32_t ring_kmax = -1;  // RLZ: kmax cap of the rings all variables share
    // bumped by every call that changes what a launch sequence captures (the
    // ahat pointer, the filter flag): batches re-capture their graphs on change
    uint64_t generation = 0;
    ss_dims d{};
    int prec = SS_PREC_F64;
    int tl = TL_F64;   // compute layout of tables and intermediates
    size_t esz = 8;    // storage bytes of physical/spectral and of intermediates
    int device = 0;
    cudaStream_t stream = nullptr;
    int nitems = 0, nslots_z = 0, pOL = 0, rlz = 0;
    int64_t frows = 0;

    void *phys = nullptr, *spec = nullptr, *C = nullptr, *F = nullptr, *G = nullptr, *H = nullptr;
    void *sa_x = nullptr, *sa_y = nullptr;  // binary32 SAtransform! scratch (alias F / phys when large enough)
    void *stage = nullptr;
    size_t stage_bytes = 0;

    RingDesc *d_rings = nullptr;
    int *d_ring_list = nullptr;
    FftPlan *d_plans = nullptr;
    void *d_pool = nullptr, *d_phase = nullptr;
    int64_t *d_fofs = nullptr;
    SplineDev *d_spl = nullptr;
    ChebDev *d_cheb = nullptr;
    double *d_ahat = nullptr, *d_fw = nullptr, *d_cw = nullptr;
    int filtered = 0;
    int ring_threads_fwd = 256, ring_threads_inv = 256;  // CTA size of the ring kernels (autotuned by batches)
    int sms = 152;                                        // SMs of the grid's device
    std::vector<RingBucket> buckets;
    // radial chunks of the host-overlapped transforms: chunk c holds rings
    // [chunk_r0[c], chunk_r0[c+1]); its rings of bucket b are the segment
    // chunk_seg[c][b] = (offset, count) of d_ring_list_chunks
    std::vector<int> chunk_r0;
    std::vector<std::vector<std::pair<int, int>>> chunk_seg;
    int *d_ring_list_chunks = nullptr;
    int *d_col_ring = nullptr;       // RLZ: ring index of every column (ring point)
    std::vector<int64_t> ring_jofs;  // first ring point of every ring, jDim at the end
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> chunk_ev;
    std::vector<void *> allocs;
    std::vector<SplineHost> spl_host;
    // stage instrumentation
    int profiling = 0;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    struct Mark { int stage; cudaEvent_t a, b; };
    std::vector<Mark> marks;
    int64_t launches[SS_NSTAGES] = {0, 0, 0, 0, 0, 0};
    double stage_ms[SS_NSTAGES] = {0, 0, 0, 0, 0, 0};
};

static cudaEvent_t next_event(ss_grid *g) {
    if (g->ev_used == g->ev_pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        g->ev_pool.push_back(e);
    }
    return g->ev_pool[g->ev_used++];
}
// brackets one stage with events when profiling is on
struct StageScope {
    ss_grid *g;
    int stage;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    StageScope(ss_grid *g_, int s_, cudaStream_t st_) : g(g_), stage(s_), st(st_) {
        if (g->profiling) {
            a = next_event(g);
            cudaEventRecord(a, st);
        }
    }
    ~StageScope() {
        if (g->profiling) {
            cudaEvent_t b = next_event(g);
            cudaEventRecord(b, st);
            g->marks.push_back({stage, a, b});
        }
    }
};


namespace ss {
// per-grid launch entry points shared by the single-grid, batch and chain paths
int32_t grid_forward(ss_grid *g, cudaStream_t st);
int32_t grid_inverse(ss_grid *g, cudaStream_t st);
// SI + ring (+ column) stages only: the spectral array holds spline coefficients a
int32_t grid_inverse_coeffs(ss_grid *g, cudaStream_t st);
}  // namespace ss

namespace ss {
struct RingLaunch;
struct SbLaunch;
struct SaLaunch;
// launch records of one grid's stages (ring_list and ib are set per launch;
// the record types are defined in ss_kernels.h)
RingLaunch ring_record(const ss_grid *g, bool inverse);
size_t ring_item_smem(const ss_grid *g, const RingBucket &bkt, bool inverse);
SbLaunch sb_record(const ss_grid *g);
SaLaunch sa_record(const ss_grid *g, int coeffs, size_t *smem_generic);
}  // namespace ss
