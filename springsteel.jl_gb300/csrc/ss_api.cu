// ss_api.cu — the C ABI of libspringsteel_gpu (include/springsteel_gpu.h).
//
// An ss_grid is the device-resident counterpart of a SpringsteelGrid of RL or
// RLZ geometry (src/types.jl:249-256): the physical and spectral arrays stay
// in HBM; the FP64 tables built by ss_setup.cpp are uploaded once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ss_grid.h"
#include "ss_internal.h"
#include "ss_kernels.h"
#include "ss_df64.cuh"

namespace ss {
static thread_local std::string g_err;
void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}
}  // namespace ss

using namespace ss;

#define CUDA_TRY(expr)                                                                      \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) {                                                            \
            set_error("%s failed: %s", #expr, cudaGetErrorString(_e));                      \
            return (_e == cudaErrorMemoryAllocation) ? SS_OUT_OF_MEMORY : SS_CUDA_ERROR;   \
        }                                                                                   \
    } while (0)

static int32_t dev_alloc(ss_grid *g, void **p, size_t bytes, bool zero = true) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        set_error("cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SS_OUT_OF_MEMORY : SS_CUDA_ERROR;
    }
    g->allocs.push_back(*p);
    if (zero) CUDA_TRY(cudaMemsetAsync(*p, 0, bytes, g->stream));
    return SS_OK;
}

template <typename V>
static int32_t upload_vec(ss_grid *g, V **dst, const std::vector<V> &src) {
    int32_t st = dev_alloc(g, (void **)dst, src.size() * sizeof(V), false);
    if (st) return st;
    if (!src.empty()) CUDA_TRY(cudaMemcpy(*dst, src.data(), src.size() * sizeof(V), cudaMemcpyHostToDevice));
    return SS_OK;
}

// FP64 host tables → the compute layout of the grid (TL_F64 / TL_DF64 / TL_F32)
static std::vector<unsigned char> real_layout(const std::vector<double> &v, int tl) {
    std::vector<unsigned char> out;
    if (tl == TL_F64) {
        out.resize(v.size() * 8);
        std::memcpy(out.data(), v.data(), out.size());
    } else if (tl == TL_F32) {
        out.resize(v.size() * 4);
        float *f = (float *)out.data();
        for (size_t i = 0; i < v.size(); i++) f[i] = (float)v[i];
    } else {
        out.resize(v.size() * 8);
        float *f = (float *)out.data();
        for (size_t i = 0; i < v.size(); i++) {
            f[2 * i] = (float)v[i];
            f[2 * i + 1] = (float)(v[i] - (double)f[2 * i]);
        }
    }
    if (out.empty()) out.resize(16, 0);
    return out;
}
// interleaved (re, im) FP64 pairs → double2 / float2 / float4 (re.hi, re.lo, im.hi, im.lo)
static std::vector<unsigned char> cplx_layout(const std::vector<double> &v, int tl) {
    if (tl != TL_DF64) return real_layout(v, tl);
    std::vector<unsigned char> out(v.size() * 8);
    float *f = (float *)out.data();
    for (size_t i = 0; i < v.size(); i++) {
        f[2 * i] = (float)v[i];
        f[2 * i + 1] = (float)(v[i] - (double)f[2 * i]);
    }
    if (out.empty()) out.resize(16, 0);
    return out;
}
static int32_t upload_bytes(ss_grid *g, const void **dst, const std::vector<unsigned char> &src) {
    void *p = nullptr;
    int32_t st = dev_alloc(g, &p, src.size(), false);
    if (st) return st;
    CUDA_TRY(cudaMemcpy(p, src.data(), src.size(), cudaMemcpyHostToDevice));
    *dst = p;
    return SS_OK;
}

static void free_grid(ss_grid *g) {
    if (!g) return;
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->copy_stream) cudaStreamSynchronize(g->copy_stream);
    for (cudaEvent_t e : g->ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : g->chunk_ev) cudaEventDestroy(e);
    for (void *p : g->allocs) cudaFree(p);
    if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}


// FFT plan-set limits of a compute layout: direct prime passes up to 67 (FP64,
// double-float) or 127 (binary32) and one Rader pass above.  Measured with the
// DFT-matrix prime passes: 200-cell FP64 RLZ ring_inverse 40.6 ms at 31, 40.0 at
// 67, 40.9 at 127, 43.8 at 199; 400-cell binary32 ring_inverse + ring_forward
// 88.1 ms at 31, 83.9 at 67, 82.4 at 127, 83.6 at 199.  Rader inner lengths with
// a prime factor above 67 run as zero-padded smooth convolutions (200-cell FP64
// ring stages 47.6 ms unpadded, 46.0 ms padded above 67, 46.6 above 31; 400-cell
// binary32 81.8 ms unpadded, 80.1 padded above 67).  Tuning overrides:
// SS_FFT_MAX_PRIME (13-199), SS_FFT_RADER (0: Bluestein), SS_FFT_RADER_PAD.
static void configure_plans(PlanSet &plans, int tl) {
    plans.max_prime = (tl == TL_F32) ? 127 : 67;
    plans.rader = true;
    if (const char *e = std::getenv("SS_FFT_MAX_PRIME")) {
        const int v = std::atoi(e);
        if (v >= 13 && v <= kMaxPrimeRadix) plans.max_prime = v;
    }
    if (const char *e = std::getenv("SS_FFT_RADER")) plans.rader = std::atoi(e) != 0;
    plans.pad_prime = 67;
    if (const char *e = std::getenv("SS_FFT_RADER_PAD")) {
        const int v = std::atoi(e);
        if (v >= 13 && v <= kMaxPrimeRadix) plans.pad_prime = v;
    }
}

static int32_t build_grid(ss_grid *g) {
    const ss_grid_params &p = g->p;
    const int nv = p.nvars;
    const int iDim = p.num_cells * p.mubar;
    g->rlz = p.geometry == SS_GEOM_RLZ;
    g->pOL = p.patchOffsetL;
    g->prec = p.precision;
    g->tl = p.precision == SS_PREC_F32_REFINED ? TL_F32 : (p.precision == SS_PREC_F64_FAST ? TL_DF64 : TL_F64);
    g->esz = p.precision == SS_PREC_F32_REFINED ? 4 : 8;
    int kz = 1, bk = 1;
    if (g->rlz) {
        kz = p.kDim;
        if (kz < 2) { set_error("RLZ needs kDim >= 2"); return SS_BAD_SHAPE; }
        bk = p.b_kDim > 0 ? p.b_kDim : (int)std::min<double>(kz, std::floor((2.0 * kz - 1) / 3.0) + 1);
        if (bk < 1 || bk > kz) { set_error("b_kDim out of range"); return SS_BAD_SHAPE; }
    }
    const int K = iDim + g->pOL;
    ss_dims &d = g->d;
    d.iDim = iDim;
    d.b_iDim = p.num_cells + 3;
    d.kDim = kz;
    d.b_kDim = bk;
    d.kDim_wn = K;
    d.nvars = nv;
    d.nslots = g->rlz ? 7 : 5;
    int64_t jDim = 0, bj = 0;
    for (int r = 1; r <= iDim; r++) { jDim += 4 + 4 * (r + g->pOL); bj += 1 + 2 * (r + g->pOL); }
    d.jDim = jDim;
    d.b_jDim = bj;
    d.n_physical = jDim * kz;
    d.n_blocks = (int64_t)bk * (1 + 2 * (int64_t)K);
    d.n_spectral = d.n_blocks * d.b_iDim;
    g->nitems = nv * bk;
    g->nslots_z = 1 + 2 * K;
    g->frows = bj;

    // ---- spline templates (one per variable; src/factory.jl:670-680)
    g->spl_host.resize(nv);
    std::vector<SplineDev> sdev(nv);
    for (int v = 0; v < nv; v++) {
        int32_t st = build_spline(p.iMin, p.iMax, p.num_cells, p.mubar, p.quadrature, g->l_q[v], g->bcl[v], g->bcr[v],
                                  g->spl_host[v]);
        if (st) return st;
        const SplineHost &sh = g->spl_host[v];
        SplineDev &sd = sdev[v];
        std::memset(&sd, 0, sizeof sd);
        sd.bDim = sh.bDim; sd.Min = sh.Min; sd.rankL = sh.rankL; sd.rankR = sh.rankR;
        sd.lk = sh.lk; sd.rk = sh.rk; sd.r3x = sh.r3x; sd.periodic = sh.periodic;
        sd.aL = sh.aL; sd.bL = sh.bL; sd.aR = sh.aR; sd.bR = sh.bR;
        std::vector<double> dinv(sh.Min);
        for (int i = 0; i < sh.Min; i++) dinv[i] = 1.0 / sh.L4[size_t(i) * 4];
        if ((st = upload_vec(g, &sd.L4, sh.L4))) return st;
        if ((st = upload_vec(g, &sd.dinv, dinv))) return st;
        if ((st = upload_vec(g, &sd.PQb, sh.PQb))) return st;
        std::vector<float> l4f(sh.L4.size()), dinvf(dinv.size());
        for (size_t i = 0; i < l4f.size(); i++) l4f[i] = (float)sh.L4[i];
        for (size_t i = 0; i < dinvf.size(); i++) dinvf[i] = (float)dinv[i];
        if ((st = upload_vec(g, &sd.L4f, l4f))) return st;
        if ((st = upload_vec(g, &sd.dinvf, dinvf))) return st;
        if ((st = upload_vec(g, &sd.Aband, sh.Aopen))) return st;
        if (sh.periodic) {  // the dense factor's last three rows and A's corners
            std::vector<float> tf(sh.tail.size());
            for (size_t i = 0; i < tf.size(); i++) tf[i] = (float)sh.tail[i];
            if ((st = upload_vec(g, &sd.tail, sh.tail))) return st;
            if ((st = upload_vec(g, &sd.tailf, tf))) return st;
            if ((st = upload_vec(g, &sd.acorner, sh.acorner))) return st;
        }
        if ((st = upload_bytes(g, &sd.sbw_t, real_layout(sh.sbw, g->tl)))) return st;
        if ((st = upload_bytes(g, &sd.siw_t, real_layout(sh.siw, g->tl)))) return st;
        if ((st = upload_vec(g, &sd.si_m0, sh.si_m0))) return st;
    }
    int32_t st = upload_vec(g, &g->d_spl, sdev);
    if (st) return st;

    // ---- rings (src/factory.jl:608-624) and FFT plans
    TwiddlePool pool;
    PlanSet plans;
    configure_plans(plans, g->tl);
    // CTA size of the ring kernels: FP64 butterflies leave fewer idle threads per
    // pass at 128 (measured on the 200-cell RLZ grid: 73.4 ms per round trip
    // against 77.2 at 256); binary32 is faster at 256 (156.9 against 172.2 ms on
    // the 400-cell grid).  Batches autotune it per grid.
    g->ring_threads_fwd = g->ring_threads_inv = (g->tl == TL_F64) ? 128 : 256;
    // tuning override (64, 128 or 256 threads)
    if (const char *e = std::getenv("SS_RING_THREADS")) {
        const int t = std::atoi(e);
        if (t == 64 || t == 128 || t == 256) g->ring_threads_fwd = g->ring_threads_inv = t;
    }
    std::vector<double> phase;
    const int nring_sets = g->rlz ? 1 : nv;
    std::vector<RingDesc> rings(size_t(nring_sets) * iDim);
    std::vector<int64_t> fofs(iDim);
    for (int set = 0; set < nring_sets; set++) {
        int64_t jo = 0, fo = 0;
        for (int r = 1; r <= iDim; r++) {
            RingDesc &rd = rings[size_t(set) * iDim + (r - 1)];
            const int ri = r + g->pOL;
            rd.L = 4 + 4 * ri;
            rd.ri = ri;
            int kmax = ri;
            const int var_kmax = g->rlz ? g->ring_kmax : g->kmaxv[set];
            if (var_kmax >= 0) kmax = std::min(var_kmax, ri);
            rd.kmax = kmax;
            rd.plan = plans.plan_for(rd.L / 2, pool);
            rd.utw = plans.unpack_for(rd.L, pool);
            // PhaseFilter(fp): cos(k*ymin), sin(k*ymin) with ymin = 0.5*(2π/L)*(ri-1)
            const double dl = 2 * 3.14159265358979323846 / rd.L;
            const double ymin = 0.5 * dl * (ri - 1);
            // cos/sin(k ymin) for every k ≤ ri, whatever this set's kmax: a CTA's
            // items (variables of an RL grid) index one ring set's table
            rd.phase = (int64_t)phase.size() / 2;
            for (int k = 1; k <= ri; k++) {
                phase.push_back(std::cos(k * ymin));
                phase.push_back(std::sin(k * ymin));
            }
            rd.jofs = jo;
            rd.fofs = fo;
            fofs[r - 1] = fo;
            jo += rd.L;
            fo += 1 + 2 * ri;
        }
    }
    if (phase.empty()) phase.assign(2, 0.0);
    if ((st = upload_vec(g, &g->d_rings, rings))) return st;
    if ((st = upload_vec(g, &g->d_fofs, fofs))) return st;
    if ((st = upload_vec(g, &g->d_plans, plans.plans))) return st;
    {
        const void *pp = nullptr, *ph = nullptr;
        if ((st = upload_bytes(g, &pp, cplx_layout(pool.v, g->tl)))) return st;
        if ((st = upload_bytes(g, &ph, cplx_layout(phase, g->tl)))) return st;
        g->d_pool = (void *)pp;
        g->d_phase = (void *)ph;
    }
    // buckets of rings by shared-memory need (largest first)
    {
        std::vector<int> order(iDim);
        for (int r = 0; r < iDim; r++) order[r] = r;
        auto bufof = [&](int r) { return fft_buffer_len(plans.plans[rings[r].plan]); };
        std::sort(order.begin(), order.end(), [&](int a, int b) { return bufof(a) > bufof(b); });
        size_t maxsm = 0;
        int dev = g->device;
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || g->sms <= 0)
            g->sms = 152;
        int i = 0;
        while (i < iDim) {
            RingBucket bkt{};
            bkt.offset = i;
            int top = bufof(order[i]);
            int j = i;
            while (j < iDim && bufof(order[j]) * 2 > top) j++;
            bkt.count = j - i;
            bkt.max_buf = top;
            int km = 0;  // the inverse kernel keeps ri + 1 ≥ kmax + 1 spectrum entries per item
            for (int q = i; q < j; q++) km = std::max(km, std::max(rings[order[q]].kmax, rings[order[q]].ri));
            bkt.max_kmax = km;
            bkt.smem_fwd_f64 = size_t(2) * top * 16;
            bkt.smem_inv_f64 = (size_t(2) * top + km + 1) * 16;
            maxsm = std::max(maxsm, bkt.smem_inv_f64 * (g->esz == 8 ? 1 : 2) / 2);
            g->buckets.push_back(bkt);
            i = j;
        }
        size_t need = 0;
        for (auto &bkt : g->buckets) need = std::max(need, (g->esz == 8) ? bkt.smem_inv_f64 : bkt.smem_inv_f64 / 2);
        if (optin > 0 && need > (size_t)optin) {
            set_error("ring of length %d needs %zu bytes of shared memory (> %d per block)", rings[order[0]].L, need, optin);
            return SS_BAD_SHAPE;
        }
        (void)maxsm;
        if ((st = upload_vec(g, &g->d_ring_list, order))) return st;

        // radial chunks of about equal point counts for the host-overlapped
        // transforms; within a chunk the rings keep their bucket order
        g->ring_jofs.resize(iDim + 1);
        for (int r = 0; r < iDim; r++) g->ring_jofs[r] = rings[r].jofs;
        g->ring_jofs[iDim] = rings[iDim - 1].jofs + rings[iDim - 1].L;
        const int nch = std::min(kHostChunks, iDim);
        g->chunk_r0.assign(1, 0);
        for (int c = 1; c < nch; c++) {
            const int64_t target = g->ring_jofs[iDim] * c / nch;
            int r = g->chunk_r0.back() + 1;
            while (r < iDim && g->ring_jofs[r] < target) r++;
            if (r < iDim) g->chunk_r0.push_back(r);
        }
        g->chunk_r0.push_back(iDim);
        std::vector<int> clist;
        g->chunk_seg.assign(g->chunk_r0.size() - 1, {});
        for (size_t c = 0; c + 1 < g->chunk_r0.size(); c++)
            for (const RingBucket &bkt : g->buckets) {
                const int off = (int)clist.size();
                for (int q = bkt.offset; q < bkt.offset + bkt.count; q++)
                    if (order[q] >= g->chunk_r0[c] && order[q] < g->chunk_r0[c + 1]) clist.push_back(order[q]);
                g->chunk_seg[c].push_back({off, (int)clist.size() - off});
            }
        if ((st = upload_vec(g, &g->d_ring_list_chunks, clist))) return st;
        if (g->rlz) {  // column → ring for the Chebyshev stages (one load instead of a search)
            std::vector<int> cr(g->ring_jofs[iDim]);
            for (int r = 0; r < iDim; r++)
                for (int64_t q = g->ring_jofs[r]; q < g->ring_jofs[r + 1]; q++) cr[q] = r;
            if ((st = upload_vec(g, &g->d_col_ring, cr))) return st;
        }
    }

    // ---- Chebyshev columns (src/factory.jl:722-728)
    if (g->rlz) {
        std::vector<ChebDev> cdev(nv);
        for (int v = 0; v < nv; v++) {
            ChebHost ch;
            st = build_cheb(kz, bk, g->bcb[v], g->bct[v], p.kMin, p.kMax, ch);
            if (st) return st;
            ChebDev &cd = cdev[v];
            std::memset(&cd, 0, sizeof cd);
            cd.N = ch.N; cd.bk = ch.bk; cd.nrank = ch.nrank; cd.half = ch.half; cd.dscale = ch.dscale;
            if ((st = upload_bytes(g, &cd.fwd_t, real_layout(ch.fwd, g->tl)))) return st;
            if ((st = upload_bytes(g, &cd.inv_e_t, real_layout(ch.inv_e, g->tl)))) return st;
            if ((st = upload_bytes(g, &cd.inv_o_t, real_layout(ch.inv_o, g->tl)))) return st;
            if ((st = upload_bytes(g, &cd.gu_t, real_layout(ch.gu, g->tl)))) return st;
            if ((st = upload_bytes(g, &cd.gv_t, real_layout(ch.gv, g->tl)))) return st;
            {
                const int N = ch.N, half = ch.half, ne = (N + 1) / 2, no = std::max(N / 2, 1);
                const int JP = cheb_pad4(half), KEP = cheb_pad4((ch.bk + 1) / 2), KOP = cheb_pad4(ch.bk / 2);
                std::vector<double> et((size_t)ne * JP, 0.0), ot((size_t)no * JP, 0.0);
                std::vector<double> fe((size_t)half * KEP, 0.0), fo((size_t)half * KOP, 0.0);
                for (int j = 0; j < half; j++) {
                    for (int k = 0; k < ne; k++) et[(size_t)k * JP + j] = ch.inv_e[(size_t)j * ne + k];
                    if (N / 2 > 0)
                        for (int k = 0; k < no; k++) ot[(size_t)k * JP + j] = ch.inv_o[(size_t)j * no + k];
                    for (int i = 0; 2 * i < ch.bk; i++) fe[(size_t)j * KEP + i] = ch.fwd[(size_t)(2 * i) * half + j];
                    for (int i = 0; 2 * i + 1 < ch.bk; i++) fo[(size_t)j * KOP + i] = ch.fwd[(size_t)(2 * i + 1) * half + j];
                }
                if ((st = upload_bytes(g, &cd.inv_et_t, real_layout(et, g->tl)))) return st;
                if ((st = upload_bytes(g, &cd.inv_ot_t, real_layout(ot, g->tl)))) return st;
                if ((st = upload_bytes(g, &cd.fwd_et_t, real_layout(fe, g->tl)))) return st;
                if ((st = upload_bytes(g, &cd.fwd_ot_t, real_layout(fo, g->tl)))) return st;
                // Composed inverse matrices.  G = Ĩ + V Uᵀ (CA: Ĩ keeps the bk modes, V = gvᵀ,
                // U = guᵀ), D the CIxcoefficients map (÷ dscale).  Columns: X_d = D^d [Ĩ | V].
                // D flips coefficient parity, so the output half of parity pe (even/odd k)
                // reads only the inputs i of parity (pe + d) mod 2 through D^d Ĩ, plus the
                // rank-nrank term through s = Uᵀ b.  Rows of table (d, pe): the K_q inputs of
                // that parity (i = 2i' + q), then the nrank rows of s; zero-padded to Kcap.
                const int B = ch.bk, nr = ch.nrank, Kcols = B + nr;
                const int Ke = (B + 1) / 2 + nr, Ko = B / 2 + nr, Kcap = std::max(Ke, Ko);
                std::vector<double> X((size_t)N * Kcols, 0.0), Xn((size_t)N * Kcols, 0.0);
                for (int k = 0; k < N; k++) {
                    if (k < B) X[(size_t)k * Kcols + k] = 1.0;
                    for (int p = 0; p < nr; p++) X[(size_t)k * Kcols + B + p] = ch.gv[(size_t)p * N + k];
                }
                std::vector<double> mt((size_t)6 * Kcap * JP, 0.0);
                for (int dd = 0; dd < 3; dd++) {
                    if (dd > 0) {
                        for (int k = 0; k < N; k++)
                            for (int c = 0; c < Kcols; c++) {
                                double acc = 0.0;  // (D X)[k][c] = Σ_{m > k, m − k odd} 2m X[m][c]
                                for (int m = k + 1; m < N; m += 2) acc += 2.0 * m * X[(size_t)m * Kcols + c];
                                Xn[(size_t)k * Kcols + c] = acc / ch.dscale;
                            }
                        X.swap(Xn);
                    }
                    for (int pe = 0; pe < 2; pe++) {
                        const int q = (pe + dd) & 1;  // input parity feeding this half
                        const int nq = q ? B / 2 : (B + 1) / 2;
                        const std::vector<double> &IT = pe ? ch.inv_o : ch.inv_e;
                        const int nk = pe ? no : ne;
                        double *tab = mt.data() + (size_t)(dd * 2 + pe) * Kcap * JP;
                        for (int j = 0; j < half; j++) {
                            for (int r = 0; r < nq + nr; r++) {
                                const int c = r < nq ? 2 * r + q : B + (r - nq);
                                double acc = 0.0;
                                for (int kk = 0; kk < nk; kk++) {
                                    const int k = 2 * kk + pe;
                                    if (k < N) acc += IT[(size_t)j * nk + kk] * X[(size_t)k * Kcols + c];
                                }
                                tab[(size_t)r * JP + j] = acc;
                            }
                        }
                    }
                }
                cd.kcap = Kcap;
                if ((st = upload_bytes(g, &cd.inv_m_t, real_layout(mt, g->tl)))) return st;
            }
        }
        if ((st = upload_vec(g, &g->d_cheb, cdev))) return st;
    }

    // ---- device arrays
    const size_t es = g->esz;
    if ((st = dev_alloc(g, &g->phys, size_t(d.n_physical) * nv * d.nslots * es))) return st;
    if ((st = dev_alloc(g, &g->spec, size_t(d.n_spectral) * nv * es))) return st;
    if ((st = dev_alloc(g, &g->F, size_t(g->nitems) * g->frows * es))) return st;
    if ((st = dev_alloc(g, &g->G, size_t(3) * g->nitems * g->frows * es))) return st;
    if (g->rlz) {
        if ((st = dev_alloc(g, &g->C, size_t(nv) * bk * jDim * es))) return st;
        if ((st = dev_alloc(g, &g->H, size_t(5) * nv * bk * jDim * es))) return st;
    }
    if (g->tl == TL_F32) {
        // the binary32 SAtransform! streams its vectors through two scratch
        // arrays; F (free during gridTransform!) and phys (overwritten by it)
        // serve when they are large enough
        const size_t need = size_t(g->nitems) * d.b_iDim * g->nslots_z;
        g->sa_x = size_t(g->nitems) * g->frows >= need ? g->F : nullptr;
        g->sa_y = size_t(d.n_physical) * nv * d.nslots >= need ? g->phys : nullptr;
        if (!g->sa_x && (st = dev_alloc(g, &g->sa_x, need * sizeof(float), false))) return st;
        if (!g->sa_y && (st = dev_alloc(g, &g->sa_y, need * sizeof(float), false))) return st;
    }
    {
        std::vector<double> ones_f(size_t(nv) * (K + 1), 1.0), ones_c(size_t(nv) * bk, 1.0);
        if ((st = upload_vec(g, &g->d_fw, ones_f))) return st;
        if ((st = upload_vec(g, &g->d_cw, ones_c))) return st;
    }
    fft_init_constants();
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    return SS_OK;
}

// ---------------------------------------------------------------- launches
// Every stage launches either over the whole grid or over one radial chunk
// (rings [chunk_r0[c], chunk_r0[c+1]), i.e. physical columns
// [ring_jofs[r0], ring_jofs[r1])).  The host-overlapped transforms run the
// ring and Chebyshev stages chunk by chunk and move each chunk's physical
// columns between host and device on copy_stream while the next chunk
// computes; a chunk of every (slot, variable) plane is one strided 2D copy.
template <typename Fn>
static int32_t for_ring_segments(ss_grid *g, int chunk, Fn fn) {
    for (size_t b = 0; b < g->buckets.size(); b++) {
        const RingBucket &bkt = g->buckets[b];
        int32_t st = SS_OK;
        if (chunk < 0) st = fn(g->d_ring_list + bkt.offset, bkt.count, bkt);
        else if (g->chunk_seg[chunk][b].second > 0)
            st = fn(g->d_ring_list_chunks + g->chunk_seg[chunk][b].first, g->chunk_seg[chunk][b].second, bkt);
        if (st) return st;
    }
    return SS_OK;
}
static int64_t chunk_col(const ss_grid *g, int chunk, int end) {
    return chunk < 0 ? (end ? g->d.jDim : 0) : g->ring_jofs[g->chunk_r0[chunk + end]];
}

template <typename P, typename T>
static int32_t fwd_columns(ss_grid *g, cudaStream_t st, int chunk) {
    const ss_dims &d = g->d;
    ChebLaunch Cl{};
    Cl.in = g->phys; Cl.out = g->C; Cl.cheb = g->d_cheb; Cl.rings = g->d_rings; Cl.col_ring = g->d_col_ring;
    Cl.jDim = d.jDim; Cl.np = d.n_physical; Cl.iDim = (int)d.iDim; Cl.bk = (int)d.b_kDim; Cl.nvars = (int)d.nvars;
    Cl.col0 = chunk_col(g, chunk, 0); Cl.col1 = chunk_col(g, chunk, 1);
    const int N = (int)d.kDim, half = (N + 1) / 2;
    size_t smem = (size_t(64) * (N | 1) + size_t(Cl.bk) * half) * sizeof(T);
    StageScope sc(g, SS_STAGE_CHEB_FWD, st);
    CUDA_TRY((launch_cheb_forward<P, T>(Cl, smem, st, N)));
    g->launches[SS_STAGE_CHEB_FWD]++;
    return SS_OK;
}

namespace ss {
// Launch records of the per-grid stages (also the records of fused batch launches)
RingLaunch ring_record(const ss_grid *g, bool inverse) {
    const ss_dims &d = g->d;
    RingLaunch L{};
    L.rings = g->d_rings;
    L.ring_var_stride = g->rlz ? 0 : d.iDim;
    L.plans = g->d_plans; L.pool = g->d_pool; L.phase = g->d_phase;
    if (inverse) {
        L.in = g->G;
        L.out = g->rlz ? g->H : g->phys;
    } else {
        L.in = g->rlz ? g->C : g->phys;
        L.out = g->F;
        L.in_item_stride = d.n_physical;
    }
    L.frows = g->frows; L.jDim = d.jDim; L.np = d.n_physical;
    L.nitems = g->nitems; L.nvars = (int)d.nvars; L.bk = (int)d.b_kDim; L.rlz = g->rlz;
    return L;
}
size_t ring_item_smem(const ss_grid *g, const RingBucket &bkt, bool inverse) {
    // the bucket sizes count 16 bytes per complex entry (binary64 and double-float)
    const size_t f64 = inverse ? bkt.smem_inv_f64 : bkt.smem_fwd_f64;
    return g->tl == TL_F32 ? f64 / 2 : f64;
}
SbLaunch sb_record(const ss_grid *g) {
    const ss_dims &d = g->d;
    SbLaunch S{};
    S.F = g->F; S.spec = g->spec; S.spl = g->d_spl; S.fofs = g->d_fofs;
    S.fw = g->filtered ? g->d_fw : nullptr;
    S.cw = g->filtered ? g->d_cw : nullptr;
    S.frows = g->frows; S.nspec = d.n_spectral;
    S.iDim = (int)d.iDim; S.b = (int)d.b_iDim; S.mubar = g->p.mubar; S.pOL = g->pOL; S.K = (int)d.kDim_wn;
    S.nslots_z = g->nslots_z; S.bk = (int)d.b_kDim; S.filtered = g->filtered;
    return S;
}
SaLaunch sa_record(const ss_grid *g, int coeffs, size_t *smem_generic) {
    const ss_dims &d = g->d;
    SaLaunch A{};
    A.spec = g->spec; A.G = g->G; A.spl = g->d_spl; A.fofs = g->d_fofs; A.ahat = g->d_ahat;
    A.frows = g->frows; A.nspec = d.n_spectral; A.nblocks = d.n_blocks;
    A.iDim = (int)d.iDim; A.b = (int)d.b_iDim; A.ld = (A.b % 2) ? A.b : A.b + 1;
    A.pOL = g->pOL; A.nslots_z = g->nslots_z; A.bk = (int)d.b_kDim; A.nitems = g->nitems; A.coeffs = coeffs;
    A.sx = (float *)g->sa_x; A.sy = (float *)g->sa_y;
    int nmax = 0;
    for (auto &sh : g->spl_host) nmax = std::max(nmax, sh.Min);
    const size_t ssz = (g->tl == TL_F32) ? 4 : 8;  // solve type: float (FP32 mode) or double
    size_t smem = (size_t(32) * A.ld + size_t(5) * nmax) * ssz;
    if (g->tl != TL_F64) smem += size_t(32) * A.ld * ssz;  // FP32 residuals / df64 coefficients
    if (smem_generic) *smem_generic = smem;
    return A;
}
}  // namespace ss

template <typename P, typename T>
static int32_t fwd_rings(ss_grid *g, cudaStream_t st, int chunk) {
    RingLaunch L = ring_record(g, false);
    StageScope sc(g, SS_STAGE_RING_FWD, st);
    return for_ring_segments(g, chunk, [&](const int *list, int count, const RingBucket &bkt) -> int32_t {
        L.ring_list = list;
        const size_t smem = ring_item_smem(g, bkt, false);
        L.ib = ring_batch(smem, g->nitems, count, 4 * g->sms, g->ring_threads_fwd, bkt.max_buf);
        CUDA_TRY((launch_ring_forward<P, T>(L, count, g->nitems, smem, g->ring_threads_fwd, st)));
        g->launches[SS_STAGE_RING_FWD]++;
        return SS_OK;
    });
}

template <typename P, typename T>
static int32_t fwd_sb(ss_grid *g, cudaStream_t st) {
    const SbLaunch S = sb_record(g);
    StageScope sc(g, SS_STAGE_SB, st);
    CUDA_TRY((launch_sb_project<P, T>(S, g->nitems, st)));
    g->launches[SS_STAGE_SB]++;
    return SS_OK;
}

// `aout` set: splineTransform! — SAtransform(spline, b) of every block of `spec_in`
// (the 2-argument form: no R3X background) written as coefficients to `aout`
template <typename P, typename T>
static int32_t inv_sa(ss_grid *g, cudaStream_t st, int coeffs, const void *spec_in = nullptr, void *aout = nullptr) {
    size_t smem = 0;
    SaLaunch A = sa_record(g, coeffs, &smem);
    if (spec_in) A.spec = spec_in;
    if (aout) {
        A.ahat = nullptr;
        A.aout = aout;
    }
    StageScope sc(g, SS_STAGE_SA_SI, st);
    bool periodic = false;
    for (auto &sh : g->spl_host) periodic |= sh.periodic != 0;
    if constexpr (std::is_same<P, float>::value && std::is_same<T, float>::value) {
        // the slot-parallel binary32 kernel has no dense-tail solve: periodic splines
        // (and the coefficient output of splineTransform!) take the tiled kernel
        if (aout || periodic) CUDA_TRY((launch_sa_si<P, T>(A, g->nitems, smem, st)));
        else CUDA_TRY((launch_sa_si_f32<P>(A, g->nitems, (float *)g->sa_x, (float *)g->sa_y, st)));
    } else {
        CUDA_TRY((launch_sa_si<P, T>(A, g->nitems, smem, st)));
    }
    g->launches[SS_STAGE_SA_SI]++;
    return SS_OK;
}

template <typename P, typename T>
static int32_t inv_rings(ss_grid *g, cudaStream_t st, int chunk) {
    RingLaunch L = ring_record(g, true);
    StageScope sc(g, SS_STAGE_RING_INV, st);
    return for_ring_segments(g, chunk, [&](const int *list, int count, const RingBucket &bkt) -> int32_t {
        L.ring_list = list;
        const size_t sm = ring_item_smem(g, bkt, true);
        L.ib = ring_batch(sm, g->nitems, count, 4 * g->sms, g->ring_threads_inv, bkt.max_buf);
        CUDA_TRY((launch_ring_inverse<P, T>(L, count, g->nitems, sm, g->ring_threads_inv, st)));
        g->launches[SS_STAGE_RING_INV]++;
        return SS_OK;
    });
}

template <typename P, typename T>
static int32_t inv_columns(ss_grid *g, cudaStream_t st, int chunk) {
    const ss_dims &d = g->d;
    ChebLaunch Cl{};
    Cl.in = g->H; Cl.out = g->phys; Cl.cheb = g->d_cheb; Cl.rings = g->d_rings; Cl.col_ring = g->d_col_ring;
    Cl.jDim = d.jDim; Cl.np = d.n_physical; Cl.iDim = (int)d.iDim; Cl.bk = (int)d.b_kDim; Cl.nvars = (int)d.nvars;
    Cl.col0 = chunk_col(g, chunk, 0); Cl.col1 = chunk_col(g, chunk, 1);
    const int N = (int)d.kDim;
    StageScope sc(g, SS_STAGE_CHEB_INV, st);
    CUDA_TRY((launch_cheb_inverse<P, T>(Cl, 0, st, N)));
    g->launches[SS_STAGE_CHEB_INV]++;
    return SS_OK;
}

static int32_t ensure_copy_stream(ss_grid *g) {
    if (!g->copy_stream) CUDA_TRY(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    while (g->chunk_ev.size() < g->chunk_r0.size()) {  // one per chunk, one to join the streams
        cudaEvent_t e = nullptr;
        CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        g->chunk_ev.push_back(e);
    }
    return SS_OK;
}
// physical columns of one chunk in `rows` (slot, variable) planes from the
// first: one linear copy per plane (measured faster than one pitched copy
// while long kernels occupy the SMs)
static cudaError_t copy_chunk(ss_grid *g, int chunk, void *host, bool to_host, int rows, cudaStream_t s) {
    const size_t es = g->esz, kz = (size_t)g->d.kDim, pitch = size_t(g->d.n_physical) * es;
    const size_t off = size_t(chunk_col(g, chunk, 0)) * kz * es;
    const size_t width = size_t(chunk_col(g, chunk, 1) - chunk_col(g, chunk, 0)) * kz * es;
    if (width == 0) return cudaSuccess;
    for (int row = 0; row < rows; row++) {
        char *dev = (char *)g->phys + off + row * pitch, *h = (char *)host + off + row * pitch;
        const cudaError_t e = to_host ? cudaMemcpyAsync(h, dev, width, cudaMemcpyDeviceToHost, s)
                                      : cudaMemcpyAsync(dev, h, width, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename P, typename T>
static int32_t run_forward(ss_grid *g, cudaStream_t st, const void *host_slot1 = nullptr) {
    int32_t rc;
    if (!host_slot1) {
        if (g->rlz && (rc = fwd_columns<P, T>(g, st, -1))) return rc;
        if ((rc = fwd_rings<P, T>(g, st, -1))) return rc;
        return fwd_sb<P, T>(g, st);
    }
    if ((rc = ensure_copy_stream(g))) return rc;
    const int nch = (int)g->chunk_r0.size() - 1;
    // the copies start after the work already queued on the stream (it may read phys)
    CUDA_TRY(cudaEventRecord(g->chunk_ev[nch], st));
    CUDA_TRY(cudaStreamWaitEvent(g->copy_stream, g->chunk_ev[nch], 0));
    for (int c = 0; c < nch; c++) {
        CUDA_TRY(copy_chunk(g, c, (void *)host_slot1, false, (int)g->d.nvars, g->copy_stream));
        CUDA_TRY(cudaEventRecord(g->chunk_ev[c], g->copy_stream));
        CUDA_TRY(cudaStreamWaitEvent(st, g->chunk_ev[c], 0));
        if (g->rlz && (rc = fwd_columns<P, T>(g, st, c))) return rc;
        if ((rc = fwd_rings<P, T>(g, st, c))) return rc;
    }
    return fwd_sb<P, T>(g, st);
}

template <typename P, typename T>
static int32_t run_inverse(ss_grid *g, cudaStream_t st, int coeffs = 0, void *host_all = nullptr) {
    int32_t rc;
    if ((rc = inv_sa<P, T>(g, st, coeffs))) return rc;
    if (!host_all) {
        if ((rc = inv_rings<P, T>(g, st, -1))) return rc;
        return g->rlz ? inv_columns<P, T>(g, st, -1) : SS_OK;
    }
    if ((rc = ensure_copy_stream(g))) return rc;
    const int nch = (int)g->chunk_r0.size() - 1;
    // every chunk's compute is queued before its copies, so that a pageable
    // host buffer (whose copies return to the caller only when done) still
    // overlaps the remaining chunks
    for (int c = 0; c < nch; c++) {
        if ((rc = inv_rings<P, T>(g, st, c))) return rc;
        if (g->rlz && (rc = inv_columns<P, T>(g, st, c))) return rc;
        CUDA_TRY(cudaEventRecord(g->chunk_ev[c], st));
    }
    const int rows = (int)(g->d.nslots * g->d.nvars);
    for (int c = 0; c < nch; c++) {
        CUDA_TRY(cudaStreamWaitEvent(g->copy_stream, g->chunk_ev[c], 0));
        CUDA_TRY(copy_chunk(g, c, host_all, true, rows, g->copy_stream));
    }
    // later work on the stream (which may overwrite phys) waits for the copies
    CUDA_TRY(cudaEventRecord(g->chunk_ev[nch], g->copy_stream));
    CUDA_TRY(cudaStreamWaitEvent(st, g->chunk_ev[nch], 0));
    return SS_OK;
}

namespace ss {
int32_t grid_forward(ss_grid *g, cudaStream_t s) {
    if (g->tl == TL_DF64) return run_forward<double, df64>(g, s);
    if (g->tl == TL_F64) return run_forward<double, double>(g, s);
    return run_forward<float, float>(g, s);
}
int32_t grid_inverse(ss_grid *g, cudaStream_t s) {
    if (g->tl == TL_DF64) return run_inverse<double, df64>(g, s);
    if (g->tl == TL_F64) return run_inverse<double, double>(g, s);
    return run_inverse<float, float>(g, s);
}
int32_t grid_inverse_coeffs(ss_grid *g, cudaStream_t s) {
    if (g->tl == TL_DF64) return run_inverse<double, df64>(g, s, 1);
    if (g->tl == TL_F64) return run_inverse<double, double>(g, s, 1);
    return run_inverse<float, float>(g, s, 1);
}
static int32_t grid_spline_coeffs(ss_grid *g, cudaStream_t s, const void *shared) {
    const void *in = shared ? shared : g->spec;
    if (g->tl == TL_DF64) return inv_sa<double, df64>(g, s, 0, in, g->spec);
    if (g->tl == TL_F64) return inv_sa<double, double>(g, s, 0, in, g->spec);
    return inv_sa<float, float>(g, s, 0, in, g->spec);
}
static int32_t grid_forward_host(ss_grid *g, cudaStream_t s, const void *host_slot1) {
    if (g->tl == TL_DF64) return run_forward<double, df64>(g, s, host_slot1);
    if (g->tl == TL_F64) return run_forward<double, double>(g, s, host_slot1);
    return run_forward<float, float>(g, s, host_slot1);
}
static int32_t grid_inverse_host(ss_grid *g, cudaStream_t s, void *host_all) {
    if (g->tl == TL_DF64) return run_inverse<double, df64>(g, s, 0, host_all);
    if (g->tl == TL_F64) return run_inverse<double, double>(g, s, 0, host_all);
    return run_inverse<float, float>(g, s, 0, host_all);
}
}  // namespace ss

// ---------------------------------------------------------------- helpers
__global__ void convert_kernel_f64_to_f32(const double *in, float *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}
__global__ void convert_kernel_f32_to_f64(const float *in, double *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

static cudaStream_t pick(ss_grid *g, void *s) { return s ? (cudaStream_t)s : g->stream; }

static int32_t ensure_stage(ss_grid *g, size_t bytes) {
    if (g->stage_bytes >= bytes) return SS_OK;
    if (g->stage) {
        cudaStreamSynchronize(g->stream);
        cudaFree(g->stage);
        g->allocs.erase(std::remove(g->allocs.begin(), g->allocs.end(), g->stage), g->allocs.end());
        g->stage = nullptr;
        g->stage_bytes = 0;
    }
    int32_t st = dev_alloc(g, &g->stage, bytes, false);
    if (st) return st;
    g->stage_bytes = bytes;
    return SS_OK;
}

static int32_t copy_in(ss_grid *g, void *dst, const void *host, int32_t dtype, size_t n, cudaStream_t s) {
    const size_t hes = dtype == SS_DTYPE_F64 ? 8 : 4;
    if (hes == g->esz) {
        CUDA_TRY(cudaMemcpyAsync(dst, host, n * hes, cudaMemcpyHostToDevice, s));
    } else {
        int32_t st = ensure_stage(g, n * hes);
        if (st) return st;
        CUDA_TRY(cudaMemcpyAsync(g->stage, host, n * hes, cudaMemcpyHostToDevice, s));
        if (hes == 8) convert_kernel_f64_to_f32<<<1216, 256, 0, s>>>((const double *)g->stage, (float *)dst, n);
        else convert_kernel_f32_to_f64<<<1216, 256, 0, s>>>((const float *)g->stage, (double *)dst, n);
        CUDA_TRY(cudaGetLastError());
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    return SS_OK;
}

static int32_t copy_out(ss_grid *g, void *host, const void *src, int32_t dtype, size_t n, cudaStream_t s) {
    const size_t hes = dtype == SS_DTYPE_F64 ? 8 : 4;
    if (hes == g->esz) {
        CUDA_TRY(cudaMemcpyAsync(host, src, n * hes, cudaMemcpyDeviceToHost, s));
    } else {
        int32_t st = ensure_stage(g, n * hes);
        if (st) return st;
        if (hes == 8) convert_kernel_f32_to_f64<<<1216, 256, 0, s>>>((const float *)src, (double *)g->stage, n);
        else convert_kernel_f64_to_f32<<<1216, 256, 0, s>>>((const double *)src, (float *)g->stage, n);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(host, g->stage, n * hes, cudaMemcpyDeviceToHost, s));
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    return SS_OK;
}

#define CHECK_GRID(g)                                         \
    do {                                                      \
        if (!(g)) { set_error("null grid"); return SS_BAD_ARG; } \
        cudaSetDevice((g)->device);                           \
    } while (0)

// ================================================================ C ABI
extern "C" {

int32_t ss_version(void) { return SS_ABI_VERSION; }

const char *ss_last_error_string(void) { return g_err.c_str(); }

int32_t ss_grid_create(const ss_grid_params *params, ss_grid **out) {
    if (!out) { set_error("null output pointer"); return SS_BAD_ARG; }
    *out = nullptr;
    if (!params) { set_error("null params"); return SS_BAD_ARG; }
    const ss_grid_params &p = *params;
    if (p.geometry != SS_GEOM_RL && p.geometry != SS_GEOM_RLZ) { set_error("geometry must be RL or RLZ"); return SS_BAD_ARG; }
    if (p.precision != SS_PREC_F64 && p.precision != SS_PREC_F32_REFINED && p.precision != SS_PREC_F64_FAST) {
        set_error("unknown precision");
        return SS_BAD_ARG;
    }
    if (p.nvars < 1 || p.num_cells < 1 || p.mubar < 1 || p.patchOffsetL < 0) { set_error("bad sizes"); return SS_BAD_SHAPE; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device visible");
        return SS_NO_DEVICE;
    }
    ss_grid *g = new ss_grid();
    g->p = p;
    const int nv = p.nvars;
    g->l_q.assign(nv, 2.0);
    g->bcl.assign(nv, ss_spline_bc{SS_SBC_R0, 0, 0.0, 0.0});
    g->bcr.assign(nv, ss_spline_bc{SS_SBC_R0, 0, 0.0, 0.0});
    g->bcb.assign(nv, SS_CBC_R0);
    g->bct.assign(nv, SS_CBC_R0);
    g->kmaxv.assign(nv, -1);
    for (int v = 0; v < nv; v++) {
        if (p.l_q) g->l_q[v] = p.l_q[v];
        if (p.BCL) g->bcl[v] = p.BCL[v];
        if (p.BCR) g->bcr[v] = p.BCR[v];
        if (p.BCB) g->bcb[v] = p.BCB[v];
        if (p.BCT) g->bct[v] = p.BCT[v];
        if (p.max_wavenumber) g->kmaxv[v] = p.max_wavenumber[v];
    }
    // RLZ rings shared by all variables: the reference's var_kmax (src/factory.jl:730-733)
    g->ring_kmax = p.ring_kmax_set ? p.ring_kmax : (nv > 0 ? g->kmaxv[nv - 1] : -1);
    g->p.l_q = nullptr; g->p.BCL = g->p.BCR = nullptr; g->p.BCB = g->p.BCT = nullptr; g->p.max_wavenumber = nullptr;
    cudaGetDevice(&g->device);
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        delete g;
        return SS_CUDA_ERROR;
    }
    int32_t st = build_grid(g);
    if (st) { free_grid(g); return st; }
    *out = g;
    return SS_OK;
}

int32_t ss_grid_destroy(ss_grid *g) {
    if (!g) return SS_OK;
    cudaSetDevice(g->device);
    free_grid(g);
    return SS_OK;
}

int32_t ss_grid_dims(const ss_grid *g, ss_dims *out) {
    if (!g || !out) { set_error("null argument"); return SS_BAD_ARG; }
    *out = g->d;
    return SS_OK;
}

int32_t ss_grid_stream(const ss_grid *g, void **s) {
    if (!g || !s) { set_error("null argument"); return SS_BAD_ARG; }
    *s = (void *)g->stream;
    return SS_OK;
}

int32_t ss_grid_device_physical(ss_grid *g, void **p) {
    if (!g || !p) { set_error("null argument"); return SS_BAD_ARG; }
    *p = g->phys;
    return SS_OK;
}
int32_t ss_grid_device_spectral(ss_grid *g, void **p) {
    if (!g || !p) { set_error("null argument"); return SS_BAD_ARG; }
    *p = g->spec;
    return SS_OK;
}

int32_t ss_upload_physical(ss_grid *g, const void *host, int32_t dtype, int32_t slot, void *stream) {
    CHECK_GRID(g);
    if (!host || (dtype != SS_DTYPE_F64 && dtype != SS_DTYPE_F32)) { set_error("bad host buffer or dtype"); return SS_BAD_ARG; }
    if (slot < 0 || slot > g->d.nslots) { set_error("slot out of range"); return SS_BAD_ARG; }
    const size_t per = size_t(g->d.n_physical) * g->d.nvars;
    char *dst = (char *)g->phys + (slot ? size_t(slot - 1) * per * g->esz : 0);
    return copy_in(g, dst, host, dtype, slot ? per : per * g->d.nslots, pick(g, stream));
}

int32_t ss_download_physical(ss_grid *g, void *host, int32_t dtype, int32_t slot, void *stream) {
    CHECK_GRID(g);
    if (!host || (dtype != SS_DTYPE_F64 && dtype != SS_DTYPE_F32)) { set_error("bad host buffer or dtype"); return SS_BAD_ARG; }
    if (slot < 0 || slot > g->d.nslots) { set_error("slot out of range"); return SS_BAD_ARG; }
    const size_t per = size_t(g->d.n_physical) * g->d.nvars;
    const char *src = (const char *)g->phys + (slot ? size_t(slot - 1) * per * g->esz : 0);
    return copy_out(g, host, src, dtype, slot ? per : per * g->d.nslots, pick(g, stream));
}

int32_t ss_upload_spectral(ss_grid *g, const void *host, int32_t dtype, void *stream) {
    CHECK_GRID(g);
    if (!host || (dtype != SS_DTYPE_F64 && dtype != SS_DTYPE_F32)) { set_error("bad host buffer or dtype"); return SS_BAD_ARG; }
    return copy_in(g, g->spec, host, dtype, size_t(g->d.n_spectral) * g->d.nvars, pick(g, stream));
}

int32_t ss_download_spectral(ss_grid *g, void *host, int32_t dtype, void *stream) {
    CHECK_GRID(g);
    if (!host || (dtype != SS_DTYPE_F64 && dtype != SS_DTYPE_F32)) { set_error("bad host buffer or dtype"); return SS_BAD_ARG; }
    return copy_out(g, host, g->spec, dtype, size_t(g->d.n_spectral) * g->d.nvars, pick(g, stream));
}

int32_t ss_spectral_transform(ss_grid *g, void *stream) {
    CHECK_GRID(g);
    return grid_forward(g, pick(g, stream));
}

int32_t ss_grid_transform(ss_grid *g, void *stream) {
    CHECK_GRID(g);
    return grid_inverse(g, pick(g, stream));
}

int32_t ss_spline_transform(ss_grid *g, const void *d_shared_spectral, void *stream) {
    CHECK_GRID(g);
    return grid_spline_coeffs(g, pick(g, stream), d_shared_spectral);
}

int32_t ss_tile_transform(ss_grid *g, void *stream) {
    CHECK_GRID(g);
    return grid_inverse_coeffs(g, pick(g, stream));
}

int32_t ss_spectral_transform_from_host(ss_grid *g, const void *host_slot1, int32_t dtype, void *stream) {
    CHECK_GRID(g);
    if (!host_slot1 || (dtype != SS_DTYPE_F64 && dtype != SS_DTYPE_F32)) { set_error("bad host buffer or dtype"); return SS_BAD_ARG; }
    cudaStream_t s = pick(g, stream);
    if ((dtype == SS_DTYPE_F64 ? 8u : 4u) != g->esz) {  // converting copy: upload, then transform
        int32_t rc = ss_upload_physical(g, host_slot1, dtype, 1, stream);
        return rc ? rc : grid_forward(g, s);
    }
    int32_t rc = grid_forward_host(g, s, host_slot1);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(g->copy_stream));  // the host buffer is free again
    return SS_OK;
}

int32_t ss_grid_transform_to_host(ss_grid *g, void *host_all, int32_t dtype, void *stream) {
    CHECK_GRID(g);
    if (!host_all || (dtype != SS_DTYPE_F64 && dtype != SS_DTYPE_F32)) { set_error("bad host buffer or dtype"); return SS_BAD_ARG; }
    cudaStream_t s = pick(g, stream);
    if ((dtype == SS_DTYPE_F64 ? 8u : 4u) != g->esz) {  // converting copy: transform, then download
        int32_t rc = grid_inverse(g, s);
        return rc ? rc : ss_download_physical(g, host_all, dtype, 0, stream);
    }
    int32_t rc = grid_inverse_host(g, s, host_all);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(g->copy_stream));
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

int32_t ss_grid_set_filter(ss_grid *g, int32_t var, const double *fw, const double *cw) {
    CHECK_GRID(g);
    if (var < 0 || var >= g->d.nvars) { set_error("var out of range"); return SS_BAD_ARG; }
    const int K = (int)g->d.kDim_wn, bk = (int)g->d.b_kDim;
    std::vector<double> f(K + 1, 1.0), c(bk, 1.0);
    if (fw) std::copy(fw, fw + K + 1, f.begin());
    if (cw) std::copy(cw, cw + bk, c.begin());
    CUDA_TRY(cudaMemcpyAsync(g->d_fw + size_t(var) * (K + 1), f.data(), f.size() * 8, cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaMemcpyAsync(g->d_cw + size_t(var) * bk, c.data(), c.size() * 8, cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    if (fw || cw) g->filtered = 1;
    g->generation++;
    return SS_OK;
}

int32_t ss_grid_set_ahat(ss_grid *g, int32_t var, int32_t block, const double *ahat) {
    CHECK_GRID(g);
    if (var < 0 || var >= g->d.nvars || block < 0 || block >= g->d.n_blocks || !ahat) {
        set_error("ahat index out of range");
        return SS_BAD_ARG;
    }
    const size_t b = g->d.b_iDim;
    if (!g->d_ahat) {
        int32_t st = dev_alloc(g, (void **)&g->d_ahat, size_t(g->d.nvars) * g->d.n_blocks * b * 8);
        if (st) return st;
        g->generation++;
    }
    CUDA_TRY(cudaMemcpyAsync(g->d_ahat + (size_t(var) * g->d.n_blocks + block) * b, ahat, b * 8, cudaMemcpyHostToDevice,
                             g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    return SS_OK;
}

int32_t ss_grid_clear_ahat(ss_grid *g) {
    CHECK_GRID(g);
    if (g->d_ahat) {
        CUDA_TRY(cudaStreamSynchronize(g->stream));
        cudaFree(g->d_ahat);
        g->allocs.erase(std::remove(g->allocs.begin(), g->allocs.end(), (void *)g->d_ahat), g->allocs.end());
        g->d_ahat = nullptr;
        g->generation++;
    }
    return SS_OK;
}

int32_t ss_grid_profile(ss_grid *g, int32_t enable) {
    CHECK_GRID(g);
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    g->profiling = enable ? 1 : 0;
    g->marks.clear();
    g->ev_used = 0;
    for (int i = 0; i < SS_NSTAGES; i++) { g->launches[i] = 0; g->stage_ms[i] = 0.0; }
    return SS_OK;
}

int32_t ss_grid_profile_read(ss_grid *g, double *ms, int64_t *launches) {
    CHECK_GRID(g);
    for (auto &m : g->marks) {
        CUDA_TRY(cudaEventSynchronize(m.b));
        float t = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&t, m.a, m.b));
        g->stage_ms[m.stage] += t;
    }
    g->marks.clear();
    g->ev_used = 0;
    for (int i = 0; i < SS_NSTAGES; i++) {
        if (ms) ms[i] = g->stage_ms[i];
        if (launches) launches[i] = g->launches[i];
    }
    return SS_OK;
}

int32_t ss_grid_synchronize(ss_grid *g) {
    CHECK_GRID(g);
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

}  // extern "C"

// ====================================================================
// Forward RL transform without any allocation
// --------------------------------------------------------------------
// Some callers cannot call cudaMalloc at the point where they transform:
// code recorded into a CUDA stream capture (allocation is not allowed while a
// capture is open), host frameworks whose device memory is owned by their own
// pool allocator (e.g. a Julia CUDA.jl array pool or a serving process with
// a fixed memory budget), and real-time loops that must not touch the driver
// allocator.  They pass their own device input and output arrays; the ring
// coefficient scratch that ring_forward writes and sb_project reads lives in
// the fixed array below instead of the grid's scratch buffer.
//
// Limit: kStaticScratchDoubles = 1,048,576 FP64 values (8 MiB), i.e.
// nvars × Σ_r (1 + 2 ri) ≤ 1,048,576 (the 100-cell one-variable RL grid needs 90,600).  Every GPU that
// loads the library keeps this 8 MiB reserved until the process exits.
// Every call shares the array and it keeps the last call's contents; the
// kernels write every entry they later read within one call, so nothing has
// to start at zero.  Calls whose work overlaps on the GPU (different streams
// without ordering, or several host threads) race on the array.
// ====================================================================
static constexpr size_t kStaticScratchDoubles = size_t(1) << 20;
static __device__ __align__(256) double g_static_ring_scratch[kStaticScratchDoubles];

// device address of g_static_ring_scratch, looked up once per device
static constexpr int kMaxDevices = 64;
static double *g_static_scratch_ptr[kMaxDevices] = {nullptr};

extern "C" int32_t ss_spectral_transform_noalloc(const ss_grid *g, const double *d_physical_slot1,
                                                 double *d_spectral, void *stream) {
    if (!g || !d_physical_slot1 || !d_spectral) { set_error("null argument"); return SS_BAD_ARG; }
    // the ring kernel reads each ring's points in aligned (2n, 2n+1) pairs
    if ((uintptr_t)d_physical_slot1 % 16) { set_error("d_physical_slot1 must be 16-byte aligned"); return SS_BAD_ARG; }
    if (g->rlz || g->esz != 8) {
        set_error("ss_spectral_transform_noalloc supports RL grids with SS_PREC_F64 only");
        return SS_BAD_ARG;
    }
    const size_t need = size_t(g->nitems) * size_t(g->frows);
    if (need > kStaticScratchDoubles) {
        set_error("ss_spectral_transform_noalloc: grid needs %zu scratch values (nvars x sum(1+2ri)), "
                  "the static scratch holds %zu", need, kStaticScratchDoubles);
        return SS_BAD_SHAPE;
    }
    if (g->device < 0 || g->device >= kMaxDevices) { set_error("device index out of range"); return SS_BAD_ARG; }
    CUDA_TRY(cudaSetDevice(g->device));
    // first call on this device: resolve the array's device address (host code
    // only sees a host-side stand-in for the symbol).  Do this first call
    // before any stream capture.
    if (!g_static_scratch_ptr[g->device]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_static_ring_scratch);
        if (e != cudaSuccess || !p) {
            set_error("cudaGetSymbolAddress(g_static_ring_scratch) failed: %s", cudaGetErrorString(e));
            return SS_CUDA_ERROR;
        }
        g_static_scratch_ptr[g->device] = p;
    }
    double *scratch = g_static_scratch_ptr[g->device];
    cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    const ss_dims &d = g->d;
    RingLaunch L{};
    L.rings = g->d_rings;
    L.ring_var_stride = d.iDim;
    L.plans = g->d_plans; L.pool = g->d_pool; L.phase = g->d_phase;
    L.in = d_physical_slot1;
    L.out = scratch;
    L.in_item_stride = d.n_physical;
    L.frows = g->frows; L.jDim = d.jDim; L.np = d.n_physical;
    L.nitems = g->nitems; L.nvars = (int)d.nvars; L.bk = 1; L.rlz = 0;
    for (const RingBucket &bkt : g->buckets) {
        L.ring_list = g->d_ring_list + bkt.offset;
        if (g->tl == TL_DF64) CUDA_TRY((launch_ring_forward<double, df64>(L, bkt.count, g->nitems, bkt.smem_fwd_f64, g->ring_threads_fwd, st)));
        else CUDA_TRY((launch_ring_forward<double, double>(L, bkt.count, g->nitems, bkt.smem_fwd_f64, g->ring_threads_fwd, st)));
    }
    SbLaunch S{};
    S.F = scratch; S.spec = d_spectral; S.spl = g->d_spl; S.fofs = g->d_fofs;
    S.fw = g->filtered ? g->d_fw : nullptr;
    S.cw = g->filtered ? g->d_cw : nullptr;
    S.frows = g->frows; S.nspec = d.n_spectral;
    S.iDim = (int)d.iDim; S.b = (int)d.b_iDim; S.mubar = g->p.mubar; S.pOL = g->pOL; S.K = (int)d.kDim_wn;
    S.nslots_z = g->nslots_z; S.bk = 1; S.filtered = g->filtered;
    if (g->tl == TL_DF64) CUDA_TRY((launch_sb_project<double, df64>(S, g->nitems, st)));
    else CUDA_TRY((launch_sb_project<double, double>(S, g->nitems, st)));
    return SS_OK;
}

// The FFT plan grid creation builds for a length-n ring DFT (host only).
extern "C" int32_t ss_fft_plan(int32_t n, int32_t precision, ss_fft_plan_info *out) {
    if (!out || n < 1 || n > (1 << 22)) { set_error("ss_fft_plan: null output or n out of range"); return SS_BAD_ARG; }
    if (precision != SS_PREC_F64 && precision != SS_PREC_F64_FAST && precision != SS_PREC_F32_REFINED) {
        set_error("ss_fft_plan: unknown precision %d", precision);
        return SS_BAD_ARG;
    }
    const int tl = precision == SS_PREC_F32_REFINED ? TL_F32 : (precision == SS_PREC_F64_FAST ? TL_DF64 : TL_F64);
    PlanSet plans;
    configure_plans(plans, tl);
    TwiddlePool pool;
    const FftPlan &p = plans.plans[plans.plan_for(n, pool)];
    std::memset(out, 0, sizeof *out);
    out->n = n;
    out->kind = p.blu ? 2 : (p.rp ? 1 : 0);
    out->max_prime = plans.max_prime;
    out->pad_prime = plans.pad_prime;
    if (p.blu) {
        out->bluestein_m = p.M;
        out->nrad = p.mnrad;
        for (int i = 0; i < p.mnrad; i++) out->rad[i] = p.mrad[i];
        return SS_OK;
    }
    out->nrad = p.nrad;
    for (int i = 0; i < p.nrad; i++) out->rad[i] = p.rad[i];
    if (p.rp) {
        out->rader_p = p.rp;
        out->rader_inner = p.rM;
        out->inner_nrad = p.rnrad;
        for (int i = 0; i < p.rnrad; i++) out->inner_rad[i] = p.rrad[i];
    }
    return SS_OK;
}
