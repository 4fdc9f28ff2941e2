// ss_io.cpp — save_grid / load_grid (src/io.jl:410-439) from and to the
// device-resident arrays.
//
// The reference archives three components of a grid in a JLD2 file: params,
// spectral and physical, with a format-version tag; load_grid rebuilds the grid
// with createGrid(params) and copies the two arrays back.  This image has no
// HDF5/JLD2 library, so the same three components go into a flat little-endian
// archive (layout in include/springsteel_gpu.h, "grid archives"): a fixed
// parameter record (the ss_grid_params fields, every variable's BCs, l_q and
// max_wavenumber, the spectral filter weights), an optional caller block (the
// host mirror stores its variable names there), then grid.spectral and
// grid.physical in the reference's column-major layout and the grid's storage
// type.  The arrays stream between HBM and the file through two page-locked
// staging buffers: the device→host copy of one chunk overlaps the file write of
// the previous one (and, loading, the read of the next chunk overlaps the
// host→device copy of the current one).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ss_grid.h"

namespace {

constexpr char kMagic[8] = {'S', 'S', 'G', 'R', 'I', 'D', '0', '1'};
constexpr size_t kChunk = size_t(32) << 20;  // bytes per staging buffer

struct FileCloser {
    FILE *f;
    ~FileCloser() {
        if (f) fclose(f);
    }
};

template <typename T>
void put(std::vector<unsigned char> &b, T v) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(&v);
    b.insert(b.end(), p, p + sizeof(T));
}
template <typename T>
bool get(const std::vector<unsigned char> &b, size_t &o, T &v) {
    if (o + sizeof(T) > b.size()) return false;
    std::memcpy(&v, b.data() + o, sizeof(T));
    o += sizeof(T);
    return true;
}

// the parameter record: everything createGrid needs, plus the filter weights
std::vector<unsigned char> param_record(const ss_grid *g, const std::vector<double> &fw,
                                        const std::vector<double> &cw) {
    std::vector<unsigned char> b;
    const ss_grid_params &p = g->p;
    const int32_t dtype = g->esz == 8 ? SS_DTYPE_F64 : SS_DTYPE_F32;
    for (int32_t v : {p.geometry, p.precision, p.num_cells, p.mubar, p.quadrature, p.nvars, p.kDim, p.b_kDim,
                      p.patchOffsetL, p.ring_kmax_set, g->ring_kmax, dtype, g->filtered})
        put<int32_t>(b, v);
    for (double v : {p.iMin, p.iMax, p.kMin, p.kMax}) put<double>(b, v);
    for (int v = 0; v < p.nvars; v++) {
        put<double>(b, g->l_q[v]);
        for (const ss_spline_bc &bc : {g->bcl[v], g->bcr[v]}) {
            put<int32_t>(b, bc.kind);
            put<int32_t>(b, 0);
            put<double>(b, bc.alpha);
            put<double>(b, bc.beta);
        }
        put<int32_t>(b, g->bcb[v]);
        put<int32_t>(b, g->bct[v]);
        put<int32_t>(b, g->kmaxv[v]);
        put<int32_t>(b, 0);
    }
    for (int64_t v : {g->d.n_spectral, g->d.n_physical, g->d.nslots, g->d.nvars, (int64_t)fw.size(), (int64_t)cw.size()})
        put<int64_t>(b, v);
    for (double v : fw) put<double>(b, v);
    for (double v : cw) put<double>(b, v);
    return b;
}

struct Record {
    ss_grid_params p{};
    std::vector<double> l_q;
    std::vector<ss_spline_bc> bcl, bcr;
    std::vector<int32_t> bcb, bct, kmax;
    int32_t ring_kmax = -1, dtype = 0, filtered = 0;
    int64_t n_spectral = 0, n_physical = 0, nslots = 0, nvars = 0;
    std::vector<double> fw, cw;
};

bool parse_record(const std::vector<unsigned char> &b, Record &r) {
    size_t o = 0;
    int32_t iv[13];
    for (int32_t &x : iv)
        if (!get(b, o, x)) return false;
    ss_grid_params &p = r.p;
    p.geometry = iv[0]; p.precision = iv[1]; p.num_cells = iv[2]; p.mubar = iv[3]; p.quadrature = iv[4];
    p.nvars = iv[5]; p.kDim = iv[6]; p.b_kDim = iv[7]; p.patchOffsetL = iv[8]; p.ring_kmax_set = iv[9];
    r.ring_kmax = iv[10]; r.dtype = iv[11]; r.filtered = iv[12];
    p.ring_kmax = r.ring_kmax;
    if (!get(b, o, p.iMin) || !get(b, o, p.iMax) || !get(b, o, p.kMin) || !get(b, o, p.kMax)) return false;
    if (p.nvars <= 0 || p.nvars > (1 << 16)) return false;
    for (int v = 0; v < p.nvars; v++) {
        double lq;
        if (!get(b, o, lq)) return false;
        r.l_q.push_back(lq);
        for (int s = 0; s < 2; s++) {
            ss_spline_bc bc{};
            int32_t pad;
            if (!get(b, o, bc.kind) || !get(b, o, pad) || !get(b, o, bc.alpha) || !get(b, o, bc.beta)) return false;
            (s ? r.bcr : r.bcl).push_back(bc);
        }
        int32_t cbb, cbt, km, pad;
        if (!get(b, o, cbb) || !get(b, o, cbt) || !get(b, o, km) || !get(b, o, pad)) return false;
        r.bcb.push_back(cbb);
        r.bct.push_back(cbt);
        r.kmax.push_back(km);
    }
    int64_t nfw, ncw;
    if (!get(b, o, r.n_spectral) || !get(b, o, r.n_physical) || !get(b, o, r.nslots) || !get(b, o, r.nvars) ||
        !get(b, o, nfw) || !get(b, o, ncw))
        return false;
    if (nfw < 0 || ncw < 0 || o + size_t(nfw + ncw) * 8 != b.size()) return false;
    r.fw.resize(nfw);
    r.cw.resize(ncw);
    for (double &x : r.fw) get(b, o, x);
    for (double &x : r.cw) get(b, o, x);
    p.l_q = r.l_q.data();
    p.BCL = r.bcl.data();
    p.BCR = r.bcr.data();
    p.BCB = r.bcb.data();
    p.BCT = r.bct.data();
    p.max_wavenumber = r.kmax.data();
    return true;
}

struct Staging {
    void *buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Staging() {
        for (int i = 0; i < 2; i++) {
            if (buf[i]) cudaFreeHost(buf[i]);
            if (ev[i]) cudaEventDestroy(ev[i]);
        }
    }
    int32_t init() {
        for (int i = 0; i < 2; i++) {
            if (cudaHostAlloc(&buf[i], kChunk, cudaHostAllocDefault) != cudaSuccess ||
                cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                set_error("page-locked staging buffers for the grid archive");
                return SS_OUT_OF_MEMORY;
            }
        }
        return SS_OK;
    }
};

// device → file, chunk k's copy overlapping chunk k−1's write
int32_t stream_out(FILE *f, const void *dev, size_t bytes, cudaStream_t st, Staging &sg) {
    const size_t n = (bytes + kChunk - 1) / kChunk;
    for (size_t k = 0; k <= n; k++) {
        if (k < n) {
            const size_t len = std::min(kChunk, bytes - k * kChunk);
            if (cudaMemcpyAsync(sg.buf[k & 1], (const char *)dev + k * kChunk, len, cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess ||
                cudaEventRecord(sg.ev[k & 1], st) != cudaSuccess) {
                set_error("device→host copy of the grid archive: %s", cudaGetErrorString(cudaGetLastError()));
                return SS_CUDA_ERROR;
            }
        }
        if (k > 0) {
            const size_t j = k - 1, len = std::min(kChunk, bytes - j * kChunk);
            if (cudaEventSynchronize(sg.ev[j & 1]) != cudaSuccess) {
                set_error("device→host copy of the grid archive: %s", cudaGetErrorString(cudaGetLastError()));
                return SS_CUDA_ERROR;
            }
            if (fwrite(sg.buf[j & 1], 1, len, f) != len) {
                set_error("short write to the grid archive");
                return SS_BAD_ARG;
            }
        }
    }
    return SS_OK;
}

// file → device, chunk k+1's read overlapping chunk k's copy
int32_t stream_in(FILE *f, void *dev, size_t bytes, cudaStream_t st, Staging &sg) {
    const size_t n = (bytes + kChunk - 1) / kChunk;
    for (size_t k = 0; k < n; k++) {
        const size_t len = std::min(kChunk, bytes - k * kChunk);
        if (k >= 2 && cudaEventSynchronize(sg.ev[k & 1]) != cudaSuccess) {  // this buffer's previous copy
            set_error("host→device copy of the grid archive: %s", cudaGetErrorString(cudaGetLastError()));
            return SS_CUDA_ERROR;
        }
        if (fread(sg.buf[k & 1], 1, len, f) != len) {
            set_error("grid archive ends early");
            return SS_BAD_SHAPE;
        }
        if (cudaMemcpyAsync((char *)dev + k * kChunk, sg.buf[k & 1], len, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaEventRecord(sg.ev[k & 1], st) != cudaSuccess) {
            set_error("host→device copy of the grid archive: %s", cudaGetErrorString(cudaGetLastError()));
            return SS_CUDA_ERROR;
        }
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("host→device copy of the grid archive: %s", cudaGetErrorString(cudaGetLastError()));
        return SS_CUDA_ERROR;
    }
    return SS_OK;
}

int32_t read_header(FILE *f, Record &r, std::vector<unsigned char> &user) {
    char magic[8];
    uint32_t rb = 0, ub = 0;
    if (fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) != 0) {
        set_error("not a grid archive (bad magic or format version)");
        return SS_BAD_ARG;
    }
    if (fread(&rb, 4, 1, f) != 1 || fread(&ub, 4, 1, f) != 1 || rb > (64u << 20) || ub > (64u << 20)) {
        set_error("grid archive header is damaged");
        return SS_BAD_SHAPE;
    }
    std::vector<unsigned char> rec(rb);
    user.resize(ub);
    if ((rb && fread(rec.data(), 1, rb, f) != rb) || (ub && fread(user.data(), 1, ub, f) != ub) ||
        !parse_record(rec, r)) {
        set_error("grid archive parameter record is damaged");
        return SS_BAD_SHAPE;
    }
    return SS_OK;
}

int32_t load_arrays(ss_grid *g, FILE *f, const Record &r, cudaStream_t st) {
    const int32_t dtype = g->esz == 8 ? SS_DTYPE_F64 : SS_DTYPE_F32;
    if (r.dtype != dtype || r.n_spectral != g->d.n_spectral || r.n_physical != g->d.n_physical ||
        r.nslots != g->d.nslots || r.nvars != g->d.nvars) {
        set_error("grid archive holds arrays of another shape or storage type than this grid");
        return SS_BAD_SHAPE;
    }
    Staging sg;
    int32_t rc = sg.init();
    if (rc) return rc;
    const size_t es = g->esz;
    if ((rc = stream_in(f, g->spec, size_t(g->d.n_spectral) * g->d.nvars * es, st, sg))) return rc;
    return stream_in(f, g->phys, size_t(g->d.n_physical) * g->d.nvars * g->d.nslots * es, st, sg);
}

}  // namespace

extern "C" {

int32_t ss_grid_save(ss_grid *g, const char *path, const void *user, int64_t user_bytes, void *stream) {
    if (!g || !path || user_bytes < 0 || (user_bytes > 0 && !user)) {
        set_error("ss_grid_save: null grid, path or caller block");
        return SS_BAD_ARG;
    }
    cudaSetDevice(g->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    const int nv = (int)g->d.nvars, K = (int)g->d.kDim_wn, bk = (int)g->d.b_kDim;
    std::vector<double> fw(size_t(nv) * (K + 1)), cw(size_t(nv) * bk);
    if (cudaMemcpyAsync(fw.data(), g->d_fw, fw.size() * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(cw.data(), g->d_cw, cw.size() * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("reading the filter weights: %s", cudaGetErrorString(cudaGetLastError()));
        return SS_CUDA_ERROR;
    }
    const std::vector<unsigned char> rec = param_record(g, fw, cw);
    FileCloser fc{fopen(path, "wb")};
    if (!fc.f) {
        set_error("cannot open %s for writing", path);
        return SS_BAD_ARG;
    }
    const uint32_t rb = (uint32_t)rec.size(), ub = (uint32_t)user_bytes;
    if (fwrite(kMagic, 1, 8, fc.f) != 8 || fwrite(&rb, 4, 1, fc.f) != 1 || fwrite(&ub, 4, 1, fc.f) != 1 ||
        fwrite(rec.data(), 1, rb, fc.f) != rb || (ub && fwrite(user, 1, ub, fc.f) != ub)) {
        set_error("short write to %s", path);
        return SS_BAD_ARG;
    }
    Staging sg;
    int32_t rc = sg.init();
    if (rc) return rc;
    const size_t es = g->esz;
    if ((rc = stream_out(fc.f, g->spec, size_t(g->d.n_spectral) * nv * es, st, sg))) return rc;
    if ((rc = stream_out(fc.f, g->phys, size_t(g->d.n_physical) * nv * g->d.nslots * es, st, sg))) return rc;
    if (fflush(fc.f) != 0) {
        set_error("short write to %s", path);
        return SS_BAD_ARG;
    }
    return SS_OK;
}

int32_t ss_grid_load(const char *path, ss_grid **out, void *stream) {
    if (!path || !out) {
        set_error("ss_grid_load: null path or output");
        return SS_BAD_ARG;
    }
    *out = nullptr;
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) {
        set_error("cannot open %s", path);
        return SS_BAD_ARG;
    }
    Record r;
    std::vector<unsigned char> user;
    int32_t rc = read_header(fc.f, r, user);
    if (rc) return rc;
    ss_grid *g = nullptr;
    if ((rc = ss_grid_create(&r.p, &g))) return rc;
    if (r.filtered) {
        const int K = (int)g->d.kDim_wn, bk = (int)g->d.b_kDim;
        for (int v = 0; v < r.p.nvars && !rc; v++)
            rc = ss_grid_set_filter(g, v, r.fw.data() + size_t(v) * (K + 1), r.cw.data() + size_t(v) * bk);
    }
    if (!rc) rc = load_arrays(g, fc.f, r, stream ? (cudaStream_t)stream : g->stream);
    if (rc) {
        ss_grid_destroy(g);
        return rc;
    }
    *out = g;
    return SS_OK;
}

int32_t ss_grid_load_arrays(ss_grid *g, const char *path, void *stream) {
    if (!g || !path) {
        set_error("ss_grid_load_arrays: null grid or path");
        return SS_BAD_ARG;
    }
    cudaSetDevice(g->device);
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) {
        set_error("cannot open %s", path);
        return SS_BAD_ARG;
    }
    Record r;
    std::vector<unsigned char> user;
    int32_t rc = read_header(fc.f, r, user);
    if (rc) return rc;
    return load_arrays(g, fc.f, r, stream ? (cudaStream_t)stream : g->stream);
}

int32_t ss_grid_archive_user(const char *path, void *buf, int64_t cap, int64_t *user_bytes) {
    if (!path || !user_bytes || cap < 0 || (cap > 0 && !buf)) {
        set_error("ss_grid_archive_user: null argument");
        return SS_BAD_ARG;
    }
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) {
        set_error("cannot open %s", path);
        return SS_BAD_ARG;
    }
    Record r;
    std::vector<unsigned char> user;
    int32_t rc = read_header(fc.f, r, user);
    if (rc) return rc;
    *user_bytes = (int64_t)user.size();
    if (buf && cap > 0) std::memcpy(buf, user.data(), std::min<size_t>((size_t)cap, user.size()));
    return SS_OK;
}

}  // extern "C"
