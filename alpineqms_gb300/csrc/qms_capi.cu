// qms_capi.cu -- extern "C" entry points of libqms_gb300.so (declared in include/qms.h).
#include "qms_solver.h"
#include "qms_pl.h"

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

struct qms_handle {
    QmsSolver s;
};

static std::mutex g_err_mu;
static std::string g_create_err;

#define HCHECK(h)                                   \
    do {                                            \
        if (!(h)) return QMS_ERR_ARG;               \
    } while (0)

#define CKH(call)                                                                              \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess) {                                                               \
            h->s.err = std::string(#call) + ": " + cudaGetErrorString(_e);                     \
            return QMS_ERR_CUDA;                                                               \
        }                                                                                      \
    } while (0)

extern "C" {

void qms_default_desc(qms_desc* d, int xs, int ys, int zs, double dx, double dy, double dz, double dt) {
    std::memset(d, 0, sizeof(*d));
    d->xs = xs; d->ys = ys; d->zs = zs;
    d->dx = dx; d->dy = dy; d->dz = dz; d->dt = dt;
    d->precision = QMS_PREC_MIXED;
    d->tol = 2e-13;
    d->max_outer = 60;
    d->max_inner = 500;
    d->inner_rtol = 1e-3;
    d->check_every = 2;
    d->device = 0;
    d->precond = QMS_PRECOND_MG;
    d->mg_sweeps = 3;
    d->mg_omega = 0.85;
    d->mg_vshift = 0.0;
    d->krylov = QMS_KRYLOV_GMRES;
    d->gmres_m = 32;
    d->use_graphs = 1;
    d->mg_region_cut = 0.0;
    d->mg_alpha = 1.5;
    d->mg_coupling = 1;
    d->extrapolate = 3;
    d->gm_first_extend = 0;
    d->start_ls = 4;
}

size_t qms_device_bytes(const qms_desc* d) { return d ? qms_device_bytes_impl(*d) : 0; }

int64_t qms_n_dims(int xs, int ys, int zs) { return qms_make_grid(xs, ys, zs, 1, 1, 1).n; }

int64_t qms_csr_nnz(int xs, int ys, int zs) { return qms_csr_nnz(qms_make_grid(xs, ys, zs, 1, 1, 1)); }

int qms_create(const qms_desc* d, qms_handle** out) {
    if (!d || !out) return QMS_ERR_ARG;
    *out = nullptr;
    qms_handle* h = new (std::nothrow) qms_handle();
    if (!h) return QMS_ERR_NOMEM;
    qms_desc dd = *d;
    if (dd.check_every <= 0) dd.check_every = 1;
    if (!(dd.mg_alpha > 0)) dd.mg_alpha = 1.0;
    if (dd.mg_coarse_sweeps < 0) dd.mg_coarse_sweeps = 0;
    if (dd.mg_v_sweeps < 0) dd.mg_v_sweeps = 0;
    dd.extrapolate = std::max(0, std::min(dd.extrapolate, 3));
    dd.start_ls = std::max(0, std::min(dd.start_ls, 4));
    if (dd.max_inner <= 0 || dd.max_outer < 0 || !(dd.tol > 0) || !(dd.inner_rtol > 0) || dd.mg_sweeps < 1 ||
        !(dd.mg_omega > 0)) {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_create_err = "tol, inner_rtol, max_inner, mg_sweeps and mg_omega must be positive";
        delete h;
        return QMS_ERR_ARG;
    }
    int rc = h->s.init(dd);
    if (rc) {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_create_err = h->s.err;
        delete h;
        return rc == QMS_ERR_CUDA && g_create_err.find("memory") != std::string::npos ? QMS_ERR_NOMEM : rc;
    }
    *out = h;
    return 0;
}

void qms_destroy(qms_handle* h) { delete h; }

const char* qms_last_error(const qms_handle* h) {
    if (!h) {
        std::lock_guard<std::mutex> lk(g_err_mu);
        return g_create_err.c_str();
    }
    return h->s.err.c_str();
}

int qms_set_materials(qms_handle* h, const uint8_t* slots, const double* rows, int nmat) {
    HCHECK(h);
    if (!slots || (nmat > 0 && !rows)) { h->s.err = "null argument"; return QMS_ERR_ARG; }
    return h->s.set_materials(slots, rows, nmat);
}

int qms_set_geometry_f64(qms_handle* h, const double* geom, const double* table, int nmat) {
    HCHECK(h);
    if (!geom || !table || nmat < 1 || nmat > 255) { h->s.err = "need geometry and 1..255 materials"; return QMS_ERR_ARG; }
    QmsSolver& s = h->s;
    CKH(cudaSetDevice(s.dev));
    int maxid = 0;
    for (int r = 0; r < nmat; r++) {
        double idv = table[r * 7];
        if (!(idv >= 0 && idv < 16777217.0)) { s.err = "material IDs must be in 0..2^24"; return QMS_ERR_ARG; }
        maxid = std::max(maxid, (int)idv);
    }
    std::vector<uint8_t> lut(maxid + 1, 0);                   // F:234-238
    std::vector<double> rows(6 * nmat);
    for (int r = 0; r < nmat; r++) {
        lut[(int)table[r * 7]] = (uint8_t)(r + 1);
        for (int q = 0; q < 6; q++) rows[r * 6 + q] = table[r * 7 + 1 + q];
    }
    const long long ncell = (long long)s.g.xs * s.g.ys * s.g.zs;
    double* dgeom = nullptr;
    uint8_t* dlut = nullptr;
    CKH(cudaMalloc(&dgeom, ncell * 8));
    cudaError_t e = cudaMalloc(&dlut, lut.size());
    if (e != cudaSuccess) { cudaFree(dgeom); s.err = cudaGetErrorString(e); return QMS_ERR_CUDA; }
    cudaMemsetAsync(s.status, 0, 4, s.st);
    cudaMemcpyAsync(dgeom, geom, ncell * 8, cudaMemcpyHostToDevice, s.st);
    cudaMemcpyAsync(dlut, lut.data(), lut.size(), cudaMemcpyHostToDevice, s.st);
    qms_launch_ids(ncell, dgeom, dlut, maxid, s.ids, s.status, s.st);
    unsigned stt = 0;
    cudaMemcpyAsync(&stt, s.status, 4, cudaMemcpyDeviceToHost, s.st);
    e = cudaStreamSynchronize(s.st);
    cudaFree(dgeom);
    cudaFree(dlut);
    if (e != cudaSuccess) { s.err = cudaGetErrorString(e); return QMS_ERR_CUDA; }
    if (stt & QMS_ST_BAD_MATERIAL) {
        s.err = "geometry holds a material ID that is negative or above the largest table ID";
        return QMS_ERR_ARG;
    }
    return s.set_materials(nullptr, rows.data(), nmat);
}

static int finish_solve(qms_handle* h, int rc) {
    if (rc) return rc;
    if (h->s.stats.status & (QMS_ST_NAN | QMS_ST_NO_CONVERGENCE)) {
        h->s.err = (h->s.stats.status & QMS_ST_NAN) ? "non-finite residual" : "iteration limit reached";
        return QMS_ERR_CONVERGE;
    }
    return 0;
}

int qms_steady(qms_handle* h, const double v[3], const double B[3], const double G[9]) {
    HCHECK(h);
    if (!v || !B || !G) { h->s.err = "null argument"; return QMS_ERR_ARG; }
    return finish_solve(h, h->s.solve(false, v, B, G));
}

int qms_step(qms_handle* h, const double v[3], const double B[3], const double G[9]) {
    HCHECK(h);
    if (!v || !B || !G) { h->s.err = "null argument"; return QMS_ERR_ARG; }
    return finish_solve(h, h->s.solve(true, v, B, G));
}

int qms_get_stats(const qms_handle* h, qms_stats* out) {
    if (!h || !out) return QMS_ERR_ARG;
    *out = h->s.stats;
    return 0;
}

int qms_wait_selftest(qms_handle* h, int spins, unsigned* status_out) {
    HCHECK(h);
    if (spins < 1 || spins > (1 << 20)) { h->s.err = "spins must be in 1..2^20"; return QMS_ERR_ARG; }
    CKH(cudaSetDevice(h->s.dev));
    cudaStream_t st = h->s.st;
    CKH(cudaMemsetAsync(h->s.status, 0, sizeof(unsigned), st));
    qms_launch_wait_selftest(spins, h->s.status, st);
    CKH(cudaGetLastError());
    unsigned stt = 0;
    CKH(cudaMemcpyAsync(&stt, h->s.status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CKH(cudaStreamSynchronize(st));
    CKH(cudaMemsetAsync(h->s.status, 0, sizeof(unsigned), st));
    h->s.stats = qms_stats{};
    h->s.stats.status = stt;
    if (status_out) *status_out = stt;
    return 0;
}

int qms_get_fields_async(qms_handle* h, int which, int axis, int index, double* out, int slot) {
    HCHECK(h);
    if (!out) { h->s.err = "null argument"; return QMS_ERR_ARG; }
    return h->s.fields_async(which, axis, index, out, slot);
}

int qms_fields_sync(qms_handle* h, int slot) {
    HCHECK(h);
    return h->s.fields_sync(slot);
}

void* qms_pinned_alloc(size_t bytes) {
    void* p = nullptr;
    if (bytes == 0 || cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}

void qms_pinned_free(void* p) {
    if (p) cudaFreeHost(p);
}

int qms_get_fields(qms_handle* h, int which, int axis, int index, double* out) {
    HCHECK(h);
    if (!out) { h->s.err = "null argument"; return QMS_ERR_ARG; }
    return h->s.fields(which, axis, index, out);
}

int qms_get_state(qms_handle* h, double* x_out) {
    HCHECK(h);
    if (!x_out) return QMS_ERR_ARG;
    CKH(cudaSetDevice(h->s.dev));
    CKH(cudaMemcpyAsync(x_out, h->s.x, h->s.g.n * 8, cudaMemcpyDeviceToHost, h->s.st));
    CKH(cudaStreamSynchronize(h->s.st));
    return 0;
}

int qms_get_rhs(qms_handle* h, double* b_out) {
    HCHECK(h);
    if (!b_out) return QMS_ERR_ARG;
    CKH(cudaSetDevice(h->s.dev));
    h->s.ensure_b();
    CKH(cudaMemcpyAsync(b_out, h->s.b, h->s.g.n * 8, cudaMemcpyDeviceToHost, h->s.st));
    CKH(cudaStreamSynchronize(h->s.st));
    return 0;
}

int qms_set_state(qms_handle* h, const double* x_in) {
    HCHECK(h);
    if (!x_in) return QMS_ERR_ARG;
    CKH(cudaSetDevice(h->s.dev));
    CKH(cudaMemcpyAsync(h->s.x, x_in, h->s.g.n * 8, cudaMemcpyHostToDevice, h->s.st));
    CKH(cudaStreamSynchronize(h->s.st));
    h->s.rfin_ok = false;          // a new state: the next solve needs an exact anchor
    h->s.hist_len = 0;             // ... and has no history to extrapolate
    h->s.w_len = 0;
    h->s.last_chained = false;
    return 0;
}

int qms_assemble_csr(qms_handle* h, int transient, const double v[3], const double B[3], const double G[9],
                     const double* d_xprev, int64_t* d_ia, int32_t* d_ja, double* d_a, double* d_b) {
    HCHECK(h);
    if (!v || !B || !G || !d_ia || !d_ja || !d_a || !d_b || (transient && !d_xprev)) {
        h->s.err = "null argument";
        return QMS_ERR_ARG;
    }
    QmsSolver& s = h->s;
    CKH(cudaSetDevice(s.dev));
    QmsExcite ex;
    for (int q = 0; q < 3; q++) { ex.B[q] = B[q]; ex.v[q] = v[q]; }
    for (int q = 0; q < 9; q++) ex.G[q] = G[q];
    qms_launch_assemble(s.g, s.ids, s.dtab64, ex, s.desc.dt, transient ? 1 : 0, d_xprev, (long long*)d_ia, d_ja, d_a,
                        d_b, s.st);
    CKH(cudaGetLastError());
    CKH(cudaStreamSynchronize(s.st));
    return 0;
}

int qms_apply(qms_handle* h, int transient, const double v[3], int fp32, const void* d_x, void* d_y) {
    HCHECK(h);
    if (!v || !d_x || !d_y) { h->s.err = "null argument"; return QMS_ERR_ARG; }
    QmsSolver& s = h->s;
    CKH(cudaSetDevice(s.dev));
    const bool adv = v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0;
    if (fp32) {
        qms_launch_operator<float>(s.g, s.coef32(), qms_step_par<float>(s.g, v[0], v[1], v[2], s.desc.dt, transient != 0),
                                   adv, QOPH_APPLY, (const float*)d_x, nullptr, (float*)d_y, nullptr, nullptr, s.st);
    } else {
        qms_launch_operator<double>(s.g, s.coef64(),
                                    qms_step_par<double>(s.g, v[0], v[1], v[2], s.desc.dt, transient != 0), adv,
                                    QOPH_APPLY, (const double*)d_x, nullptr, (double*)d_y, nullptr, nullptr, s.st);
    }
    CKH(cudaGetLastError());
    CKH(cudaStreamSynchronize(s.st));
    return 0;
}

int qms_csr_spmv(qms_handle* h, const int64_t* d_ia, const int32_t* d_ja, const double* d_a, const double* d_x,
                 double* d_y) {
    HCHECK(h);
    if (!d_ia || !d_ja || !d_a || !d_x || !d_y) { h->s.err = "null argument"; return QMS_ERR_ARG; }
    CKH(cudaSetDevice(h->s.dev));
    qms_launch_csr_spmv(h->s.g.n, (const long long*)d_ia, d_ja, d_a, d_x, d_y, h->s.st);
    CKH(cudaGetLastError());
    CKH(cudaStreamSynchronize(h->s.st));
    return 0;
}

int qms_residual_norm(qms_handle* h, int transient, const double v[3], double* rel_out) {
    HCHECK(h);
    if (!v || !rel_out) return QMS_ERR_ARG;
    QmsSolver& s = h->s;
    CKH(cudaSetDevice(s.dev));
    const bool adv = v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0;
    s.ensure_b();
    int rc = s.residual(adv, transient != 0, v, true);
    if (rc) return rc;
    double xn = std::sqrt(s.hS[0 + 2] + s.hS[0 + 3]);
    double rn = std::sqrt(s.hS[0] + s.hS[1]);
    *rel_out = xn > 0 ? rn / xn : rn;
    return 0;
}

int qms_profile_enable(qms_handle* h, int on) {
    HCHECK(h);
    CKH(cudaSetDevice(h->s.dev));
    return h->s.profile_enable(on != 0);
}

int qms_get_profile(qms_handle* h, qms_profile* out) {
    HCHECK(h);
    if (!out) return QMS_ERR_ARG;
    CKH(cudaSetDevice(h->s.dev));
    return h->s.profile_collect(out);
}

void* qms_get_stream(qms_handle* h) { return h ? (void*)h->s.st : nullptr; }

}  // extern "C"
