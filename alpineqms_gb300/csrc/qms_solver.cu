// qms_solver.cu -- the per-step linear solve that replaces MKL PARDISO
// (3D/QMS_3D.f90:1314-1317 phase 13, F:2193-2203 phases 23/33).
//
// Structure of one solve (steady init or one backward-Euler step):
//   b, Dirichlet values of x  <- K7 (qms_exact.cu)
//   repeat (FP64 iterative refinement):
//       r = D^-1 (b - M x)                       FP64 matrix-free residual (K3)
//       stop when ||r|| <= tol * ||x||
//       e ~= (D^-1 M)^-1 r / ||r||               inner Krylov in T (FP32 = mixed, FP64 = plain)
//       x += ||r|| e                             FP64 accumulation
// Inner Krylov: PCG (Jacobi) for the symmetric steady magnetostatic problem
// (v = 0, V block identically zero), BiCGSTAB on the row-scaled operator for
// every nonsymmetric system.  All Krylov scalars (alpha, beta, omega, rho)
// live in device memory and are formed by one-block finalize kernels from
// deterministic block partial sums, so the vector kernels never wait for the
// host; the host only reads the residual estimate to decide when to stop.
#include "qms_internal.h"
#include "qms_solver.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

// --------------------------------------------------------------------------
// scalar slots in the device array S
// --------------------------------------------------------------------------
enum {
    S_RA = 0, S_RV, S_XA, S_XV,   // IR residual / solution norms (squared, by block)
    S_NRM, S_INVNRM,              // ||r||, 1/||r|| of the IR residual
    S_RR0, S_RR,                  // inner residual norms^2 (initial, current)
    S_RHO, S_ALPHA, S_OMEGA, S_BETA,
    S_RZ, S_RZ0,
    S_COUNT = 32
};

enum FinOp {
    FIN_RESID = 0, FIN_BICG_INIT, FIN_BICG_ALPHA, FIN_BICG_OMEGA, FIN_BICG_RHO,
    FIN_CG_INIT, FIN_CG_ALPHA, FIN_CG_BETA
};

__global__ void qk_finalize(const double* __restrict__ part, long long nb, int nsum, double* __restrict__ S, int op,
                            unsigned* __restrict__ status) {
    __shared__ double sh[32];
    double sums[4];
    for (int q = 0; q < nsum; q++) {
        double acc = 0.0;
        for (long long t = threadIdx.x; t < nb; t += blockDim.x) acc += part[q * nb + t];
        sums[q] = qBlockSum(acc, sh);
    }
    if (threadIdx.x != 0) return;
    switch (op) {
    case FIN_RESID: {
        S[S_RA] = sums[0]; S[S_RV] = sums[1]; S[S_XA] = sums[2]; S[S_XV] = sums[3];
        double nr = sqrt(sums[0] + sums[1]);
        if (!isfinite(nr)) { atomicOr(status, (unsigned)QMS_ST_NAN); nr = 0.0; }
        S[S_NRM] = nr;
        S[S_INVNRM] = nr > 0.0 ? 1.0 / nr : 0.0;
        break;
    }
    case FIN_BICG_INIT:
        S[S_RR0] = sums[0]; S[S_RR] = sums[0]; S[S_RHO] = sums[0];
        S[S_ALPHA] = 1.0; S[S_OMEGA] = 1.0; S[S_BETA] = 0.0;
        break;
    case FIN_BICG_ALPHA: {
        double rv = sums[0];
        if (rv == 0.0 || !isfinite(rv)) { atomicOr(status, (unsigned)QMS_ST_BREAKDOWN); S[S_ALPHA] = 0.0; }
        else S[S_ALPHA] = S[S_RHO] / rv;
        break;
    }
    case FIN_BICG_OMEGA: {
        double ts = sums[0], tt = sums[1];
        S[S_OMEGA] = (tt > 0.0 && isfinite(tt)) ? ts / tt : 0.0;
        break;
    }
    case FIN_BICG_RHO: {
        double rho_new = sums[0];
        double om = S[S_OMEGA];
        if (S[S_RHO] == 0.0 || om == 0.0) { atomicOr(status, (unsigned)QMS_ST_BREAKDOWN); S[S_BETA] = 0.0; }
        else S[S_BETA] = (rho_new / S[S_RHO]) * (S[S_ALPHA] / om);
        S[S_RHO] = rho_new;
        S[S_RR] = sums[1];
        break;
    }
    case FIN_CG_INIT:
        S[S_RZ] = sums[0]; S[S_RZ0] = sums[0]; S[S_RR0] = sums[1]; S[S_RR] = sums[1];
        break;
    case FIN_CG_ALPHA: {
        double pq = sums[0];
        if (pq <= 0.0 || !isfinite(pq)) { atomicOr(status, (unsigned)QMS_ST_BREAKDOWN); S[S_ALPHA] = 0.0; }
        else S[S_ALPHA] = S[S_RZ] / pq;
        break;
    }
    case FIN_CG_BETA: {
        double rz_new = sums[0];
        S[S_BETA] = S[S_RZ] != 0.0 ? rz_new / S[S_RZ] : 0.0;
        S[S_RZ] = rz_new;
        S[S_RR] = sums[1];
        break;
    }
    }
}

// --------------------------------------------------------------------------
// fused vector kernels (grid-stride; block partials for the dot products)
// --------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void store_partials(double* part, float a, float b) {
    __shared__ double sh[32];
    double s0 = qBlockSum(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s0;
    double s1 = qBlockSum(b, sh);
    if (threadIdx.x == 0) part[gridDim.x + blockIdx.x] = s1;
}

template <typename T>
__global__ void qk_bicg_init(long long n, const double* __restrict__ r64, const double* __restrict__ S,
                             T* __restrict__ r, T* __restrict__ rh, T* __restrict__ p, T* __restrict__ v,
                             T* __restrict__ e, double* __restrict__ part) {
    const double inv = S[S_INVNRM];
    float acc = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        T rv = (T)(r64[t] * inv);
        r[t] = rv; rh[t] = rv; p[t] = T(0); v[t] = T(0); e[t] = T(0);
        acc += (float)(rv * rv);
    }
    store_partials<T>(part, acc, 0.f);
}

template <typename T>
__global__ void qk_bicg_p(long long n, const T* __restrict__ r, T* __restrict__ p, const T* __restrict__ v,
                          const double* __restrict__ S) {
    const T beta = (T)S[S_BETA], om = (T)S[S_OMEGA];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        p[t] = r[t] + beta * (p[t] - om * v[t]);
}

template <typename T>
__global__ void qk_bicg_s(long long n, const T* __restrict__ r, const T* __restrict__ v, T* __restrict__ s,
                          const double* __restrict__ S) {
    const T al = (T)S[S_ALPHA];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        s[t] = r[t] - al * v[t];
}

template <typename T>
__global__ void qk_bicg_xr(long long n, const T* __restrict__ p, const T* __restrict__ s, const T* __restrict__ tt,
                           const T* __restrict__ rh, T* __restrict__ e, T* __restrict__ r, const double* __restrict__ S,
                           double* __restrict__ part) {
    const T al = (T)S[S_ALPHA], om = (T)S[S_OMEGA];
    float a0 = 0.f, a1 = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        T st = s[t];
        e[t] += al * p[t] + om * st;
        T rn = st - om * tt[t];
        r[t] = rn;
        a0 += (float)(rh[t] * rn);
        a1 += (float)(rn * rn);
    }
    store_partials<T>(part, a0, a1);
}

template <typename T>
__global__ void qk_cg_init(long long n, long long mask_from, const double* __restrict__ r64,
                           const float* __restrict__ dg, const double* __restrict__ S, T* __restrict__ r,
                           T* __restrict__ z, T* __restrict__ p, T* __restrict__ e, double* __restrict__ part) {
    const double inv = S[S_INVNRM];
    float a0 = 0.f, a1 = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        T d = (T)dg[t];
        T rs = (T)(r64[t] * inv);           // scaled residual D^-1 r
        T rv = d * rs;                      // unscaled residual
        T zv = t < mask_from ? rs : T(0);   // Jacobi: z = D^-1 r
        r[t] = rv; z[t] = zv; p[t] = zv; e[t] = T(0);
        a0 += (float)(rv * zv);
        a1 += (float)(rs * rs);
    }
    store_partials<T>(part, a0, a1);
}

template <typename T>
__global__ void qk_cg_update(long long n, long long mask_from, const T* __restrict__ p, const T* __restrict__ q,
                             const float* __restrict__ dg, const double* __restrict__ S, T* __restrict__ e,
                             T* __restrict__ r, T* __restrict__ z, double* __restrict__ part) {
    const T al = (T)S[S_ALPHA];
    float a0 = 0.f, a1 = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        e[t] += al * p[t];
        T rv = r[t] - al * q[t];
        r[t] = rv;
        T zv = t < mask_from ? rv / (T)dg[t] : T(0);
        z[t] = zv;
        a0 += (float)(rv * zv);
        a1 += (float)(zv * zv);
    }
    store_partials<T>(part, a0, a1);
}

template <typename T>
__global__ void qk_cg_p(long long n, const T* __restrict__ z, T* __restrict__ p, const double* __restrict__ S) {
    const T be = (T)S[S_BETA];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        p[t] = z[t] + be * p[t];
}

template <typename T>
__global__ void qk_ir_update(long long n, const T* __restrict__ e, const double* __restrict__ S, double* __restrict__ x) {
    const double nr = S[S_NRM];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        x[t] += nr * (double)e[t];
}

// --------------------------------------------------------------------------
// material table
// --------------------------------------------------------------------------
template <typename T>
void qms_fill_table(QMatTable<T>& t, const double* rows6, int nmat) {
    for (int s = 0; s < QMS_MAX_SLOTS; s++) {
        for (int d = 0; d < 3; d++) {
            double mu = QMS_MU0, sg = 0.0;                    // slot 0 and unused slots: vacuum (F:211-225)
            if (s >= 1 && s <= nmat) {
                mu = rows6[(s - 1) * 6 + d] * QMS_MU0;        // F:245-247
                sg = rows6[(s - 1) * 6 + 3 + d];              // F:248-250
            }
            t.mu[3 * s + d] = (T)mu;
            t.imu[3 * s + d] = (T)(1.0 / mu);
            t.sig[3 * s + d] = (T)sg;
        }
    }
}
template void qms_fill_table<double>(QMatTable<double>&, const double*, int);
template void qms_fill_table<float>(QMatTable<float>&, const double*, int);

// --------------------------------------------------------------------------
// solver object
// --------------------------------------------------------------------------
#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t _e = (call);                                                          \
        if (_e != cudaSuccess) {                                                          \
            err = std::string(#call) + ": " + cudaGetErrorString(_e);                     \
            return QMS_ERR_CUDA;                                                          \
        }                                                                                 \
    } while (0)

QmsSolver::~QmsSolver() { release(); }

void QmsSolver::release() {
    if (dev >= 0) cudaSetDevice(dev);
    void* ptrs[] = {ids, dtab64, dtab32, x, b, r64, H, slicebuf, part, S, status, dg_steady, dg_tr};
    for (void* q : ptrs) if (q) cudaFree(q);
    if (hS) cudaFreeHost(hS);
    for (auto& p : vec) if (p) cudaFree(p);
    for (auto& e : evpool) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    evpool.clear();
    if (st && own_stream) cudaStreamDestroy(st);
    ids = nullptr; dtab64 = nullptr; dtab32 = nullptr; x = b = r64 = H = slicebuf = part = S = nullptr;
    status = nullptr; dg_steady = dg_tr = nullptr; hS = nullptr; st = nullptr;
    for (auto& p : vec) p = nullptr;
}

int QmsSolver::init(const qms_desc& d) {
    desc = d;
    dev = d.device;
    CK(cudaSetDevice(dev));
    if (d.xs < 4 || d.ys < 4 || d.zs < 4) { err = "grid must have at least 4 cells per axis"; return QMS_ERR_ARG; }
    if (!(d.dx > 0 && d.dy > 0 && d.dz > 0 && d.dt > 0)) { err = "dx, dy, dz, dt must be positive"; return QMS_ERR_ARG; }
    g = qms_make_grid(d.xs, d.ys, d.zs, d.dx, d.dy, d.dz);
    fp64_inner = d.precision == QMS_PREC_FP64;
    tsize = fp64_inner ? sizeof(double) : sizeof(float);
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    vec_blocks = (long long)nsm * 8;
    long long need = (g.n + 255) / 256;
    if (need < vec_blocks) vec_blocks = need;
    nbop = qms_op_num_blocks(g);
    long long npart = std::max(4 * nbop, 2 * vec_blocks) + 64;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    own_stream = true;
    const long long n = g.n, ncell = (long long)g.xs * g.ys * g.zs;
    CK(cudaMalloc(&ids, ncell));
    CK(cudaMemset(ids, 0, ncell));
    CK(cudaMalloc(&dtab64, sizeof(QMatTable<double>)));
    CK(cudaMalloc(&dtab32, sizeof(QMatTable<float>)));
    CK(cudaMalloc(&x, n * 8));
    CK(cudaMalloc(&b, n * 8));
    CK(cudaMalloc(&r64, n * 8));
    CK(cudaMalloc(&H, 3 * ncell * 8));
    long long smax = std::max({(long long)g.ys * g.zs, (long long)g.xs * g.zs, (long long)g.xs * g.ys});
    CK(cudaMalloc(&slicebuf, 3 * smax * 8));
    CK(cudaMalloc(&part, npart * 8));
    CK(cudaMalloc(&S, S_COUNT * 8));
    CK(cudaMemset(S, 0, S_COUNT * 8));
    CK(cudaMalloc(&status, sizeof(unsigned)));
    CK(cudaMemset(status, 0, sizeof(unsigned)));
    CK(cudaMalloc(&dg_steady, n * 4));
    CK(cudaMalloc(&dg_tr, n * 4));
    for (auto& p : vec) CK(cudaMalloc(&p, n * tsize));
    CK(cudaMallocHost(&hS, S_COUNT * 8));
    CK(cudaMemset(x, 0, n * 8));
    double vac[6] = {1, 1, 1, 0, 0, 0};
    return set_materials(nullptr, vac, 0);
}

size_t qms_device_bytes_impl(const qms_desc& d) {
    QGrid g = qms_make_grid(d.xs, d.ys, d.zs, d.dx, d.dy, d.dz);
    size_t ts = d.precision == QMS_PREC_FP64 ? 8 : 4;
    size_t ncell = (size_t)g.xs * g.ys * g.zs;
    size_t smax = std::max({(size_t)g.ys * g.zs, (size_t)g.xs * g.zs, (size_t)g.xs * g.ys});
    size_t nb = (size_t)qms_op_num_blocks(g);
    return ncell + sizeof(QMatTable<double>) + sizeof(QMatTable<float>) + 3 * g.n * 8 + 3 * ncell * 8 +
           3 * smax * 8 + (4 * nb + 64) * 8 + 2 * g.n * 4 + QMS_NVEC * g.n * ts + 4096;
}

int QmsSolver::set_materials(const uint8_t* host_slots, const double* rows6, int nmat) {
    CK(cudaSetDevice(dev));
    if (nmat < 0 || nmat > QMS_MAX_SLOTS - 1) { err = "nmat must be in 0..255"; return QMS_ERR_ARG; }
    const long long ncell = (long long)g.xs * g.ys * g.zs;
    if (host_slots) {
        for (long long c = 0; c < ncell; c++)
            if (host_slots[c] > nmat) { err = "material slot above nmat"; return QMS_ERR_ARG; }
        CK(cudaMemcpyAsync(ids, host_slots, ncell, cudaMemcpyHostToDevice, st));
    }
    qms_fill_table(htab64, rows6, nmat);
    qms_fill_table(htab32, rows6, nmat);
    CK(cudaMemcpyAsync(dtab64, &htab64, sizeof(htab64), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dtab32, &htab32, sizeof(htab32), cudaMemcpyHostToDevice, st));
    // Jacobi diagonals of the steady and transient operators (velocity does not enter the diagonal)
    QCoef<float> c32 = coef32();
    qms_launch_diag(g, c32, qms_step_par<float>(g, 0, 0, 0, desc.dt, false), dg_steady, st);
    qms_launch_diag(g, c32, qms_step_par<float>(g, 0, 0, 0, desc.dt, true), dg_tr, st);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    return 0;
}

QCoef<float> QmsSolver::coef32() const { return QCoef<float>{g, ids, dtab32, (float)(1.0 / QMS_MU0)}; }
QCoef<double> QmsSolver::coef64() const { return QCoef<double>{g, ids, dtab64, 1.0 / QMS_MU0}; }

int QmsSolver::finalize(int fop, int nsum, long long nb) {
    qk_finalize<<<1, 512, 0, st>>>(part, nb, nsum, S, fop, status);
    nlaunch++;
    return 0;
}

template <typename T>
void QmsSolver::op(bool adv, int mode, const QStepPar<T>& P, const T* xin, const T* bin, T* y, const T* w,
                   double* partials) {
    OpEv* ev = nullptr;
    if (prof) {
        if (evused == evpool.size()) {
            OpEv e{};
            cudaEventCreate(&e.a);
            cudaEventCreate(&e.b);
            evpool.push_back(e);
        }
        ev = &evpool[evused++];
        ev->fp64 = sizeof(T) == 8;
        const double ncell = (double)g.xs * g.ys * g.zs;
        ev->bytes = (double)g.n * sizeof(T) * (2 + (w && w != xin ? 1 : 0) + (bin ? 1 : 0)) + ncell;
        cudaEventRecord(ev->a, st);
    }
    qms_launch_operator<T>(g, coef<T>(), P, adv, mode, xin, bin, y, w, partials, st);
    nlaunch++;
    if (ev) cudaEventRecord(ev->b, st);
}
template void QmsSolver::op<float>(bool, int, const QStepPar<float>&, const float*, const float*, float*,
                                   const float*, double*);
template void QmsSolver::op<double>(bool, int, const QStepPar<double>&, const double*, const double*, double*,
                                    const double*, double*);

int QmsSolver::profile_enable(bool on) {
    if (prof || on) {
        cudaStreamSynchronize(st);
    }
    prof = on;
    nlaunch = 0;
    evused = 0;
    profacc = qms_profile{};
    return 0;
}

int QmsSolver::profile_collect(qms_profile* out) {
    CK(cudaStreamSynchronize(st));
    for (size_t q = 0; q < evused; q++) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, evpool[q].a, evpool[q].b));
        if (evpool[q].fp64) { profacc.op64_launches++; profacc.op64_ms += ms; profacc.op64_bytes += evpool[q].bytes; }
        else { profacc.op32_launches++; profacc.op32_ms += ms; profacc.op32_bytes += evpool[q].bytes; }
    }
    evused = 0;
    profacc.launches = nlaunch;
    *out = profacc;
    return 0;
}

int QmsSolver::read_scalars() {
    CK(cudaMemcpyAsync(hS, S, S_COUNT * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

template <typename T>
int QmsSolver::inner_bicgstab(bool adv, bool transient, const double v[3], int& iters) {
    const long long n = g.n;
    T* r = (T*)vec[0]; T* rh = (T*)vec[1]; T* p = (T*)vec[2]; T* vv = (T*)vec[3];
    T* s = (T*)vec[4]; T* t = (T*)vec[5]; T* e = (T*)vec[6];
    QStepPar<T> P = qms_step_par<T>(g, v[0], v[1], v[2], desc.dt, transient);
    const int vb = (int)vec_blocks;
    qk_bicg_init<T><<<vb, 256, 0, st>>>(n, r64, S, r, rh, p, vv, e, part);
    nlaunch++;
    finalize(FIN_BICG_INIT, 1, vec_blocks);
    const double tol2 = desc.inner_rtol * desc.inner_rtol;
    iters = 0;
    for (int it = 0; it < desc.max_inner; it++) {
        qk_bicg_p<T><<<vb, 256, 0, st>>>(n, r, p, vv, S);
        nlaunch++;
        op<T>(adv, QOPH_SCALED, P, p, nullptr, vv, rh, part);
        finalize(FIN_BICG_ALPHA, 1, nbop);
        qk_bicg_s<T><<<vb, 256, 0, st>>>(n, r, vv, s, S);
        nlaunch++;
        op<T>(adv, QOPH_SCALED, P, s, nullptr, t, s, part);
        finalize(FIN_BICG_OMEGA, 2, nbop);
        qk_bicg_xr<T><<<vb, 256, 0, st>>>(n, p, s, t, rh, e, r, S, part);
        nlaunch++;
        finalize(FIN_BICG_RHO, 2, vec_blocks);
        iters = it + 1;
        if ((it + 1) % desc.check_every == 0 || it + 1 == desc.max_inner) {
            int rc = read_scalars();
            if (rc) return rc;
            if (!(hS[S_RR] <= tol2 * hS[S_RR0])) {
                unsigned stt = 0;
                CK(cudaMemcpy(&stt, status, 4, cudaMemcpyDeviceToHost));
                if (stt & QMS_ST_BREAKDOWN) break;
                continue;
            }
            break;
        }
    }
    qk_ir_update<T><<<vb, 256, 0, st>>>(n, e, S, x);
    nlaunch++;
    CK(cudaGetLastError());
    return 0;
}

template <typename T>
int QmsSolver::inner_pcg(bool transient, int& iters) {
    const long long n = g.n;
    T* r = (T*)vec[0]; T* z = (T*)vec[1]; T* p = (T*)vec[2]; T* q = (T*)vec[3]; T* e = (T*)vec[6];
    const float* dg = transient ? dg_tr : dg_steady;
    QStepPar<T> P = qms_step_par<T>(g, 0, 0, 0, desc.dt, transient);
    const int vb = (int)vec_blocks;
    const long long mask_from = g.oV;     // V block frozen at zero (steady, v = 0)
    qk_cg_init<T><<<vb, 256, 0, st>>>(n, mask_from, r64, dg, S, r, z, p, e, part);
    nlaunch++;
    finalize(FIN_CG_INIT, 2, vec_blocks);
    const double tol2 = desc.inner_rtol * desc.inner_rtol;
    iters = 0;
    for (int it = 0; it < desc.max_inner; it++) {
        op<T>(false, QOPH_APPLY, P, p, nullptr, q, p, part);
        finalize(FIN_CG_ALPHA, 1, nbop);
        qk_cg_update<T><<<vb, 256, 0, st>>>(n, mask_from, p, q, dg, S, e, r, z, part);
        nlaunch++;
        finalize(FIN_CG_BETA, 2, vec_blocks);
        iters = it + 1;
        if ((it + 1) % desc.check_every == 0 || it + 1 == desc.max_inner) {
            int rc = read_scalars();
            if (rc) return rc;
            if (hS[S_RZ] <= tol2 * hS[S_RZ0]) break;
        }
        qk_cg_p<T><<<vb, 256, 0, st>>>(n, z, p, S);
        nlaunch++;
    }
    qk_ir_update<T><<<vb, 256, 0, st>>>(n, e, S, x);
    nlaunch++;
    CK(cudaGetLastError());
    return 0;
}

int QmsSolver::residual(bool adv, bool transient, const double v[3]) {
    QStepPar<double> P = qms_step_par<double>(g, v[0], v[1], v[2], desc.dt, transient);
    op<double>(adv, QOPH_RESID, P, x, b, r64, nullptr, part);
    finalize(FIN_RESID, 4, nbop);
    CK(cudaGetLastError());
    return read_scalars();
}

int QmsSolver::solve(bool transient, const double v[3], const double B[3], const double G[9]) {
    CK(cudaSetDevice(dev));
    QmsExcite ex;
    for (int q = 0; q < 3; q++) { ex.B[q] = B[q]; ex.v[q] = v[q]; }
    for (int q = 0; q < 9; q++) ex.G[q] = G[q];
    // b from the previous solution (x); Dirichlet values written into x (warm start keeps them exact)
    qms_launch_rhs(g, ids, dtab64, ex, desc.dt, transient ? 1 : 0, x, b, x, st);
    nlaunch++;
    CK(cudaMemsetAsync(status, 0, 4, st));
    const bool adv = v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0;
    const bool use_cg = !transient && !adv;
    stats = qms_stats{};
    double rel = INFINITY;
    int outer = 0;
    for (;;) {
        int rc = residual(adv, transient, v);
        if (rc) return rc;
        double xn = std::sqrt(hS[S_XA] + hS[S_XV]);
        double rn = std::sqrt(hS[S_RA] + hS[S_RV]);
        rel = xn > 0 ? rn / xn : rn;
        if (outer == 0) stats.initial_residual = rel;
        if (!std::isfinite(rel)) { stats.status |= QMS_ST_NAN; break; }
        if (rel <= desc.tol || rn == 0.0) break;
        if (outer >= desc.max_outer) { stats.status |= QMS_ST_NO_CONVERGENCE; break; }
        int it = 0;
        if (use_cg) rc = fp64_inner ? inner_pcg<double>(transient, it) : inner_pcg<float>(transient, it);
        else rc = fp64_inner ? inner_bicgstab<double>(adv, transient, v, it)
                             : inner_bicgstab<float>(adv, transient, v, it);
        if (rc) return rc;
        stats.inner_iterations += it;
        outer++;
    }
    unsigned stt = 0;
    CK(cudaMemcpyAsync(&stt, status, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    stats.status |= stt & ~(unsigned)QMS_ST_BREAKDOWN;
    stats.outer_iterations = outer;
    stats.final_residual = rel;
    return 0;
}

int QmsSolver::fields(int which, int axis, int index, double* host_out) {
    CK(cudaSetDevice(dev));
    const long long ncell = (long long)g.xs * g.ys * g.zs;
    qms_launch_hfield(g, ids, dtab64, x, H, H + ncell, H + 2 * ncell, st);
    nlaunch++;
    if (which == QMS_FIELD_CUBES) {
        CK(cudaMemcpyAsync(host_out, H, 3 * ncell * 8, cudaMemcpyDeviceToHost, st));
    } else {
        int lim = axis == 0 ? g.xs : axis == 1 ? g.ys : g.zs;
        if (axis < 0 || axis > 2 || index < 1 || index > lim) { err = "slice axis/index out of range"; return QMS_ERR_ARG; }
        qms_launch_slice(g, axis, index, H, H + ncell, H + 2 * ncell, slicebuf, st);
        nlaunch++;
        long long m = (long long)(axis == 0 ? g.ys : g.xs) * (axis == 2 ? g.ys : g.zs);
        CK(cudaMemcpyAsync(host_out, slicebuf, 3 * m * 8, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    return 0;
}

template int QmsSolver::inner_bicgstab<float>(bool, bool, const double*, int&);
template int QmsSolver::inner_bicgstab<double>(bool, bool, const double*, int&);
template int QmsSolver::inner_pcg<float>(bool, int&);
template int QmsSolver::inner_pcg<double>(bool, int&);
