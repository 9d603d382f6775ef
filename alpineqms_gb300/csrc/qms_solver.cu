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
#include "qms_pl.h"

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
    // the convergence test of a step captured whole (qk_cond_init / qk_cond_next)
    S_SREF = 23, S_REL, S_REL0, S_CYC, S_PRN, S_PRN_LAST,
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
// convergence test of a whole step captured in one graph: the host loop's relative residual
// rel = |r| / min(max(|x|, s), 100 s), s = |x| at the start of the solve, from the finalized
// residual sums; the WHILE node runs another refinement cycle while rel > tol, at most
// maxcyc cycles, and while each cycle at least removes a tenth of the residual
// --------------------------------------------------------------------------
__global__ void qk_cond_init(double* __restrict__ S, double tol, cudaGraphConditionalHandle hc) {
    if (threadIdx.x != 0) return;
    const double xn = sqrt(S[S_XA] + S[S_XV]), rn = S[S_NRM];
    const double sref = xn > 0.0 ? xn : 1.0;
    const double rel = rn / fmin(fmax(xn, sref), 100.0 * sref);
    S[S_SREF] = sref;
    S[S_REL] = rel;
    S[S_REL0] = rel;
    S[S_CYC] = 0.0;
    S[S_PRN] = rn;
    S[S_PRN_LAST] = rn;
    cudaGraphSetConditional(hc, (isfinite(rel) && rel > tol && rn != 0.0) ? 1u : 0u);
}

__global__ void qk_cond_next(double* __restrict__ S, double tol, int maxcyc, cudaGraphConditionalHandle hc) {
    if (threadIdx.x != 0) return;
    const double xn = sqrt(S[S_XA] + S[S_XV]), rn = S[S_NRM], sref = S[S_SREF];
    const double rel = rn / fmin(fmax(xn, sref), 100.0 * sref);
    const double prev = S[S_PRN];
    const double cyc = S[S_CYC] + 1.0;
    S[S_CYC] = cyc;
    S[S_REL] = rel;
    S[S_PRN_LAST] = prev;
    S[S_PRN] = rn;
    const bool more = isfinite(rel) && rel > tol && rn != 0.0 && cyc < (double)maxcyc && rn < 0.9 * prev;
    cudaGraphSetConditional(hc, more ? 1u : 0u);
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

// r holds the normalised residual (converted from the FP64 residual): rh = r, p = v = e = 0
template <typename T>
__global__ void qk_bicg_init(long long n, const T* __restrict__ r, T* __restrict__ rh, T* __restrict__ p,
                             T* __restrict__ v, T* __restrict__ e, double* __restrict__ part) {
    float acc = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const T rv = r[t];
        rh[t] = rv; p[t] = T(0); v[t] = T(0); e[t] = T(0);
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
__global__ void qk_bicg_xr(long long n, const T* __restrict__ y, const T* __restrict__ z, const T* __restrict__ s,
                           const T* __restrict__ tt, const T* __restrict__ rh, T* __restrict__ e, T* __restrict__ r,
                           const double* __restrict__ S, double* __restrict__ part) {
    const T al = (T)S[S_ALPHA], om = (T)S[S_OMEGA];
    float a0 = 0.f, a1 = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        T st = s[t];
        e[t] += al * y[t] + om * z[t];
        T rn = st - om * tt[t];
        r[t] = rn;
        a0 += (float)(rh[t] * rn);
        a1 += (float)(rn * rn);
    }
    store_partials<T>(part, a0, a1);
}

// r = D r, the unscaled residual of the normalised system (r holds the normalised scaled
// residual converted from the FP64 one), e = 0
template <typename T>
__global__ void qk_cg_init(long long n, const float* __restrict__ dg, T* __restrict__ r, T* __restrict__ e) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        r[t] = (T)dg[t] * r[t];
        e[t] = T(0);
    }
}

// Jacobi preconditioner of the unscaled system (V block frozen when mask_from < n)
template <typename T>
__global__ void qk_jacobi(long long n, long long mask_from, const T* __restrict__ r, const float* __restrict__ dg,
                          T* __restrict__ z) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const float d = dg[t];                   // 0 on the padding of the layout
        z[t] = t < mask_from && d != 0.f ? r[t] / (T)d : T(0);
    }
}

// partials of r.z and z.z; optionally p = z (first iteration)
template <typename T>
__global__ void qk_cg_dot(long long n, const T* __restrict__ r, const T* __restrict__ z, T* __restrict__ p,
                          double* __restrict__ part) {
    float a0 = 0.f, a1 = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        T zv = z[t];
        if (p) p[t] = zv;
        a0 += (float)(r[t] * zv);
        a1 += (float)(zv * zv);
    }
    store_partials<T>(part, a0, a1);
}

template <typename T>
__global__ void qk_cg_update(long long n, const T* __restrict__ p, const T* __restrict__ q,
                             const double* __restrict__ S, T* __restrict__ e, T* __restrict__ r) {
    const T al = (T)S[S_ALPHA];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        e[t] += al * p[t];
        r[t] -= al * q[t];
    }
}

template <typename T>
__global__ void qk_cg_p(long long n, const T* __restrict__ z, T* __restrict__ p, const double* __restrict__ S) {
    const T be = (T)S[S_BETA];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        p[t] = z[t] + be * p[t];
}



// --------------------------------------------------------------------------
// FGMRES (right preconditioned, restarted by the outer refinement) with the
// Hessenberg matrix, Givens rotations and the residual estimate on the device.
// --------------------------------------------------------------------------
// basis of up to 64 vectors; the Gram-Schmidt and update kernels take at most GM_PASS of them
// per launch (compile-time counts), so longer bases run as two passes
#define GM_MAXM 64
#define GM_PASS 32
struct GmPtrs { const void* p[GM_MAXM + 1]; };

// block partials of V_i . w for i = 0..NV-1 (classical Gram-Schmidt projections).
// NV is a compile-time count so every load of the unrolled loop is unconditional
// and independent (memory-level parallelism over all basis vectors).
// 16-byte packets: the padded layout's length is a multiple of 4 elements and every vector
// starts on a 256-byte boundary, so the Gram-Schmidt sweeps move whole packets
template <typename T> struct GmPack;
template <> struct GmPack<float> {
    using V = float4;
    static constexpr int W = 4;
    static __device__ __forceinline__ float at(const V& v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }
};
template <> struct GmPack<double> {
    using V = double2;
    static constexpr int W = 2;
    static __device__ __forceinline__ double at(const V& v, int q) { return q == 0 ? v.x : v.y; }
};

// h_ij = V_i . w for i < NV, and w . w (partials at NV nb + block)
template <typename T, int NV>
__global__ void __launch_bounds__(256) qk_gm_dots(long long n, GmPtrs V, const T* __restrict__ w,
                                                  double* __restrict__ part) {
    using PK = GmPack<T>;
    using PV = typename PK::V;
    float acc[NV];
    float accw = 0.f;
#pragma unroll
    for (int i = 0; i < NV; i++) acc[i] = 0.f;
    const PV* vp[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) vp[i] = (const PV*)V.p[i];
    const PV* wp = (const PV*)w;
    const long long np = n / PK::W;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < np; t += (long long)gridDim.x * blockDim.x) {
        const PV wv = wp[t];
        PV vv[NV];
#pragma unroll
        for (int i = 0; i < NV; i++) vv[i] = __ldg(vp[i] + t);
#pragma unroll
        for (int i = 0; i < NV; i++)
#pragma unroll
            for (int q = 0; q < PK::W; q++) acc[i] += (float)(PK::at(vv[i], q) * PK::at(wv, q));
#pragma unroll
        for (int q = 0; q < PK::W; q++) accw += (float)(PK::at(wv, q) * PK::at(wv, q));
    }
    __shared__ double sh[32];
#pragma unroll
    for (int i = 0; i < NV; i++) {
        double sum = qBlockSum(acc[i], sh);
        if (threadIdx.x == 0) part[(long long)i * gridDim.x + blockIdx.x] = sum;
    }
    const double sw = qBlockSum(accw, sh);
    if (threadIdx.x == 0) part[(long long)NV * gridDim.x + blockIdx.x] = sw;
}

// column j of H from the partials (h_ij = V_i . w), and the norm of the orthogonalised w from
// Pythagoras, |w'|^2 = |w|^2 - sum_i h_ij^2: when that keeps at least a hundredth of |w|^2 (no
// severe cancellation), Gm[4] = |w'| and Gm[3] = 1, and the orthogonalisation writes V_{j+1}
// = w' / |w'| directly (no norm pass over w', no scaling pass); otherwise Gm[3] = 0
__global__ void qk_gm_hcol(const double* __restrict__ part, long long nb, int j, int m, double* __restrict__ Hm,
                           double* __restrict__ Gm) {
    __shared__ double sh[32];
    double hh = 0.0;
    for (int i = 0; i <= j + 1; i++) {
        double acc = 0.0;
        for (long long t = threadIdx.x; t < nb; t += blockDim.x) acc += part[(long long)i * nb + t];
        double s = qBlockSum(acc, sh);
        if (threadIdx.x == 0) {
            if (i <= j) {
                Hm[i * m + j] = s;
                hh += s * s;
            } else {
                const double est = s - hh;
                const bool ok = isfinite(est) && est > 1e-2 * s;
                Gm[3] = ok ? 1.0 : 0.0;
                Gm[4] = ok ? sqrt(est) : 0.0;
            }
        }
    }
}

// w' = w - sum_i h_ij V_i (NV = j + 1, compile-time; 16-byte packets): with Gm[3] set, V_{j+1} =
// w' / Gm[4] goes to vout; otherwise w' back into w with the partials of |w'|^2
template <typename T, int NV>
// final = 0: a first pass over part of the basis (w' back into w, no norm partials, no direct write)
__global__ void __launch_bounds__(256) qk_gm_orth(long long n, int j, int m, GmPtrs V, const double* __restrict__ Hm,
                                                  T* __restrict__ w, double* __restrict__ part,
                                                  const double* __restrict__ Gm, T* __restrict__ vout, int final) {
    using PK = GmPack<T>;
    using PV = typename PK::V;
    T h[NV];
    const PV* vp[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) { h[i] = (T)Hm[i * m + j]; vp[i] = (const PV*)V.p[i]; }
    const bool direct = final && Gm[3] != 0.0;
    const T inv = direct ? (T)(1.0 / Gm[4]) : T(1);
    PV* wp = (PV*)w;
    PV* op = direct ? (PV*)vout : wp;
    const long long np = n / PK::W;
    float acc = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < np; t += (long long)gridDim.x * blockDim.x) {
        PV vv[NV];
#pragma unroll
        for (int i = 0; i < NV; i++) vv[i] = __ldg(vp[i] + t);
        PV wv = wp[t];
        T* wq = reinterpret_cast<T*>(&wv);
#pragma unroll
        for (int q = 0; q < PK::W; q++) {
            T a = wq[q];
#pragma unroll
            for (int i = 0; i < NV; i++) a -= h[i] * PK::at(vv[i], q);
            wq[q] = direct ? a * inv : a;
            acc += (float)(a * a);
        }
        op[t] = wv;
    }
    if (direct || !final) return;
    __shared__ double sh[32];
    double s0 = qBlockSum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s0;
}

// h_{j+1,j} = |w|, Givens rotations, residual estimate; Gm layout:
// [0]: beta, [1]: |g_{j+1}|, [2]: 1/h_{j+1,j}, cs[m] at 8, sn[m] at 8+m, g[m+1] at 8+2m
__global__ void qk_gm_givens(const double* __restrict__ part, long long nb, int j, int m, double* __restrict__ Hm,
                             double* __restrict__ Gm, unsigned* __restrict__ status) {
    __shared__ double sh[32];
    const bool direct = Gm[3] != 0.0;
    double acc = 0.0;
    if (!direct)
        for (long long t = threadIdx.x; t < nb; t += blockDim.x) acc += part[t];
    double nw = qBlockSum(acc, sh);
    if (threadIdx.x != 0) return;
    double hn = direct ? Gm[4] : sqrt(nw);
    double* cs = Gm + 8;
    double* sn = Gm + 8 + m;
    double* gv = Gm + 8 + 2 * m;
    Gm[2] = hn > 0.0 ? 1.0 / hn : 0.0;
    for (int i = 0; i < j; i++) {                // previous rotations on column j
        double a = Hm[i * m + j], b = Hm[(i + 1) * m + j];
        Hm[i * m + j] = cs[i] * a + sn[i] * b;
        Hm[(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
    }
    double a = Hm[j * m + j], b = hn;
    double r = sqrt(a * a + b * b);
    double c = r > 0.0 ? a / r : 1.0, s = r > 0.0 ? b / r : 0.0;
    cs[j] = c; sn[j] = s;
    Hm[j * m + j] = r;
    gv[j + 1] = -s * gv[j];
    gv[j] = c * gv[j];
    Gm[1] = fabs(gv[j + 1]);
    if (!(r > 0.0) || !isfinite(r)) atomicOr(status, (unsigned)QMS_ST_BREAKDOWN);
}

// V_{j+1} = w / h_{j+1,j} (nothing to do when the orthogonalisation wrote it, Gm[3])
template <typename T>
__global__ void qk_gm_scale(long long n, const T* __restrict__ w, T* __restrict__ vout, const double* __restrict__ Gm) {
    if (Gm[3] != 0.0) return;
    const T inv = (T)Gm[2];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        vout[t] = w[t] * inv;
}


__global__ void qk_gm_reset(int m, double* __restrict__ Gm) {
    for (int q = threadIdx.x; q < 8 + 3 * m + 1; q += blockDim.x) Gm[q] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0) { Gm[0] = 1.0; Gm[8 + 2 * m] = 1.0; Gm[1] = 1.0; }
}

// back substitution H(0:k,0:k) y = g(0:k); y stored at Gm + 8 + 3m + 1
__global__ void qk_gm_solve(int k, int m, const double* __restrict__ Hm, double* __restrict__ Gm) {
    if (threadIdx.x != 0) return;
    const double* gv = Gm + 8 + 2 * m;
    double* y = Gm + 8 + 3 * m + 1;
    for (int i = k - 1; i >= 0; i--) {
        double acc = gv[i];
        for (int q = i + 1; q < k; q++) acc -= Hm[i * m + q] * y[q];
        const double d = Hm[i * m + i];
        y[i] = d != 0.0 ? acc / d : 0.0;
    }
}

// x[ref] += nrm * sum_i y_i Z_i[PL]   (FP64 accumulation of the refinement); one thread per
// node, its (up to) four unknowns
template <typename T, int NV>
__global__ void __launch_bounds__(QMS_NODE_BX * QMS_NODE_BY) qk_gm_update(QGrid g, int m, GmPtrs Z, const double* __restrict__ Gm,
                                                    const double* __restrict__ S, double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const double* yv = Gm + 8 + 3 * m + 1;
    T y[NV];
    const T* zp[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) { y[q] = (T)yv[q]; zp[q] = (const T*)Z.p[q]; }
    const double nr = S[S_NRM];
    const QPL L = qms_pl(g);
    const long long nd = qms_pl_node(g, L, i, j, k);
    auto comb = [&](long long t) {
        T acc = T(0);
#pragma unroll
        for (int q = 0; q < NV; q++) acc += y[q] * __ldg(zp[q] + t);
        return nr * (double)acc;
    };
    if (i <= g.xs) x[qAX(g, i, j, k)] += comb(nd);
    if (j <= g.ys) x[qAY(g, i, j, k)] += comb(L.comp + nd);
    if (k <= g.zs) x[qAZ(g, i, j, k)] += comb(2 * L.comp + nd);
    x[qV(g, i, j, k)] += comb(3 * L.comp + nd);
}

// compile-time dispatch on the number of basis vectors (1..GM_MAXM)
#define GM_CASES(M) M(1) M(2) M(3) M(4) M(5) M(6) M(7) M(8) M(9) M(10) M(11) M(12) M(13) M(14) M(15) M(16) \
    M(17) M(18) M(19) M(20) M(21) M(22) M(23) M(24) M(25) M(26) M(27) M(28) M(29) M(30) M(31) M(32)

static GmPtrs gm_shift(const GmPtrs& V, int off) {
    GmPtrs r{};
    for (int i = 0; i + off <= GM_MAXM; i++) r.p[i] = V.p[i + off];
    return r;
}
// returns the kernel launches
template <typename T>
static int gm_dots(int nv, int vb, cudaStream_t st, long long n, const GmPtrs& V, const T* w, double* part) {
    if (nv > GM_PASS) {
        // the first GM_PASS projections, then the rest (whose |w|^2 partials land at nv * vb)
        gm_dots<T>(GM_PASS, vb, st, n, V, w, part);
        return 1 + gm_dots<T>(nv - GM_PASS, vb, st, n, gm_shift(V, GM_PASS), w, part + (long long)GM_PASS * vb);
    }
    switch (nv) {
#define C(N) case N: qk_gm_dots<T, N><<<vb, 256, 0, st>>>(n, V, w, part); break;
        GM_CASES(C)
#undef C
    }
    return 1;
}
template <typename T>
static int gm_orth(int nv, int vb, cudaStream_t st, long long n, int j, int m, const GmPtrs& V, const double* Hm, T* w,
                   double* part, const double* Gm, T* vout, int final = 1) {
    if (nv > GM_PASS) {
        gm_orth<T>(GM_PASS, vb, st, n, j, m, V, Hm, w, part, Gm, vout, 0);
        return 1 + gm_orth<T>(nv - GM_PASS, vb, st, n, j, m, gm_shift(V, GM_PASS), Hm + (long long)GM_PASS * m, w,
                              part, Gm, vout, final);
    }
    switch (nv) {
#define C(N) case N: qk_gm_orth<T, N><<<vb, 256, 0, st>>>(n, j, m, V, Hm, w, part, Gm, vout, final); break;
        GM_CASES(C)
#undef C
    }
    return 1;
}
template <typename T>
static int gm_update(int nv, cudaStream_t st, const QGrid& g, int m, const GmPtrs& Z, const double* Gm,
                     const double* S, double* x) {
    if (nv > GM_PASS) {
        // x += nr (sum of the first GM_PASS terms) + nr (the rest): the y of the second pass start
        // GM_PASS further into Gm
        gm_update<T>(GM_PASS, st, g, m, Z, Gm, S, x);
        return 1 + gm_update<T>(nv - GM_PASS, st, g, m, gm_shift(Z, GM_PASS), Gm + GM_PASS, S, x);
    }
    switch (nv) {
#define C(N) case N: qk_gm_update<T, N><<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, m, Z, Gm, S, x); break;
        GM_CASES(C)
#undef C
    }
    return 1;
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
    mgf[0].release(); mgf[1].release(); mgd[0].release(); mgd[1].release();
    for (auto& p : gmV) { if (p) cudaFree(p); p = nullptr; }
    for (auto& p : gmZ) { if (p) cudaFree(p); p = nullptr; }
    if (gm_H) cudaFree(gm_H);
    if (gm_scal) cudaFree(gm_scal);
    gm_H = gm_scal = nullptr;
    if (nc16) cudaFree(nc16);
    nc16 = nullptr;
    void* ptrs[] = {ids,   dtab64, dtab32,    x,     b,      r64,    xbest, H,   slicebuf, part,   S,
                    status, dg_steady, dg_tr, mgtmp, mgtmp2, nc32,  nc64,  xdf, r0df,     ncdf, rpl, x0,
                    rsg,   rsdt,   bprev,     rfin,  dinvdf, xold, xold2, hist_x, xold3, wh[0], wh[1], wh[2],
                    wh[3], xold4, lsp, lsg};
    for (void* q : ptrs) if (q) cudaFree(q);
    if (hS) cudaFreeHost(hS);
    if (hptrs) cudaFreeHost(hptrs);
    if (dptrs) cudaFree(dptrs);
    hptrs = nullptr;
    dptrs = nullptr;
    for (auto& p : vec) if (p) cudaFree(p);
    drop_graphs();
    for (auto& e : evpool) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    evpool.clear();
    for (int q = 0; q < kFieldSlots; q++) {
        if (fev_done[q]) cudaEventSynchronize(fev_done[q]);
        if (fev_ready[q]) cudaEventDestroy(fev_ready[q]);
        if (fev_done[q]) cudaEventDestroy(fev_done[q]);
        if (fbuf[q]) cudaFree(fbuf[q]);
        fev_ready[q] = fev_done[q] = nullptr;
        fbuf[q] = nullptr;
        fbuf_n[q] = 0;
    }
    if (cst) cudaStreamDestroy(cst);
    cst = nullptr;
    if (st && own_stream) cudaStreamDestroy(st);
    ids = nullptr; dtab64 = nullptr; dtab32 = nullptr; x = b = r64 = H = slicebuf = part = S = nullptr;
    status = nullptr; dg_steady = dg_tr = nullptr; hS = nullptr; st = nullptr; mgtmp = nullptr; mgtmp2 = nullptr; xbest = nullptr;
    xdf = r0df = ncdf = nullptr; rpl = nullptr; x0 = nullptr; df_resid = false; anchor_ready = false;
    rsg = rsdt = nullptr;
    bprev = nullptr; rfin = dinvdf = nullptr; rfin_ok = false; chain_len = 0; xold = xold2 = nullptr;
    hist_x = nullptr; hist_len = 0; xold3 = xold4 = nullptr; wh[0] = wh[1] = wh[2] = wh[3] = nullptr; w_len = 0;
    nwh = 0; lsp = lsg = nullptr; last_chained = false;
    field_run = 0; start_resid_ready = false;
    nc32 = nullptr; nc64 = nullptr;
    for (auto& p : vec) p = nullptr;
}

int QmsSolver::init(const qms_desc& d) {
    desc = d;
    mghook.s = this;
    for (int q = 0; q < 2; q++) { mgf[q].prof = &mghook; mgd[q].prof = &mghook; }
    dev = d.device;
    CK(cudaSetDevice(dev));
    if (d.xs < 4 || d.ys < 4 || d.zs < 4) { err = "grid must have at least 4 cells per axis"; return QMS_ERR_ARG; }
    if (!(d.dx > 0 && d.dy > 0 && d.dz > 0 && d.dt > 0)) { err = "dx, dy, dz, dt must be positive"; return QMS_ERR_ARG; }
    g = qms_make_grid(d.xs, d.ys, d.zs, d.dx, d.dy, d.dz);
    // the stencil kernels index rows with 32-bit integers (and the padded layout is a little larger)
    npl = qms_pl(g).n;
    if (g.n >= 0x7fffffffLL || npl >= 0x7fffffffLL) {
        err = "grid too large: more than 2^31 - 1 unknowns";
        return QMS_ERR_ARG;
    }
    fp64_inner = d.precision == QMS_PREC_FP64;
    trace = std::getenv("QMS_TRACE") != nullptr;
    tsize = fp64_inner ? sizeof(double) : sizeof(float);
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    vec_blocks = (long long)nsm * 8;
    long long need = (npl + 255) / 256;
    if (need < vec_blocks) vec_blocks = need;
    nbop = qms_op_num_blocks(g);
    long long npart = std::max(4 * nbop, (long long)(GM_MAXM + 1) * vec_blocks) + 64;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    own_stream = true;
    const long long n = g.n, ncell = (long long)g.xs * g.ys * g.zs;
    CK(cudaMalloc(&ids, ncell));
    CK(cudaMemsetAsync(ids, 0, ncell, st));
    CK(cudaMalloc(&dtab64, sizeof(QMatTable<double>)));
    CK(cudaMalloc(&dtab32, sizeof(QMatTable<float>)));
    CK(cudaMalloc(&x, n * 8));
    CK(cudaMalloc(&b, n * 8));
    CK(cudaMalloc(&r64, n * 8));
    CK(cudaMalloc(&xbest, n * 8));
    CK(cudaMalloc(&H, 3 * ncell * 8));
    long long smax = std::max({(long long)g.ys * g.zs, (long long)g.xs * g.zs, (long long)g.xs * g.ys});
    CK(cudaMalloc(&slicebuf, 3 * smax * 8));
    CK(cudaMalloc(&part, npart * 8));
    CK(cudaMalloc(&S, S_COUNT * 8));
    CK(cudaMemsetAsync(S, 0, S_COUNT * 8, st));
    CK(cudaMalloc(&status, sizeof(unsigned)));
    CK(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
    CK(cudaMalloc(&nc32, 6 * qms_pl(g).comp * 4));
    CK(cudaMalloc(&nc64, 6 * qms_pl(g).comp * 8));
    // inner-solver vectors in the padded layout; the padding stays zero
    auto pl_alloc = [&](void** p, size_t es) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, npl * es);
        return e != cudaSuccess ? e : cudaMemsetAsync(*p, 0, npl * es, st);
    };
    CK(pl_alloc((void**)&dg_steady, 4));
    CK(pl_alloc((void**)&dg_tr, 4));
    for (auto& p : vec) CK(pl_alloc(&p, tsize));
    // multigrid needs at least two levels (grids of a few cells use the Jacobi / identity fallback)
    use_mg = d.precond == QMS_PRECOND_MG && QmsMG<float>::levels_for(g, 5) >= 2;
    CK(pl_alloc((void**)&mgtmp, tsize));
    if (use_mg) CK(pl_alloc((void**)&mgtmp2, tsize));
    if (d.krylov == QMS_KRYLOV_GMRES) {
        const int m = std::min(std::max(d.gmres_m, 1), GM_MAXM);
        desc.gmres_m = m;
        for (int i = 0; i <= m; i++) CK(pl_alloc(&gmV[i], tsize));
        if (use_mg) for (int i = 0; i < m; i++) CK(pl_alloc(&gmZ[i], tsize));
        CK(cudaMalloc(&gm_H, (size_t)m * (m + 1) * 8));
        CK(cudaMalloc(&gm_scal, (size_t)(8 + 4 * m + 8) * 8));
    }
    CK(cudaMallocHost(&hS, S_COUNT * 8));
    CK(cudaMemsetAsync(x, 0, n * 8, st));
    // tensor maps of every padded vector that feeds a stencil kernel, and of the coefficients
    std::vector<const void*> mapped(vec, vec + QMS_NVEC);
    mapped.push_back(mgtmp);
    for (int i = 0; i <= GM_MAXM; i++) if (gmV[i]) mapped.push_back(gmV[i]);
    for (int i = 0; i < GM_MAXM; i++) if (gmZ[i]) mapped.push_back(gmZ[i]);
    if (mgtmp2) mapped.push_back(mgtmp2);
    if (!fp64_inner) {
        df_resid = true;
        CK(pl_alloc((void**)&xdf, 8));
        CK(pl_alloc((void**)&r0df, 8));
        CK(cudaMalloc(&rsg, g.oV * 8));
        CK(cudaMalloc(&rsdt, g.oV * 8));
        CK(cudaMalloc(&bprev, n * 8));
        CK(cudaMalloc(&xold, n * 8));
        CK(cudaMalloc(&hist_x, n * 8));
        const int hx_need = std::max(std::min(d.extrapolate, 3), d.start_ls);   // history beyond x_n, x_(n-1)
        if (hx_need >= 2) CK(cudaMalloc(&xold2, n * 8));
        if (hx_need >= 3) CK(cudaMalloc(&xold3, n * 8));
        if (hx_need >= 4) CK(cudaMalloc(&xold4, n * 8));
        nwh = hx_need;
        for (int q = 0; q < nwh; q++) CK(pl_alloc((void**)&wh[q], 8));
        if (d.start_ls > 0) {
            CK(cudaMalloc(&lsp, (size_t)QMS_LS_SUMS * nbop * 8));
            CK(cudaMalloc(&lsg, 8 * 8));
        }
        CK(pl_alloc((void**)&rfin, 8));
        CK(pl_alloc((void**)&dinvdf, 8));
        CK(cudaMalloc(&x0, n * 8));
        CK(pl_alloc((void**)&rpl, 4));
        CK(cudaMallocHost(&hptrs, sizeof(QStepPtrs)));
        CK(cudaMalloc(&dptrs, sizeof(QStepPtrs)));
        CK(cudaMalloc(&ncdf, 6 * qms_pl(g).comp * 8));
        CK(cudaMemsetAsync(ncdf, 0, 6 * qms_pl(g).comp * 8, st));
        if (!qms_make_pl_map(&xdfmap, xdf, g, 8, 4, PLXY) || !qms_make_pl_map(&cdfmap, ncdf, g, 8, 6, PLCY)) {
            err = "tensor map encoding failed";
            return QMS_ERR_CUDA;
        }
    }
    const long long vbytes = 3 * qms_pl(g).comp * (long long)tsize;   // offset of the V block
    for (const void* p : mapped) {
        CUtensorMap mp, ma, mv;
        if (!qms_make_pl_map(&mp, p, g, (int)tsize, 4, PLXY) || !qms_make_pl_map(&ma, p, g, (int)tsize, 3, PLXY) ||
            !qms_make_pl_map(&mv, (const char*)p + vbytes, g, (int)tsize, 1, PLXY)) {
            err = "tensor map encoding failed";
            return QMS_ERR_CUDA;
        }
        tmaps[p] = mp;
        tmapsA[p] = ma;
        tmapsV[p] = mv;
    }
    if (!fp64_inner) {
        const long long comp16 = (long long)qms_pl16_pitch(g) * g.Ny * g.Nz;
        CK(cudaMalloc(&nc16, 6 * comp16 * sizeof(__nv_bfloat16)));
        if (!qms_make_pl16_map(&cmap16, nc16, g, 6) || !qms_make_pl16_map(&cmapV16, nc16 + 3 * comp16, g, 3)) {
            err = "tensor map encoding failed";
            return QMS_ERR_CUDA;
        }
    }
    const long long cv = 3 * qms_pl(g).comp;                          // first conductivity array
    if (!qms_make_pl_map(&cmap32, nc32, g, 4, 6, PLCY) || !qms_make_pl_map(&cmap64, nc64, g, 8, 6, PLCY) ||
        !qms_make_pl_map(&cmapV32, nc32 + cv, g, 4, 3, PLCY) || !qms_make_pl_map(&cmapV64, nc64 + cv, g, 8, 3, PLCY)) {
        err = "tensor map encoding failed";
        return QMS_ERR_CUDA;
    }
    double vac[6] = {1, 1, 1, 0, 0, 0};
    return set_materials(nullptr, vac, 0);
}

size_t qms_device_bytes_impl(const qms_desc& d) {
    QGrid g = qms_make_grid(d.xs, d.ys, d.zs, d.dx, d.dy, d.dz);
    size_t ts = d.precision == QMS_PREC_FP64 ? 8 : 4;
    // the block-triangular preconditioner's V right-hand side; the double-float residual's x, b,
    // coefficients and FP32 result (mixed precision)
    size_t tri = d.precond == QMS_PRECOND_MG ? qms_pl(g).n * ts : 0;
    // history of the extrapolated and least-squares starts: x_(n-2).. and the residual images
    const int lsn = std::max(0, std::min(d.start_ls, 4));
    const size_t hxn = (size_t)std::max(std::max(0, std::min(d.extrapolate, 3)), lsn);
    if (ts == 4) tri += (size_t)6 * qms_pl16_pitch(g) * g.Ny * g.Nz * 2;       // bf16 node coefficients
    if (ts == 4) tri += qms_pl(g).n * (8 + 8 + 4 + 8 + 8) + 6 * qms_pl(g).comp * 8 + 5 * g.n * 8 + 2 * g.oV * 8 +
                        (hxn > 2 ? hxn - 2 : 0) * g.n * 8 + hxn * qms_pl(g).n * 8 +
                        (lsn > 0 ? (QMS_LS_SUMS * (size_t)qms_op_num_blocks(g) + 8) * 8 : 0);
    size_t ncell = (size_t)g.xs * g.ys * g.zs;
    size_t smax = std::max({(size_t)g.ys * g.zs, (size_t)g.xs * g.zs, (size_t)g.xs * g.ys});
    size_t nb = (size_t)qms_op_num_blocks(g);
    return tri + ncell + sizeof(QMatTable<double>) + sizeof(QMatTable<float>) + 4 * g.n * 8 + 3 * ncell * 8 +
           6 * qms_pl(g).comp * 12 +
           3 * smax * 8 + (4 * nb + 64) * 8 + 2 * qms_pl(g).n * 4 + (QMS_NVEC + 1) * qms_pl(g).n * ts + 4096 +
           (d.krylov == QMS_KRYLOV_GMRES ? (size_t)(2 * d.gmres_m + 1) * qms_pl(g).n * ts : 0) +
           (d.precond == QMS_PRECOND_MG ? 2 * (ts == 8 ? QmsMG<double>::bytes_for(g, 5, true) : QmsMG<float>::bytes_for(g, 5, true)) : 0) +
           // conductor-region coarse space: node lists (at most every node) and the K x K pseudo-inverse
           (d.precond == QMS_PRECOND_MG ? (size_t)g.Nn * 8 + (size_t)QMS_REGION_MAX * QMS_REGION_MAX * 8 + 64 * 1024 : 0);
}

int QmsSolver::set_materials(const uint8_t* host_slots, const double* rows6, int nmat) {
    CK(cudaSetDevice(dev));
    drop_graphs();
    gm_k_est = 0;
    gm_k_seen = 0;
    gm_lrate[0] = gm_lrate[1] = 0.0;
    gm_k_fine = false;
    gm_k_floor = 0;
    gm_k_floor_age = 0;
    gm_ls_floor = 0;
    gm_ls_floor_age = 0;
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
    // node coefficients, then the Jacobi diagonals (velocity does not enter the diagonal)
    qms_launch_node_coef<float>(g, coef32(), nc32, st);
    qms_launch_node_coef<double>(g, coef64(), nc64, st);
    if (nc16) qms_launch_coef_bf16(g, nc32, nc16, st);
    if (df_resid) qms_launch_split_flat(6 * qms_pl(g).comp, nc64, ncdf, st);
    if (rsg) qms_launch_rhs_coef(g, ids, dtab64, desc.dt, rsg, rsdt, st);
    if (dinvdf) qms_launch_dinv_df(g, coef64(), qms_step_par<double>(g, 0, 0, 0, desc.dt, true), dinvdf, st);
    rfin_ok = false;
    hist_len = 0;
    w_len = 0;
    last_chained = false;
    QCoef<float> c32 = coef32();
    qms_launch_diag_pl(g, c32, qms_step_par<float>(g, 0, 0, 0, desc.dt, false), dg_steady, st);
    qms_launch_diag_pl(g, c32, qms_step_par<float>(g, 0, 0, 0, desc.dt, true), dg_tr, st);
    CK(cudaGetLastError());
    if (use_mg) {
        const double vshift = desc.mg_vshift;
        for (int tr = 0; tr < 2; tr++) {
            int rc;
            if (fp64_inner) {
                QmsMG<double>& M = mgd[tr];
                M.nu1 = M.nu2 = desc.mg_sweeps; M.omega = desc.mg_omega; M.alpha = desc.mg_alpha;
                M.nu_coarse = desc.mg_coarse_sweeps;
                M.nu_v = desc.mg_v_sweeps;
                M.tail_points = desc.mg_tail_points == 0 ? 4096 : std::max(0, desc.mg_tail_points);
                M.vcut = desc.mg_v_coarse_cut;
                rc = M.build(g, coef64(), qms_step_par<double>(g, 0, 0, 0, desc.dt, tr == 1), vshift, st);
                if (rc) { err = M.err; return QMS_ERR_CUDA; }
            } else {
                QmsMG<float>& M = mgf[tr];
                M.nu1 = M.nu2 = desc.mg_sweeps; M.omega = (float)desc.mg_omega; M.alpha = (float)desc.mg_alpha;
                M.nu_coarse = desc.mg_coarse_sweeps;
                M.nu_v = desc.mg_v_sweeps;
                M.tail_points = desc.mg_tail_points == 0 ? 4096 : std::max(0, desc.mg_tail_points);
                M.vcut = desc.mg_v_coarse_cut;
                rc = M.build(g, coef32(), qms_step_par<float>(g, 0, 0, 0, desc.dt, tr == 1), (float)vshift, st);
                if (rc) { err = M.err; return QMS_ERR_CUDA; }
            }
        }
    }
    regions.release();
    if (use_mg) {
        // the region space needs the slots on the host
        std::vector<uint8_t> hslots;
        const uint8_t* sl = host_slots;
        if (!sl) {
            hslots.resize(ncell);
            CK(cudaMemcpyAsync(hslots.data(), ids, ncell, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            sl = hslots.data();
        }
        const double cut = desc.mg_region_cut != 0.0 ? desc.mg_region_cut : (fp64_inner ? 1e-9 : 1e-6);
        if (cut > 0.0 && regions.build(g, sl, rows6, nmat, desc.mg_vshift, cut, st)) {
            err = regions.err;
            return QMS_ERR_CUDA;
        }
    }
    CK(cudaStreamSynchronize(st));
    return 0;
}

QCoef<float> QmsSolver::coef32() const { return QCoef<float>{g, ids, dtab32, (float)(1.0 / QMS_MU0), nc32}; }
QCoef<double> QmsSolver::coef64() const { return QCoef<double>{g, ids, dtab64, 1.0 / QMS_MU0, nc64}; }

int QmsSolver::finalize(int fop, int nsum, long long nb) {
    qk_finalize<<<1, 512, 0, st>>>(part, nb, nsum, S, fop, status);
    nlaunch++;
    return 0;
}

template <typename T>
void QmsSolver::op(bool adv, int mode, const QStepPar<T>& P, const T* xin, const T* bin, T* y, const T* w,
                   double* partials) {
    const double ncell = (double)g.xs * g.ys * g.zs;
    // the reference-layout operator serves the FP64 refinement residual (profile kind 3)
    OpEv* ev = prof_begin(mode == QOPH_RESID ? 3 : (sizeof(T) == 8 ? 1 : 0),
                          (double)g.n * sizeof(T) * (2 + (w && w != xin ? 1 : 0) + (bin ? 1 : 0)) + ncell);
    qms_launch_operator<T>(g, coef<T>(), P, adv, mode, xin, bin, y, w, partials, st);
    nlaunch++;
    prof_end(ev);
}
template void QmsSolver::op<float>(bool, int, const QStepPar<float>&, const float*, const float*, float*,
                                   const float*, double*);

const CUtensorMap& QmsSolver::tmap(const void* p) const { return tmaps.at(p); }
const CUtensorMap& QmsSolver::tmapq(const void* p, int qs) const {
    return qs == 1 ? tmapsA.at(p) : (qs == 2 ? tmapsV.at(p) : tmaps.at(p));
}

template <typename T>
void QmsSolver::op_pl(bool adv, int mode, const QStepPar<T>& P, const T* xin, T* y, const T* w, double* partials) {
    const double ncell = (double)g.xs * g.ys * g.zs;
    OpEv* ev = prof_begin(sizeof(T) == 8 ? 1 : 0, (double)g.n * sizeof(T) * (2 + (w && w != xin ? 1 : 0)) + ncell);
    qms_launch_op_pl<T>(g, P, tmap(xin), sizeof(T) == 8 ? cmap64 : cmap32, adv, mode, y, w, partials, status, st);
    nlaunch++;
    prof_end(ev);
}
template void QmsSolver::op_pl<float>(bool, int, const QStepPar<float>&, const float*, float*, const float*, double*);
template void QmsSolver::op_pl<double>(bool, int, const QStepPar<double>&, const double*, double*, const double*,
                                       double*);
template void QmsSolver::op<double>(bool, int, const QStepPar<double>&, const double*, const double*, double*,
                                    const double*, double*);

QmsSolver::OpEv* QmsSolver::prof_begin(int kind, double bytes) {
    if (!prof) return nullptr;
    if (evused == evpool.size()) {
        OpEv e{};
        cudaEventCreate(&e.a);
        cudaEventCreate(&e.b);
        evpool.push_back(e);
    }
    OpEv* ev = &evpool[evused++];
    ev->kind = kind;
    ev->bytes = bytes;
    // inside a capture the record must become an event-record node of the graph
    cudaEventRecordWithFlags(ev->a, st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    return ev;
}

void QmsSolver::prof_end(OpEv* ev) {
    if (ev) cudaEventRecordWithFlags(ev->b, st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
}

bool QmsSolver::prof_accum(const OpEv& e) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e.a, e.b) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (e.kind == 1) { profacc.op64_launches++; profacc.op64_ms += ms; profacc.op64_bytes += e.bytes; }
    else if (e.kind == 0) { profacc.op32_launches++; profacc.op32_ms += ms; profacc.op32_bytes += e.bytes; }
    else if (e.kind == 3) { profacc.resid_launches++; profacc.resid_ms += ms; profacc.resid_bytes += e.bytes; }
    else if (e.kind == MGPROF_A_SWEEP) { profacc.mg0a_launches++; profacc.mg0a_ms += ms; profacc.mg0a_bytes += e.bytes; }
    else { profacc.mg_cycles++; profacc.mg_ms += ms; }
    return true;
}

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
    for (size_t q = 0; q < evused; q++)
        if (!prof_accum(evpool[q])) { err = "profile events could not be timed"; return QMS_ERR_CUDA; }
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
void QmsSolver::precond(const T* r, const float* bscale, T* z, bool mask_v, bool transient, bool jacobi_pcg,
                        const QStepPar<T>* P, bool adv) {
    if (use_mg) {
        OpEv* ev = prof_begin(2, 0.0);
        const bool f32 = sizeof(T) == 4;
        // the cycles' level-0 tiles read the bf16 coefficients in an FP32 hierarchy
        const CUtensorMap& cm = f32 ? cmap16 : cmap64;
        auto cycle = [&](const T* b, int qs, const CUtensorMap& cmq) {
            // b's own tile map for the fused first sweeps of the subset cycles (a mapped vector)
            const CUtensorMap* bm = nullptr;
            if (qs != 0) {
                auto& tm = qs == 1 ? tmapsA : tmapsV;
                auto it = tm.find((const void*)b);
                if (it != tm.end()) bm = &it->second;
            }
            if (f32)
                nlaunch += mgf[transient ? 1 : 0].vcycle((const float*)b, bscale != nullptr, (float*)z, tmapq(z, qs),
                                                         mgtmp, tmapq(mgtmp, qs), cmq, mask_v, status, st, qs, bm);
            else
                nlaunch += mgd[transient ? 1 : 0].vcycle((const double*)b, bscale != nullptr, (double*)z,
                                                         tmapq(z, qs), (double*)mgtmp, tmapq(mgtmp, qs), cmq, mask_v,
                                                         status, st, qs);
        };
        if (P && !mask_v && bscale && desc.mg_coupling == 1) {
            // lower block-triangular: the A blocks first, then the V block on the residual that
            // the A correction leaves in the V rows (row-scaled like r)
            T* tv = (T*)mgtmp2;
            cycle(r, 1, cm);
            qms_launch_op_pl<T>(g, *P, tmapq(z, 1), f32 ? cmapV32 : cmapV64, adv, QOPH_VCOUPLE, tv, r, nullptr,
                                status, st);
            cycle(tv, 2, f32 ? cmapV16 : cmapV64);
            nlaunch++;
            regions.apply<T>(tv, bscale, z, st, nlaunch);
        } else {
            cycle(r, 0, cm);
            if (!mask_v) regions.apply<T>(r, bscale, z, st, nlaunch);
        }
        prof_end(ev);
    } else if (jacobi_pcg) {
        qk_jacobi<T><<<(int)vec_blocks, 256, 0, st>>>(npl, mask_v ? 3 * qms_pl(g).comp : npl, r,
                                                        transient ? dg_tr : dg_steady, z);
        nlaunch++;
    }
}

template <typename T>
int QmsSolver::inner_bicgstab(bool adv, bool transient, const double v[3], int& iters) {
    const long long n = npl;
    T* r = (T*)vec[0]; T* rh = (T*)vec[1]; T* p = (T*)vec[2]; T* vv = (T*)vec[3];
    T* s = (T*)vec[4]; T* t = (T*)vec[5]; T* e = (T*)vec[6];
    // right preconditioner of the row-scaled operator D^-1 M: y = MG(D p); identity without MG
    T* y = use_mg ? (T*)vec[7] : p;
    T* z = use_mg ? (T*)vec[8] : s;
    const float* dg = transient ? dg_tr : dg_steady;
    QStepPar<T> P = qms_step_par<T>(g, v[0], v[1], v[2], desc.dt, transient);
    const int vb = (int)vec_blocks;
    resid_to_inner<T>(r);
    qk_bicg_init<T><<<vb, 256, 0, st>>>(n, r, rh, p, vv, e, part);
    nlaunch++;
    finalize(FIN_BICG_INIT, 1, vec_blocks);
    const double tol2 = desc.inner_rtol * desc.inner_rtol;
    iters = 0;
    for (int it = 0; it < desc.max_inner; it++) {
        qk_bicg_p<T><<<vb, 256, 0, st>>>(n, r, p, vv, S);
        nlaunch++;
        if (use_mg) precond<T>(p, dg, y, false, transient, false, &P, adv);
        op_pl<T>(adv, QOPH_SCALED, P, y, vv, rh, part);
        finalize(FIN_BICG_ALPHA, 1, nbop);
        qk_bicg_s<T><<<vb, 256, 0, st>>>(n, r, vv, s, S);
        nlaunch++;
        if (use_mg) precond<T>(s, dg, z, false, transient, false, &P, adv);
        op_pl<T>(adv, QOPH_SCALED, P, z, t, s, part);
        finalize(FIN_BICG_OMEGA, 2, nbop);
        qk_bicg_xr<T><<<vb, 256, 0, st>>>(n, y, z, s, t, rh, e, r, S, part);
        nlaunch++;
        finalize(FIN_BICG_RHO, 2, vec_blocks);
        iters = it + 1;
        if ((it + 1) % desc.check_every == 0 || it + 1 == desc.max_inner) {
            int rc = read_scalars();
            if (rc) return rc;
            if (!(hS[S_RR] <= tol2 * hS[S_RR0])) {
                unsigned stt = 0;
                CK(cudaMemcpyAsync(&stt, status, 4, cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (stt & QMS_ST_BREAKDOWN) break;
                continue;
            }
            break;
        }
    }
    qms_launch_ref_add_pl<T>(g, e, S + S_NRM, x, st);
    nlaunch++;
    CK(cudaGetLastError());
    return 0;
}


template <typename T>
int QmsSolver::inner_gmres(bool adv, bool transient, const double v[3], int& iters, int fixed_k) {
    const long long n = npl;
    const int m = std::min(desc.gmres_m, GM_MAXM);
    const int kmax = fixed_k > 0 ? std::min(fixed_k, m) : m;
    const float* dg = transient ? dg_tr : dg_steady;
    QStepPar<T> P = qms_step_par<T>(g, v[0], v[1], v[2], desc.dt, transient);
    const int vb = (int)vec_blocks;
    GmPtrs Vp{}, Zp{};
    for (int i = 0; i <= m; i++) Vp.p[i] = gmV[i];
    for (int i = 0; i < m; i++) Zp.p[i] = use_mg ? gmZ[i] : gmV[i];
    T* w = (T*)vec[0];
    qk_gm_reset<<<1, 128, 0, st>>>(m, gm_scal);
    resid_to_inner<T>((T*)gmV[0]);
    nlaunch++;
    const double tol = desc.inner_rtol;
    int k = 0;
    for (int j = 0; j < kmax; j++) {
        T* vj = (T*)gmV[j];
        T* zj = use_mg ? (T*)gmZ[j] : vj;
        if (use_mg) precond<T>(vj, dg, zj, false, transient, false, &P, adv);
        op_pl<T>(adv, QOPH_SCALED, P, zj, w, nullptr, nullptr);
        nlaunch += gm_dots<T>(j + 1, vb, st, n, Vp, w, part);
        qk_gm_hcol<<<1, 512, 0, st>>>(part, vec_blocks, j, m, gm_H, gm_scal);
        nlaunch += gm_orth<T>(j + 1, vb, st, n, j, m, Vp, gm_H, w, part, gm_scal, (T*)gmV[j + 1]);
        qk_gm_givens<<<1, 512, 0, st>>>(part, vec_blocks, j, m, gm_H, gm_scal, status);
        qk_gm_scale<T><<<vb, 256, 0, st>>>(n, w, (T*)gmV[j + 1], gm_scal);
        nlaunch += 3;
        k = j + 1;
        if (fixed_k <= 0 && ((j + 1) % desc.check_every == 0 || j + 1 == m)) {
            CK(cudaMemcpyAsync(hS, gm_scal, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (!(hS[1] > tol * hS[0])) break;       // also stops on a non-finite estimate
        }
    }
    qk_gm_solve<<<1, 32, 0, st>>>(k, m, gm_H, gm_scal);
    nlaunch += 1 + gm_update<T>(k, st, g, m, Zp, gm_scal, S, x);
    last_gm_k = k;
    iters = k;
    CK(cudaGetLastError());
    return 0;
}


template <typename T>
int QmsSolver::inner_pcg(bool transient, int& iters) {
    const long long n = npl;
    T* r = (T*)vec[0]; T* z = (T*)vec[1]; T* p = (T*)vec[2]; T* q = (T*)vec[3]; T* e = (T*)vec[6];
    const float* dg = transient ? dg_tr : dg_steady;
    QStepPar<T> P = qms_step_par<T>(g, 0, 0, 0, desc.dt, transient);
    const int vb = (int)vec_blocks;
    // V block frozen at zero: the steady magnetostatic system with v = 0 has V = 0
    resid_to_inner<T>(r);
    qk_cg_init<T><<<vb, 256, 0, st>>>(n, dg, r, e);
    nlaunch++;
    precond<T>(r, nullptr, z, true, transient, true);
    qk_cg_dot<T><<<vb, 256, 0, st>>>(n, r, z, p, part);
    nlaunch++;
    finalize(FIN_CG_INIT, 2, vec_blocks);
    const double tol2 = desc.inner_rtol * desc.inner_rtol;
    iters = 0;
    for (int it = 0; it < desc.max_inner; it++) {
        op_pl<T>(false, QOPH_APPLY, P, p, q, p, part);
        finalize(FIN_CG_ALPHA, 1, nbop);
        qk_cg_update<T><<<vb, 256, 0, st>>>(n, p, q, S, e, r);
        nlaunch++;
        precond<T>(r, nullptr, z, true, transient, true);
        qk_cg_dot<T><<<vb, 256, 0, st>>>(n, r, z, (T*)nullptr, part);
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
    qms_launch_ref_add_pl<T>(g, e, S + S_NRM, x, st);
    nlaunch++;
    CK(cudaGetLastError());
    return 0;
}

int QmsSolver::residual_launch(bool adv, bool transient, const double v[3], bool exact) {
    if (start_resid_ready && !exact) {
        // the step start (qk_step_start) formed this residual and its partials
        start_resid_ready = false;
        last_resid_df = true;
        finalize(FIN_RESID, 4, nbop);
        return 0;
    } else if (df_resid && anchor_ready && anchor_is_residual && !exact) {
        // x is the anchor state: the residual is the anchor's
        OpEv* ev = prof_begin(3, (double)g.n * 8 * 3);
        qms_launch_anchor_resid(g, r0df, x, rpl, rfin, part, nbop, st);
        nlaunch++;
        prof_end(ev);
        anchor_is_residual = false;
        last_resid_df = true;
    } else if (df_resid && anchor_ready && !exact) {
        // double-float from the anchor: dx = x - x0 split into the padded layout (with the |x|^2
        // partials), then the TMA-staged stencil on the FP32 pipe
        OpEv* ev = prof_begin(3, (double)g.n * 8 * 4 + (double)g.xs * g.ys * g.zs);
        qms_launch_delta_split(g, x, x0, xdf, part, nbop, st);
        qms_launch_resid_df(g, qms_step_par<qdf>(g, v[0], v[1], v[2], desc.dt, transient), xdfmap, cdfmap, adv, rpl,
                            r0df, part, status, st, rfin);
        nlaunch += 2;
        prof_end(ev);
        last_resid_df = true;
    } else {
        QStepPar<double> P = qms_step_par<double>(g, v[0], v[1], v[2], desc.dt, transient);
        op<double>(adv, QOPH_RESID, P, x, b, r64, nullptr, part);
        if (df_resid && !exact) {
            // the anchor of the double-float residuals that follow in this solve (an exact
            // residual asked for between solves leaves the anchor and its chain as they are)
            qms_launch_split_ref_pl(g, r64, r0df, rpl, st);
            CK(cudaMemcpyAsync(x0, x, g.n * 8, cudaMemcpyDeviceToDevice, st));
            nlaunch++;
            anchor_ready = true;
        }
        last_resid_df = false;
    }
    finalize(FIN_RESID, 4, nbop);
    return 0;
}

template <typename T>
void QmsSolver::resid_to_inner(T* out) {
    if constexpr (sizeof(T) == 4) {
        if (df_resid) {
            qms_launch_pl_scale(npl, rpl, S + S_INVNRM, out, st);
            nlaunch++;
            return;
        }
    }
    qms_launch_pl_from_ref<T>(g, r64, S + S_INVNRM, out, st);
    nlaunch++;
}

// b of the last solve, formed from its start state (x0) when that solve took b - b_prev from
// the state difference instead
void QmsSolver::ensure_b() {
    if (b_fresh) return;
    qms_launch_rhs(g, ids, dtab64, last_ex, desc.dt, last_tr ? 1 : 0, x0, b, nullptr, st, rsg, rsdt);
    nlaunch++;
    b_fresh = true;
}

int QmsSolver::residual(bool adv, bool transient, const double v[3], bool exact) {
    int rc = residual_launch(adv, transient, v, exact);
    if (rc) return rc;
    CK(cudaGetLastError());
    return read_scalars();
}

// One refinement iteration (FGMRES with k iterations, FP64 update, FP64 residual) as a
// CUDA graph, captured once per (velocity, form, k) and replayed.
void QmsSolver::drop_graphs() {
    for (IrGraph& G : graphs) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        for (auto& e : G.ev) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    }
    graphs.clear();
    for (StepGraph& G : sgraphs)
        if (G.exec) cudaGraphExecDestroy(G.exec);
    sgraphs.clear();
}

// One whole chained step as a graph (captured once per k, start variant and velocity, then
// replayed): returns after the step with the residual sums in hS and the cycles it ran.
int QmsSolver::step_graph(bool adv, const double v[3], const QStepStart& hs, bool wcalc, int k, int& cycles) {
    const bool dbx = hs.hx != nullptr;
    StepGraph* G = nullptr;
    for (StepGraph& e : sgraphs)
        if (e.k == k && e.xo == hs.xo && e.ls == hs.ls && e.wcalc == wcalc && e.dbx == dbx && e.v[0] == v[0] && e.v[1] == v[1] &&
            e.v[2] == v[2]) { G = &e; break; }
    if (!G) {
        constexpr size_t kMax = 4;
        if (sgraphs.size() >= kMax) {
            size_t lru = 0;
            for (size_t q = 1; q < sgraphs.size(); q++) if (sgraphs[q].used < sgraphs[lru].used) lru = q;
            if (sgraphs[lru].exec) cudaGraphExecDestroy(sgraphs[lru].exec);
            sgraphs.erase(sgraphs.begin() + (long)lru);
        }
        StepGraph ng;
        cudaGraph_t graph = nullptr;
        CK(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle hc;
        cudaError_t e = cudaGraphConditionalHandleCreate(&hc, graph, 0, cudaGraphCondAssignDefault);
        const long long n0 = nlaunch;
        int rc = 0;
        if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            capturing = true;
            cudaMemsetAsync(status, 0, 4, st);
            cudaMemcpyAsync(dptrs, hptrs, sizeof(QStepPtrs), cudaMemcpyHostToDevice, st);
            qms_launch_step_start(g, rfin, b, bprev, dinvdf, r0df, hs, rpl, part, nbop, st, dptrs);
            finalize(FIN_RESID, 4, nbop);
            qk_cond_init<<<1, 32, 0, st>>>(S, desc.tol, hc);
            nlaunch += 2;
            ng.pro = nlaunch - n0;
            // the conditional node at the end of the prologue
            cudaStreamCaptureStatus cs;
            cudaGraph_t cg = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &nd);
            cudaGraphNodeParams cp = {};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = hc;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t cn = nullptr;
            if (e == cudaSuccess) e = cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &cp);
            if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(st, &cn, nullptr, 1, cudaStreamSetCaptureDependencies);
            cudaGraph_t got = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(st, &got);
            if (e == cudaSuccess) e = e2;
            // the body: one refinement cycle and the test that sets the condition
            if (e == cudaSuccess) {
                cudaGraph_t body = cp.conditional.phGraph_out[0];
                e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    const long long n1 = nlaunch;
                    int it = 0;
                    start_resid_ready = false;          // the body's residual is the double-float one
                    rc = inner_gmres<float>(adv, true, v, it, k);
                    if (rc == 0) rc = residual_launch(adv, true, v);
                    qk_cond_next<<<1, 32, 0, st>>>(S, desc.tol, kStepGraphCycles, hc);
                    nlaunch++;
                    ng.body = nlaunch - n1;
                    cudaGraph_t bg = nullptr;
                    e2 = cudaStreamEndCapture(st, &bg);
                    if (e == cudaSuccess) e = e2;
                }
            }
            capturing = false;
        }
        nlaunch = n0;
        if (rc == 0 && e == cudaSuccess) e = cudaGraphInstantiate(&ng.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (rc || e != cudaSuccess) {
            cudaGetLastError();
            if (ng.exec) cudaGraphExecDestroy(ng.exec);
            if (rc) return rc;
            err = std::string("step graph: ") + cudaGetErrorString(e);
            return QMS_ERR_CUDA;
        }
        ng.k = k; ng.xo = hs.xo; ng.ls = hs.ls; ng.wcalc = wcalc; ng.dbx = dbx;
        ng.v[0] = v[0]; ng.v[1] = v[1]; ng.v[2] = v[2];
        sgraphs.push_back(ng);
        G = &sgraphs.back();
    }
    // the rotating pointers of this step, read by the graph's copy node at launch
    *hptrs = QStepPtrs{hs.xo1, hs.xo2, hs.xo3, hs.wnew, hs.w1, hs.w2, hs.hx, b, bprev, hs.xo4, hs.w3};
    G->used = ++graph_clock;
    CK(cudaGraphLaunch(G->exec, st));
    int rc = read_scalars();                    // synchronises the stream
    if (rc) return rc;
    cycles = (int)hS[S_CYC];
    nlaunch += G->pro + (long long)cycles * G->body;
    last_resid_df = true;
    start_resid_ready = false;
    return 0;
}

int QmsSolver::ir_iteration_graph(bool adv, bool transient, const double v[3], int k) {
    const bool want_prof = prof && !graph_prof_broken;
    IrGraph* G = nullptr;
    for (IrGraph& e : graphs)
        if (e.k == k && e.tr == transient && e.adv == adv && e.v[0] == v[0] && e.v[1] == v[1] && e.v[2] == v[2] &&
            e.prof == want_prof) { G = &e; break; }
    if (!G) {
        // a small cache: the least recently used capture makes room
        constexpr size_t kMaxGraphs = 6;
        if (graphs.size() >= kMaxGraphs) {
            size_t lru = 0;
            for (size_t q = 1; q < graphs.size(); q++) if (graphs[q].used < graphs[lru].used) lru = q;
            if (graphs[lru].exec) cudaGraphExecDestroy(graphs[lru].exec);
            for (auto& e : graphs[lru].ev) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
            graphs.erase(graphs.begin() + (long)lru);
        }
        graphs.emplace_back();
        G = &graphs.back();
        // with profiling on, the operator / V-cycle event records are captured as graph nodes
        // on the entry's own event set and read back after every replay
        const bool prof_was = prof;
        const size_t ev_saved = evused;
        prof = want_prof;
        std::swap(evpool, G->ev);
        evused = 0;
        capturing = true;
        const long long n0 = nlaunch;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        int rc = 0;
        if (e == cudaSuccess) {
            int it = 0;
            rc = fp64_inner ? inner_gmres<double>(adv, transient, v, it, k) : inner_gmres<float>(adv, transient, v, it, k);
            if (rc == 0) rc = residual_launch(adv, transient, v);
            G->resid_df = last_resid_df;
        }
        cudaGraph_t graph = nullptr;
        if (e == cudaSuccess) e = cudaStreamEndCapture(st, &graph);
        capturing = false;
        G->evn = evused;
        std::swap(evpool, G->ev);
        evused = ev_saved;
        prof = prof_was;
        if (rc == 0 && e == cudaSuccess) e = cudaGraphInstantiate(&G->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (rc || e != cudaSuccess) {
            if (G->exec) cudaGraphExecDestroy(G->exec);
            for (auto& q : G->ev) { cudaEventDestroy(q.a); cudaEventDestroy(q.b); }
            graphs.pop_back();
            if (rc) return rc;
            err = std::string("graph capture: ") + cudaGetErrorString(e);
            return QMS_ERR_CUDA;
        }
        G->launches = nlaunch - n0;
        nlaunch = n0;
        G->k = k; G->tr = transient; G->adv = adv; G->prof = want_prof;
        G->v[0] = v[0]; G->v[1] = v[1]; G->v[2] = v[2];
    }
    G->used = ++graph_clock;
    CK(cudaGraphLaunch(G->exec, st));
    nlaunch += G->launches;
    // host state that the captured residual sets: a replay ends in the same kind of residual
    last_resid_df = G->resid_df;
    last_inner = 2;
    last_gm_k = k;
    int rc = read_scalars();                     // synchronises the stream
    if (rc == 0 && G->prof && prof)
        for (size_t q = 0; q < G->evn; q++)
            if (!prof_accum(G->ev[q])) { graph_prof_broken = true; break; }
    return rc;
}

int QmsSolver::solve(bool transient, const double v[3], const double B[3], const double G[9]) {
    CK(cudaSetDevice(dev));
    QmsExcite ex;
    for (int q = 0; q < 3; q++) { ex.B[q] = B[q]; ex.v[q] = v[q]; }
    for (int q = 0; q < 9; q++) ex.G[q] = G[q];
    // the previous solve's final residual anchors this one when the operator is the same
    const bool chain = df_resid && transient && rfin_ok && chain_len < QMS_CHAIN_MAX && chain_v[0] == v[0] &&
                       chain_v[1] == v[1] && chain_v[2] == v[2];
    // the start of a transient solve that follows solves with the same operator: an extrapolation
    // of the last solutions (x = hist[0], the one before in hist[1], ...), independent of how the
    // residual is anchored
    const bool same_op = transient && chain_v[0] == v[0] && chain_v[1] == v[1] && chain_v[2] == v[2];
    if (!same_op) hist_len = 0;
    // order of the extrapolation: the known solutions (hist_len, x_n included) less one
    int xo = !same_op || !xold ? 0 : std::max(0, std::min(std::min(desc.extrapolate, 3), hist_len - 1));
    bool same_field = true;
    for (int q = 0; q < 3; q++) same_field = same_field && chain_B[q] == B[q];
    for (int q = 0; q < 9; q++) same_field = same_field && chain_G[q] == G[q];
    field_run = same_field ? field_run + 1 : 1;
    // w_n = D^-1 M (x_n - x_{n-1}) follows when this solve and the last one are chained; the
    // residual of the extrapolated start then follows from the w of the last xo steps when the
    // Dirichlet values did not change over them
    const bool wcalc = chain && last_chained && wh[0];
    // the least-squares start over ls of the last state differences: the known solutions less
    // one, the stored residual images of the differences before d_n plus the one formed now,
    // and the solves with the same Dirichlet values all bound it
    int ls = 0;
    if (wcalc && same_op && xold && desc.start_ls > 0)
        ls = std::max(0, std::min(std::min(desc.start_ls, hist_len - 1), std::min(w_len + 1, field_run - 2)));
    if (ls > 0) xo = ls;
    const bool start_fused = wcalc && xo > 0 && w_len >= xo - 1 && field_run >= xo + 2;
    // with the field unchanged and x_(n-1) known, the anchor takes b - b_prev from x_n - x_(n-1)
    // (the step start, in double-float) and this solve forms no FP64 right-hand side
    const bool db_from_x = chain && same_field && hist_len >= 2 && hist_x && xold && rsg;
    start_resid_ready = false;
    // the whole step as one graph: a chained step whose start also forms the first residual, with
    // replayed refinement cycles of a known count (no profile events inside: they cannot live in
    // a conditional body)
    const bool use_step_graph = desc.use_graphs && desc.krylov == QMS_KRYLOV_GMRES && start_fused && db_from_x &&
                                gm_k_est > 0 && !prof && !trace && hptrs && !(desc.tol_v > 0.0);
    QStepStart sg_hs{};
    bool sg_wcalc = false;
    if (chain && !db_from_x) {
        ensure_b();                // b_prev: the last solve's right-hand side
        // x0 is copied, not swapped: the captured refinement graphs hold its address
        CK(cudaMemcpyAsync(x0, x, g.n * 8, cudaMemcpyDeviceToDevice, st));   // the previous solution
        std::swap(b, bprev);
    }
    last_ex = ex;
    last_tr = transient;
    if (!db_from_x) {
        // b from the previous solution (x); Dirichlet values written into x (warm start keeps them exact)
        qms_launch_rhs(g, ids, dtab64, ex, desc.dt, transient ? 1 : 0, x, b, x, st, rsg, rsdt);
        nlaunch++;
        b_fresh = true;
    } else {
        b_fresh = false;           // formed from x0 when asked for (ensure_b)
    }
    anchor_ready = false;          // the first residual of this solve is the FP64 anchor ...
    anchor_is_residual = false;
    if (chain) {                   // ... unless it follows from the previous one
        // the anchor, w_n and the extrapolated start in one pass; the residual of that start too
        // when start_fused (otherwise the double-float residual from the anchor follows)
        const int nw = nwh;                                     // w buffers: w_(n-1), w_(n-2), ..., the new one
        QStepStart hs{x,    xold, xold2, xold3, xo, wcalc ? wh[nw - 1] : nullptr, wh[0], wh[1],
                      db_from_x ? hist_x : nullptr, rsg, rsdt, desc.dt, db_from_x ? x0 : nullptr,
                      xold4, wh[2], ls, lsp, lsg};
        if (use_step_graph) {
            sg_hs = hs;                  // launched inside the step's graph below
            sg_wcalc = wcalc;
        } else {
            OpEv* ev = start_fused ? prof_begin(3, (double)g.n * (ls > 0 ? 8 * 11 + 8 * (ls - 1) + 8 * (2 * ls + 5) + 4
                                                                         : 8 * 11 + 8 * 2 * xo + 4)) : nullptr;
            qms_launch_step_start(g, rfin, b, bprev, dinvdf, r0df, hs, start_fused ? rpl : nullptr, part, nbop, st);
            nlaunch++;
            prof_end(ev);
        }
        if (wcalc) {               // wh[0]: w_n, wh[1]: w_(n-1), the oldest becomes the next one's buffer
            qdf* fresh = wh[nw - 1];
            for (int q = nw - 1; q > 0; q--) wh[q] = wh[q - 1];
            wh[0] = fresh;
        }
        w_len = wcalc ? std::min(w_len + 1, std::max(1, nw - 1)) : 0;
        anchor_ready = true;
        chain_len++;
        // same field and no extrapolation: the Dirichlet values did not move, x is the anchor state
        anchor_is_residual = same_field && xo == 0;
        start_resid_ready = start_fused;
    } else {
        chain_len = 0;
        w_len = 0;
        if (xo > 0) {
            // the extrapolated start (Dirichlet rows keep the values just written); its residual
            // is the FP64 anchor
            qms_launch_extrapolate(g, x, xold, xold2, xold3, xo, st);
            nlaunch++;
        }
    }
    last_chained = chain;
    rfin_ok = false;
    if (!use_step_graph) CK(cudaMemsetAsync(status, 0, 4, st));
    const bool adv = v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0;
    const bool use_cg = !transient && !adv;
    stats = qms_stats{};
    double rel = INFINITY, prev_rn = INFINITY, sref = 0.0;
    int outer = 0, stalled = 0;
    graph_resid_ready = false;
    const int gm_m = std::min(desc.gmres_m, GM_MAXM);
    int graph_k_used = 0;                 // k of the graph replay that produced this residual (0: none)
    int gm_k_last = 0;                    // FGMRES steps of the last cycle (graph or host-checked)
    int gm_cycles = 0;                    // FGMRES cycles run in this solve
    int graph_cycles = 0;                 // ... of them replayed from graphs
    double best_rn = INFINITY, best_rel = INFINITY;
    if (use_step_graph) {
        // the step (start and up to kStepGraphCycles cycles) in one graph; the loop below takes
        // over from the residual it leaves, as after a replayed cycle
        int cyc = 0;
        int rc = step_graph(adv, v, sg_hs, sg_wcalc, gm_k_est, cyc);
        if (rc) return rc;
        graph_resid_ready = true;
        stats.step_graph = 1;
        stats.initial_residual = hS[S_REL0];
        if (cyc > 0) {
            outer = cyc;
            sref = hS[S_SREF];
            prev_rn = hS[S_PRN_LAST];
            gm_k_last = graph_k_used = gm_k_est;
            gm_cycles = graph_cycles = cyc;
            stats.inner_iterations = cyc * gm_k_est;
            last_inner = 2;
            last_gm_k = gm_k_est;
        }
    }
    for (;;) {
        int rc = 0;
        if (!graph_resid_ready) {
            rc = residual(adv, transient, v);
            if (rc) return rc;
        }
        graph_resid_ready = false;
        const double xn = std::sqrt(hS[S_XA] + hS[S_XV]);
        const double rn = std::sqrt(hS[S_RA] + hS[S_RV]);
        // The scale is fixed by the state at the start of the solve (the previous step, or the
        // Dirichlet values for the steady state): a correction that blew up x must not make
        // ||r|| / ||x|| look small.
        if (outer == 0) sref = xn > 0 ? xn : 1.0;
        const double scale = std::min(std::max(xn, sref), 100.0 * sref);
        rel = rn / scale;
        if (outer == 0) stats.initial_residual = rel;
        if (!std::isfinite(rel)) { stats.status |= QMS_ST_NAN; break; }
        // optionally the potential block on its own scale as well: where |x| is dominated by A
        // (slow fields, small potentials), rel alone does not bound V's relative error
        const bool v_ok = !(desc.tol_v > 0.0) || hS[S_XV] == 0.0 ||
                          std::sqrt(hS[S_RV]) <= desc.tol_v * std::sqrt(hS[S_XV]);
        if ((rel <= desc.tol && v_ok) || rn == 0.0) break;
        // Per-step reduction rate of FGMRES from the true residuals around each cycle, kept
        // apart for the first cycle of a solve and the later ones and smoothed in log space;
        // it sizes the next replay.  A replay that gained less than a tenth per cycle while k
        // can still grow is not a stall.
        bool k_limited = false;
        if (gm_k_last > 0 && std::isfinite(prev_rn) && prev_rn > 0 && rn > 0 && rn < prev_rn) {
            const double rho = rn / prev_rn;
            const double lr = std::log(rho) / gm_k_last;
            double& slot = gm_lrate[gm_cycles == 1 ? 0 : 1];
            slot = slot < 0.0 ? 0.5 * (slot + lr) : lr;
            if (graph_k_used > 0 && graph_k_used < gm_m && rho > 0.1) k_limited = true;
        }
        graph_k_used = 0;
        gm_k_last = 0;
        // Stall: near the round-off floor (within 1e3 of the tolerance) two iterations without
        // halving the residual end the solve; elsewhere only three iterations that gain less
        // than 10 % do, so that slowly but steadily converging solves continue.
        const bool near_floor = rel <= 1e3 * desc.tol;
        const bool slow = near_floor ? rn > 0.5 * prev_rn : rn > 0.9 * prev_rn;
        stalled = slow && !k_limited ? stalled + 1 : 0;
        if (stalled >= (near_floor ? 2 : 3)) {
            if (rel > 1e3 * desc.tol) stats.status |= QMS_ST_NO_CONVERGENCE;
            break;
        }
        // best state so far: a hard solve may lose ground for an iteration or two before it
        // gains again; whatever ends the solve, it ends at the best iterate
        if (rn < best_rn) {
            best_rn = rn;
            best_rel = rel;
            CK(cudaMemcpyAsync(xbest, x, g.n * 8, cudaMemcpyDeviceToDevice, st));
        }
        if (trace) {
            double est = 0.0;
            if (outer > 0 && last_inner == 2) {
                CK(cudaMemcpyAsync(hS + S_COUNT - 2, gm_scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                est = hS[S_COUNT - 1] / hS[S_COUNT - 2];
            }
            std::fprintf(stderr, "qms: %s outer %d |r| %.3e rel %.3e |x| %.3e |rA| %.3e |rV| %.3e inner-est %.2e k %d\n",
                         transient ? "step" : "steady", outer, rn, rel, xn, std::sqrt(hS[S_RA]), std::sqrt(hS[S_RV]),
                         est, last_gm_k);
        }
        if (outer >= desc.max_outer) { stats.status |= QMS_ST_NO_CONVERGENCE; break; }
        prev_rn = rn;
        int it = 0;
        if (use_cg) {
            last_inner = 0;
            rc = fp64_inner ? inner_pcg<double>(transient, it) : inner_pcg<float>(transient, it);
        } else if (desc.krylov == QMS_KRYLOV_BICGSTAB) {
            last_inner = 1;
            rc = fp64_inner ? inner_bicgstab<double>(adv, transient, v, it)
                            : inner_bicgstab<float>(adv, transient, v, it);
        } else if (desc.use_graphs && gm_k_est > 0) {
            // replay a captured refinement iteration; its residual is read back with it.  The
            // first two cycles of a solve run gm_k_est steps each (tuned across solves so that two
            // cycles just suffice); a further cycle runs what the observed rate of the later cycles
            // needs to reach tol / 2
            it = gm_k_est;
            const double lgoal = std::log(0.5 * desc.tol / rel);
            if (graph_cycles >= 2 && gm_lrate[1] < -1e-3 && lgoal < 0.0)
                it = std::min(gm_m, std::max(6, (int)std::ceil(lgoal / gm_lrate[1]) + 2));
            // a start residual that the usual count would leave just above the tolerance: one
            // cycle a few steps longer (at the observed first-cycle rate) instead of two cycles
            if (graph_cycles == 0 && desc.gm_first_extend > 0 && gm_lrate[0] < -1e-3 && lgoal < 0.0) {
                const int need = (int)std::ceil(lgoal / gm_lrate[0]) + 1;
                if (need > it && need <= std::min(gm_m, gm_k_est + desc.gm_first_extend)) it = need;
            }
            graph_cycles++;
            rc = ir_iteration_graph(adv, transient, v, it);
            if (rc) return rc;
            graph_k_used = it;
            gm_k_last = it;
            gm_cycles++;
            stats.inner_iterations += it;
            outer++;
            graph_resid_ready = true;
            continue;
        } else {
            last_inner = 2;
            rc = fp64_inner ? inner_gmres<double>(adv, transient, v, it, 0) : inner_gmres<float>(adv, transient, v, it, 0);
            if (!rc) gm_k_seen = std::max(gm_k_seen, it);
            gm_k_last = it;
            gm_cycles++;
        }
        if (rc) return rc;
        stats.inner_iterations += it;
        outer++;
    }
    // the final residual (rfin) anchors the next transient solve when it belongs to the state
    // that this solve leaves in x
    rfin_ok = df_resid && transient && last_resid_df && rel <= desc.tol;
    // history of converged transient solutions for the extrapolated start (x itself is the newest;
    // xold and xold2 the two before, rotated by pointer: only the extrapolation reads them)
    if (transient && rel <= desc.tol && xold) {
        double* freed = xold4 ? xold4 : xold3 ? xold3 : xold2 ? xold2 : xold;
        if (xold4) xold4 = xold3;
        if (xold3) xold3 = xold2;
        if (xold2) xold2 = xold;
        xold = hist_x;
        hist_x = freed;
        CK(cudaMemcpyAsync(hist_x, x, g.n * 8, cudaMemcpyDeviceToDevice, st));
        hist_len = std::min(hist_len + 1, xold4 ? 5 : xold3 ? 4 : xold2 ? 3 : 2);
    } else {
        hist_len = 0;
        last_chained = false;
    }
    for (int q = 0; q < 3; q++) { chain_v[q] = v[q]; chain_B[q] = B[q]; }
    for (int q = 0; q < 9; q++) chain_G[q] = G[q];
    if (!(rel <= desc.tol) && best_rel < rel && std::isfinite(best_rel)) {
        rfin_ok = false;
        CK(cudaMemcpyAsync(x, xbest, g.n * 8, cudaMemcpyDeviceToDevice, st));
        rel = best_rel;
        if (rel <= desc.tol) stats.status &= ~(unsigned)QMS_ST_NO_CONVERGENCE;
    }
    // replays start short: a solve that needs a third cycle costs less than two long cycles,
    // and the count below adapts either way
    if (!use_cg && desc.krylov == QMS_KRYLOV_GMRES && desc.use_graphs && gm_k_est == 0 && gm_k_seen > 0)
        gm_k_est = std::min(std::min(desc.gmres_m, GM_MAXM), std::min(gm_k_seen + 1, 12));
    // per-cycle count of the replays.  The FP32 inner solve gains little past ~1e-3 per cycle
    // (its own rounding), so a longer cycle buys less than a restart from a fresh residual:
    // probe downwards after every solve that two replays brought below tol / 3 (in steps of a
    // fifth of k until the first solve that needed a third replay, one step after that), and
    // step back up by two when a solve needed a third
    // A count that needed a third replay is not probed again for 32 solves.  (One longer cycle
    // in place of two does not pay: the FP32 inner solve stalls within a cycle, and a single
    // cycle needed ~23 steps where two of 7 sufficed.)
    // One-replay solves probe down to 5 steps; a probe below 6 that needed a second replay goes
    // back to 6, which then holds for 32 solves.  (Letting any count step back up after a
    // second replay raised it instead: one slow step pinned it at 7-8 for 32 solves.)
    // After a least-squares start the start residual is within a few times the tolerance and
    // falls from step to step, so the count follows the measured rate: a one-replay solve that
    // ended below tol / 4 takes the count that this solve's reduction per FGMRES step says
    // reaches tol / 4 from its start (at least one less); a solve that needed a second replay
    // goes up by one (two after a third), and when its start had every direction it holds there
    // for 4 solves (the first steps of a run know fewer directions and start worse: floors from
    // them kept the count high well after).  Floors set by solves without this start do not apply.
    // (On steps 6-25 of the moving plate at 256^3, targets of tol / 10, tol / 4 and tol / 2 ran
    // 26.80, 25.51 and 24.74 ms per step; tol / 2 left the field 1.05e-8 from the plain FP64
    // solve's at one step of 200, tol / 4 at most 9.8e-9.)
    if (graph_cycles > 0 && rel <= desc.tol && ls > 0) {
        if (gm_ls_floor > 0 && ++gm_ls_floor_age > 4) { gm_ls_floor = 0; gm_ls_floor_age = 0; }
        if (graph_cycles >= 2) {
            gm_k_est = std::min(gm_m, gm_k_est + (graph_cycles >= 3 ? 2 : 1));
            if (ls >= desc.start_ls) {
                gm_ls_floor = gm_k_est;
                gm_ls_floor_age = 0;
            }
        } else if (rel < desc.tol / 4.0) {
            const double r0 = stats.initial_residual;
            int need = 1;
            if (r0 > desc.tol / 4.0 && rel > 0.0 && r0 > rel) {
                const double rate = std::log(r0 / rel) / std::max(1, gm_k_est);
                need = (int)std::ceil(std::log(r0 / (desc.tol / 4.0)) / rate);
            }
            gm_k_est = std::max(std::max(1, gm_ls_floor), std::min(gm_k_est - 1, need));
        }
    } else if (graph_cycles > 0 && rel <= desc.tol) {
        if (gm_k_floor > 0 && ++gm_k_floor_age >= 32) { gm_k_floor--; gm_k_floor_age = 0; }
        if (graph_cycles >= 3) {
            gm_k_floor = gm_k_est + 1;
            gm_k_floor_age = 0;
            gm_k_est = std::min(gm_m, gm_k_est + 2);
            gm_k_fine = true;
        } else if (graph_cycles == 2 && gm_cycles == 2) {
            if (gm_k_est < 6) {
                gm_k_est = 6;
                gm_k_floor = 6;
                gm_k_floor_age = 0;
            } else if (rel < desc.tol / 3.0) {
                gm_k_est = std::max(std::max(6, gm_k_floor),
                                    gm_k_est - (gm_k_fine ? 1 : std::max(1, gm_k_est / 5)));
            }
        } else if (graph_cycles == 1 && gm_cycles == 1 && rel < desc.tol / 3.0) {
            gm_k_est = std::max(std::max(5, gm_k_floor), gm_k_est - 1);
        }
    }
    unsigned stt = 0;
    double lsv[8] = {};
    CK(cudaMemcpyAsync(&stt, status, 4, cudaMemcpyDeviceToHost, st));
    if (ls > 0) CK(cudaMemcpyAsync(lsv, lsg, sizeof(lsv), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (ls > 0) {
        stats.start_ls = ls;
        for (int q = 0; q < 4; q++) stats.start_coef[q] = lsv[q];
        stats.start_base = lsv[4];
        stats.start_pred = lsv[5];
    }
    stats.status |= stt & ~(unsigned)QMS_ST_BREAKDOWN;
    stats.outer_iterations = outer;
    stats.final_residual = rel;
    return 0;
}

int QmsSolver::fields(int which, int axis, int index, double* host_out) {
    CK(cudaSetDevice(dev));
    const long long ncell = (long long)g.xs * g.ys * g.zs;
    if (which == QMS_FIELD_CUBES) {
        qms_launch_hfield(g, ids, dtab64, x, H, H + ncell, H + 2 * ncell, st);
        nlaunch++;
        CK(cudaMemcpyAsync(host_out, H, 3 * ncell * 8, cudaMemcpyDeviceToHost, st));
    } else {
        int lim = axis == 0 ? g.xs : axis == 1 ? g.ys : g.zs;
        if (axis < 0 || axis > 2 || index < 1 || index > lim) { err = "slice axis/index out of range"; return QMS_ERR_ARG; }
        // only the slice's cells (what the reference dumps every step)
        qms_launch_hslice(g, ids, dtab64, x, axis, index, slicebuf, st);
        nlaunch++;
        long long m = (long long)(axis == 0 ? g.ys : g.xs) * (axis == 2 ? g.ys : g.zs);
        CK(cudaMemcpyAsync(host_out, slicebuf, 3 * m * 8, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    return 0;
}

int QmsSolver::fields_async(int which, int axis, int index, double* host_out, int slot) {
    CK(cudaSetDevice(dev));
    if (slot < 0 || slot >= kFieldSlots) { err = "field slot out of range"; return QMS_ERR_ARG; }
    const long long ncell = (long long)g.xs * g.ys * g.zs;
    long long m = 3 * ncell;
    if (which == QMS_FIELD_SLICE) {
        int lim = axis == 0 ? g.xs : axis == 1 ? g.ys : g.zs;
        if (axis < 0 || axis > 2 || index < 1 || index > lim) { err = "slice axis/index out of range"; return QMS_ERR_ARG; }
        m = 3LL * (axis == 0 ? g.ys : g.xs) * (axis == 2 ? g.ys : g.zs);
    } else if (which != QMS_FIELD_CUBES) {
        err = "unknown field kind";
        return QMS_ERR_ARG;
    }
    if (!cst) CK(cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking));
    if (!fev_ready[slot]) {
        CK(cudaEventCreateWithFlags(&fev_ready[slot], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&fev_done[slot], cudaEventDisableTiming));
    }
    // the slot's previous copy must be finished before its device buffer is reused
    CK(cudaEventSynchronize(fev_done[slot]));
    if (fbuf_n[slot] < (size_t)m) {
        if (fbuf[slot]) CK(cudaFree(fbuf[slot]));
        fbuf[slot] = nullptr;
        fbuf_n[slot] = 0;
        CK(cudaMalloc(&fbuf[slot], m * 8));
        fbuf_n[slot] = (size_t)m;
    }
    double* d = fbuf[slot];
    if (which == QMS_FIELD_CUBES)
        qms_launch_hfield(g, ids, dtab64, x, d, d + ncell, d + 2 * ncell, st);
    else
        qms_launch_hslice(g, ids, dtab64, x, axis, index, d, st);
    nlaunch++;
    CK(cudaGetLastError());
    CK(cudaEventRecord(fev_ready[slot], st));
    CK(cudaStreamWaitEvent(cst, fev_ready[slot], 0));
    CK(cudaMemcpyAsync(host_out, d, m * 8, cudaMemcpyDeviceToHost, cst));
    CK(cudaEventRecord(fev_done[slot], cst));
    return 0;
}

int QmsSolver::fields_sync(int slot) {
    if (slot < 0 || slot >= kFieldSlots) return QMS_ERR_ARG;
    if (!fev_done[slot]) return 0;
    cudaError_t e = cudaEventSynchronize(fev_done[slot]);
    return e == cudaSuccess ? 0 : QMS_ERR_CUDA;
}

template int QmsSolver::inner_bicgstab<float>(bool, bool, const double*, int&);
template int QmsSolver::inner_bicgstab<double>(bool, bool, const double*, int&);
template int QmsSolver::inner_pcg<float>(bool, int&);
template int QmsSolver::inner_pcg<double>(bool, int&);
template int QmsSolver::inner_gmres<float>(bool, bool, const double*, int&, int);
template int QmsSolver::inner_gmres<double>(bool, bool, const double*, int&, int);
template void QmsSolver::precond<float>(const float*, const float*, float*, bool, bool, bool,
                                        const QStepPar<float>*, bool);
template void QmsSolver::precond<double>(const double*, const float*, double*, bool, bool, bool,
                                         const QStepPar<double>*, bool);
