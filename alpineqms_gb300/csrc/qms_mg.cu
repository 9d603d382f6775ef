// qms_mg.cu -- block-diagonal multigrid preconditioner for the Yee A-V system.
//
// The preconditioner treats the four unknown blocks (Ax, Ay, Az on edges, V on
// nodes) as four scalar 7-point problems: for each A component the
// same-direction couplings of its own row (curl-curl + gauge penalty
// coefficients 1/(mu h^2), F:476-525, F:682-731, F:888-937) plus the sigma/dt
// edge mass (F:1500-1504); for V the sigma-weighted Laplacian (F:1236-1285)
// with its diagonal shifted by a relative 1e-5: an isolated conductor's
// potential is fixed only through the 1e-12 S/m floor, a mode ~19 decades
// below the conductor scale that an exact inverse would amplify without bound.  Cross-component, advective and A-V
// coupling terms are left to the outer Krylov method.  For constant
// coefficients the A-block symbol |xi|^2 I - xi xi^T + diag(xi^2) lies
// between 1/3 and 2 times the vector Laplacian's, so the block-diagonal
// Laplacian preconditioner is spectrally equivalent.
//
// Hierarchy: unsmoothed 2x2x2 aggregation on each block's structured grid
// (general sizes; the two-layer Dirichlet shell leaves 253/254-point
// interiors that are not powers of two).  With piecewise-constant
// prolongation the Galerkin coarse operator of a 7-point operator is again
// 7-point: a coarse link is the sum of the fine links crossing between the two
// aggregates and a coarse diagonal is the sum of the fine diagonals minus
// twice the internal links.  All four blocks of a level are stored back to
// back and processed by one launch through a packed block-descriptor table.
// Smoother: weighted Jacobi.  Coarsest level: dense FP64 inverse per block.
#include "qms_mg.h"
#include "qms_pl.h"
#include "qms_tile.cuh"

#include <cuda_bf16.h>

#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

namespace {

// (i, j, k) of offset q in a block of n1 x n2 x n3 points, in 32-bit arithmetic (a block of a
// level holds far fewer than 2^32 points)
__device__ __forceinline__ void mg_ijk(long long q, int n1, int n2, int& i, int& j, int& k) {
    const unsigned u = (unsigned)q, a = u / (unsigned)n1, c = a / (unsigned)n2;
    i = (int)(u - a * (unsigned)n1);
    j = (int)(a - c * (unsigned)n2);
    k = (int)c;
}

template <typename T>
__device__ __forceinline__ int find_block(const MGLevelDev<T>& L, long long t) {
    int b = 0;
#pragma unroll
    for (int q = 1; q < MG_MAX_BLOCKS; q++)
        if (q < L.nb && t >= L.blk[q].off) b = q;
    return b;
}

// ---------------------------------------------------------------- fine level
// links (+1 neighbour along each axis), diagonal and activity of fine point
// (i, j, k) (1-based) of block b
template <typename T>
__device__ __forceinline__ bool mg_fine_point(const QGrid& g, const QCoef<T>& c, const QStepPar<T>& P, T vshift,
                                              int b, int i, int j, int k, T& w1, T& w2, T& w3, T& d) {
    bool active;
    w1 = w2 = w3 = T(0);
    d = T(1);
    if (b == 0) {            // Ax
        active = !qFixX(g, i, j, k);
        w1 = i < g.xs ? c.imux(i, j, k) * P.idx2 : T(0);
        w2 = j < g.Ny ? c.imuz(i, j, k) * P.idy2 : T(0);
        w3 = k < g.Nz ? c.imuy(i, j, k) * P.idz2 : T(0);
        if (active)
            d = (c.imuz(i, j, k) + c.imuz(i, j - 1, k)) * P.idy2 + (c.imuy(i, j, k) + c.imuy(i, j, k - 1)) * P.idz2 +
                (c.imux(i, j, k) + c.imux(i - 1, j, k)) * P.idx2 + c.sgx(i, j, k) * P.idt;
    } else if (b == 1) {     // Ay
        active = !qFixY(g, i, j, k);
        w1 = i < g.Nx ? c.imuz(i, j, k) * P.idx2 : T(0);
        w2 = j < g.ys ? c.imuy(i, j, k) * P.idy2 : T(0);
        w3 = k < g.Nz ? c.imux(i, j, k) * P.idz2 : T(0);
        if (active)
            d = (c.imuz(i, j, k) + c.imuz(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j, k - 1)) * P.idz2 +
                (c.imuy(i, j, k) + c.imuy(i, j - 1, k)) * P.idy2 + c.sgy(i, j, k) * P.idt;
    } else if (b == 2) {     // Az
        active = !qFixZ(g, i, j, k);
        w1 = i < g.Nx ? c.imuy(i, j, k) * P.idx2 : T(0);
        w2 = j < g.Ny ? c.imux(i, j, k) * P.idy2 : T(0);
        w3 = k < g.zs ? c.imuz(i, j, k) * P.idz2 : T(0);
        if (active)
            d = (c.imuy(i, j, k) + c.imuy(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j - 1, k)) * P.idy2 +
                (c.imuz(i, j, k) + c.imuz(i, j, k - 1)) * P.idz2 + c.sgz(i, j, k) * P.idt;
    } else {                 // V: the operator's own floor, diagonal shifted by (1 + vshift)
        const T fl = P.sigfloor;
        active = !qFixV(g, i, j, k);
        w1 = i < g.Nx ? fmax(c.sgx(i, j, k), fl) * P.idx2 : T(0);
        w2 = j < g.Ny ? fmax(c.sgy(i, j, k), fl) * P.idy2 : T(0);
        w3 = k < g.Nz ? fmax(c.sgz(i, j, k), fl) * P.idz2 : T(0);
        if (active)
            d = ((fmax(c.sgx(i, j, k), fl) + fmax(c.sgx(i - 1, j, k), fl)) * P.idx2 +
                 (fmax(c.sgy(i, j, k), fl) + fmax(c.sgy(i, j - 1, k), fl)) * P.idy2 +
                 (fmax(c.sgz(i, j, k), fl) + fmax(c.sgz(i, j, k - 1), fl)) * P.idz2) * (T(1) + vshift);
    }
    return active;
}

__device__ __forceinline__ bool mg_fine_active(const QGrid& g, int b, int i, int j, int k) {
    return b == 0 ? !qFixX(g, i, j, k) : b == 1 ? !qFixY(g, i, j, k) : b == 2 ? !qFixZ(g, i, j, k) : !qFixV(g, i, j, k);
}

// -------------------------------------------------------------- coarsening
// coarse point (I,J,K) aggregates fine points (2I..2I+1, 2J..2J+1, 2K..2K+1) (0-based):
// a coarse link is the sum of the fine links crossing between two aggregates, a
// coarse diagonal the sum of the fine diagonals minus twice the internal links.
// `fine(b, f, i, j, k, w1, w2, w3, d, m)` gives fine point f = (i, j, k) of block b (m: the
// summed level-0 diagonals it stands for) and returns whether it is active; `act(b, f, i, j, k)`
// only its activity.
// A coarse V point whose diagonal is at or below ncut times its summed level-0 diagonals is a
// near-null mode (a floating conductor collapsed into one aggregate: the constant over it costs
// almost no energy, and the computed diagonal is the cancellation noise of the sums above); it
// leaves the hierarchy (inactive) instead of amplifying its right-hand side by 1 / noise.  The
// conductor-region coarse space carries such modes exactly.
template <typename T, typename Fine, typename Act>
__device__ __forceinline__ void mg_coarsen_point(const MGBlockDesc& fb, const MGBlockDesc& cb, int b, long long t,
                                                 MGLevelDev<T>& C, double ncut, Fine fine, Act act) {
    long long q = t - cb.off;
    int I, J, K;
    mg_ijk(q, cb.n1, cb.n2, I, J, K);
    double d = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0, ms = 0.0;
    bool any = false;
    const long long s2 = fb.n1, s3 = (long long)fb.n1 * fb.n2;
    for (int dk = 0; dk < 2; dk++) for (int dj = 0; dj < 2; dj++) for (int di = 0; di < 2; di++) {
        int i = 2 * I + di, j = 2 * J + dj, k = 2 * K + dk;
        if (i >= fb.n1 || j >= fb.n2 || k >= fb.n3) continue;
        long long f = fb.off + i + (long long)j * s2 + (long long)k * s3;
        T fw1, fw2, fw3, fd, fm;
        if (!fine(b, f, i, j, k, fw1, fw2, fw3, fd, fm)) continue;
        any = true;
        d += fd;
        ms += fm;
        // +x link of f: internal if di == 0, crossing to I+1 if di == 1
        if (i + 1 < fb.n1 && act(b, f + 1, i + 1, j, k)) {
            if (di == 0) d -= 2.0 * fw1;
            else w1 += fw1;
        }
        if (j + 1 < fb.n2 && act(b, f + s2, i, j + 1, k)) {
            if (dj == 0) d -= 2.0 * fw2;
            else w2 += fw2;
        }
        if (k + 1 < fb.n3 && act(b, f + s3, i, j, k + 1)) {
            if (dk == 0) d -= 2.0 * fw3;
            else w3 += fw3;
        }
    }
    C.w1[t] = I + 1 < cb.n1 ? (T)w1 : T(0);
    C.w2[t] = J + 1 < cb.n2 ? (T)w2 : T(0);
    C.w3[t] = K + 1 < cb.n3 ? (T)w3 : T(0);
    C.dg[t] = any ? (T)d : T(1);
    C.mass[t] = any ? (T)ms : T(1);
    const bool null_mode = b == MG_MAX_BLOCKS - 1 && !(d > ncut * ms);
    C.dinv[t] = any && d > 0.0 && !null_mode ? (T)(1.0 / d) : T(0);
}

// level l+1 from the stored arrays of level l
template <typename T>
__global__ void mg_coarsen(MGLevelDev<T> F, MGLevelDev<T> C, double ncut) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.total) return;
    const int b = find_block(C, t);
    mg_coarsen_point(F.blk[b], C.blk[b], b, t, C, ncut,
                     [&](int, long long f, int, int, int, T& w1, T& w2, T& w3, T& d, T& m) {
                         w1 = F.w1[f]; w2 = F.w2[f]; w3 = F.w3[f]; d = F.dg[f]; m = F.mass[f];
                         return F.dinv[f] != T(0);
                     },
                     [&](int, long long f, int, int, int) { return F.dinv[f] != T(0); });
}

// level 1 straight from the node coefficients (level 0 keeps no arrays of its own)
template <typename T>
__global__ void mg_coarsen_fine(QGrid g, QCoef<T> c, QStepPar<T> P, T vshift, MGLevelDev<T> F, MGLevelDev<T> C,
                                double ncut) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.total) return;
    const int b = find_block(C, t);
    mg_coarsen_point(F.blk[b], C.blk[b], b, t, C, ncut,
                     [&](int bb, long long, int i, int j, int k, T& w1, T& w2, T& w3, T& d, T& m) {
                         const bool a = mg_fine_point(g, c, P, vshift, bb, i + 1, j + 1, k + 1, w1, w2, w3, d);
                         m = d;
                         return a;
                     },
                     [&](int bb, long long, int i, int j, int k) { return mg_fine_active(g, bb, i + 1, j + 1, k + 1); });
}

// a crossing link is only kept if both aggregates are active
template <typename T>
__global__ void mg_mask_links(MGLevelDev<T> C) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.total) return;
    const int b = find_block(C, t);
    const MGBlockDesc& cb = C.blk[b];
    long long q = t - cb.off;
    int I, J, K;
    mg_ijk(q, cb.n1, cb.n2, I, J, K);
    if (C.dinv[t] == T(0)) { C.w1[t] = C.w2[t] = C.w3[t] = T(0); return; }
    if (I + 1 < cb.n1 && C.dinv[t + 1] == T(0)) C.w1[t] = T(0);
    if (J + 1 < cb.n2 && C.dinv[t + cb.n1] == T(0)) C.w2[t] = T(0);
    if (K + 1 < cb.n3 && C.dinv[t + (long long)cb.n1 * cb.n2] == T(0)) C.w3[t] = T(0);
}

// A x at point t of block (n1, n2, n3) -- links to inactive points carry w = 0
template <typename T>
__device__ __forceinline__ T apply7(const MGLevelDev<T>& L, const MGBlockDesc& B, long long t, int i, int j, int k,
                                    const T* __restrict__ x) {
    const long long s2 = B.n1, s3 = (long long)B.n1 * B.n2;
    T acc = L.dg[t] * x[t];
    if (i > 0) acc -= L.w1[t - 1] * x[t - 1];
    if (i + 1 < B.n1) acc -= L.w1[t] * x[t + 1];
    if (j > 0) acc -= L.w2[t - s2] * x[t - s2];
    if (j + 1 < B.n2) acc -= L.w2[t] * x[t + s2];
    if (k > 0) acc -= L.w3[t - s3] * x[t - s3];
    if (k + 1 < B.n3) acc -= L.w3[t] * x[t + s3];
    return acc;
}

// ------------------------------------------------------------------ smoother
// first sweep from a zero guess: x = omega D^-1 b   (b scaled by bscale on level 0)
template <typename T>
__global__ void mg_smooth0(MGLevelDev<T> L, const T* __restrict__ b, const float* __restrict__ bscale, T omega,
                           T* __restrict__ x, int mask_v) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.total) return;
    T bv = b[t];
    if (bscale) bv *= (T)bscale[t];
    T di = L.dinv[t];
    if (mask_v && t >= L.blk[L.nb - 1].off) di = T(0);
    x[t] = omega * di * bv;
}

// x_out = x_in + omega D^-1 (b - A x_in)
template <typename T>
__global__ void mg_smooth(MGLevelDev<T> L, const T* __restrict__ b, const float* __restrict__ bscale, T omega,
                          const T* __restrict__ xin, T* __restrict__ xout, int mask_v) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.total) return;
    T di = L.dinv[t];
    if (mask_v && t >= L.blk[L.nb - 1].off) di = T(0);
    if (di == T(0)) { xout[t] = T(0); return; }
    const int bk = find_block(L, t);
    const MGBlockDesc& B = L.blk[bk];
    long long q = t - B.off;
    int i, j, k;
    mg_ijk(q, B.n1, B.n2, i, j, k);
    T bv = b[t];
    if (bscale) bv *= (T)bscale[t];
    xout[t] = xin[t] + omega * di * (bv - apply7(L, B, t, i, j, k, xin));
}

// residual of the fine level summed over each aggregate -> coarse right-hand side
template <typename T>
__global__ void mg_restrict(MGLevelDev<T> F, const T* __restrict__ bf, const float* __restrict__ bscale,
                            const T* __restrict__ xf, MGLevelDev<T> C, T* __restrict__ bc, int mask_v) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.total) return;
    const int b = find_block(C, t);
    const MGBlockDesc& cb = C.blk[b];
    const MGBlockDesc& fb = F.blk[b];
    long long q = t - cb.off;
    int I, J, K;
    mg_ijk(q, cb.n1, cb.n2, I, J, K);
    T acc = T(0);
    if (!(mask_v && b == C.nb - 1)) {
        for (int dk = 0; dk < 2; dk++) for (int dj = 0; dj < 2; dj++) for (int di = 0; di < 2; di++) {
            int i = 2 * I + di, j = 2 * J + dj, k = 2 * K + dk;
            if (i >= fb.n1 || j >= fb.n2 || k >= fb.n3) continue;
            long long f = fb.off + i + (long long)j * fb.n1 + (long long)k * fb.n1 * fb.n2;
            if (F.dinv[f] == T(0)) continue;
            T bv = bf[f];
            if (bscale) bv *= (T)bscale[f];
            acc += bv - apply7(F, fb, f, i, j, k, xf);
        }
    }
    bc[t] = acc;
}

// x_out = x_in + alpha x_c(aggregate of f) on active fine points (x_out may alias x_in)
template <typename T>
__global__ void mg_prolong(MGLevelDev<T> F, const T* xin, T* xf, MGLevelDev<T> C, const T* __restrict__ xc, T alpha) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= F.total) return;
    if (F.dinv[t] == T(0)) { xf[t] = T(0); return; }
    const int b = find_block(F, t);
    const MGBlockDesc& fb = F.blk[b];
    const MGBlockDesc& cb = C.blk[b];
    long long q = t - fb.off;
    int i, j, k;
    mg_ijk(q, fb.n1, fb.n2, i, j, k);
    xf[t] = xin[t] + alpha * xc[cb.off + (i >> 1) + (long long)(j >> 1) * cb.n1 + (long long)(k >> 1) * cb.n1 * cb.n2];
}

// coarsest level: x = Minv b per block, dense FP64 (one CTA per block)
template <typename T>
__global__ void mg_dense(MGLevelDev<T> L, const double* __restrict__ minv, const long long* __restrict__ moff,
                         const T* __restrict__ b, T* __restrict__ x, int mask_v) {
    const int blk = blockIdx.x;
    const MGBlockDesc& B = L.blk[blk];
    const int m = B.n1 * B.n2 * B.n3;
    const double* M = minv + moff[blk];
    for (int r = threadIdx.x; r < m; r += blockDim.x) {
        double acc = 0.0;
        if (!(mask_v && blk == L.nb - 1))
            for (int c = 0; c < m; c++) acc += M[(long long)r * m + c] * (double)b[B.off + c];
        x[B.off + r] = (T)acc;
    }
}


// ------------------------------------------------------------------ coarse tail
// The last levels of a cycle (a few thousand points per block at most) in one launch: one CTA
// per block runs their whole V-cycle for that block, passes separated by __syncthreads, the
// data L2-resident.  These levels otherwise cost a launch per sweep, most of it latency.
#define MG_TAIL_MAX_LEVELS 8
template <typename T>
struct MGTail {
    int nl;                                     // tail levels; the last is the coarsest
    MGLevelDev<T> L[MG_TAIL_MAX_LEVELS];
};

template <typename T>
__global__ void __launch_bounds__(1024) mg_tail(MGTail<T> tl, const double* __restrict__ minv,
                                                const long long* __restrict__ moff, T omega, T alpha, int nu1,
                                                int nu2, int mask_v) {
    const int b = blockIdx.x;
    const int nb = tl.L[0].nb;
    const bool masked = mask_v && b == nb - 1;
    T* xcur[MG_TAIL_MAX_LEVELS];
    T* tcur[MG_TAIL_MAX_LEVELS];
    auto npts = [&](const MGBlockDesc& B) { return (long long)B.n1 * B.n2 * B.n3; };
    // x_out = x_in + omega D^-1 (b - A x_in) over the block's points
    auto sweep = [&](const MGLevelDev<T>& L, const T* xin, T* xout) {
        const MGBlockDesc& B = L.blk[b];
        const long long n = npts(B);
        for (long long q = threadIdx.x; q < n; q += blockDim.x) {
            const long long t = B.off + q;
            const T di = masked ? T(0) : L.dinv[t];
            if (di == T(0)) { xout[t] = T(0); continue; }
            int i, j, k;
            mg_ijk(q, B.n1, B.n2, i, j, k);
            xout[t] = xin[t] + omega * di * (L.b[t] - apply7(L, B, t, i, j, k, xin));
        }
        __syncthreads();
    };
    const int last = tl.nl - 1;
    for (int l = 0; l < last; l++) {
        const MGLevelDev<T>& L = tl.L[l];
        const MGBlockDesc& B = L.blk[b];
        const long long n = npts(B);
        T* x = L.x;
        T* t = L.t;
        for (long long q = threadIdx.x; q < n; q += blockDim.x) {
            const long long p = B.off + q;
            x[p] = masked ? T(0) : omega * L.dinv[p] * L.b[p];
        }
        __syncthreads();
        for (int s = 1; s < nu1; s++) {
            sweep(L, x, t);
            T* w = x; x = t; t = w;
        }
        xcur[l] = x;
        tcur[l] = t;
        // residual summed over each 2x2x2 aggregate -> the next level's right-hand side
        const MGLevelDev<T>& C = tl.L[l + 1];
        const MGBlockDesc& cb = C.blk[b];
        const long long nc = npts(cb);
        for (long long q = threadIdx.x; q < nc; q += blockDim.x) {
            int I, J, K;
            mg_ijk(q, cb.n1, cb.n2, I, J, K);
            T acc = T(0);
            if (!masked)
                for (int dk = 0; dk < 2; dk++) for (int dj = 0; dj < 2; dj++) for (int dd = 0; dd < 2; dd++) {
                    const int i = 2 * I + dd, j = 2 * J + dj, k = 2 * K + dk;
                    if (i >= B.n1 || j >= B.n2 || k >= B.n3) continue;
                    const long long f = B.off + i + (long long)j * B.n1 + (long long)k * B.n1 * B.n2;
                    if (L.dinv[f] == T(0)) continue;
                    acc += L.b[f] - apply7(L, B, f, i, j, k, x);
                }
            C.b[cb.off + q] = acc;
        }
        __syncthreads();
    }
    {   // coarsest: x = Minv b (FP64 dense; pseudo-inverse for V)
        const MGLevelDev<T>& C = tl.L[last];
        const MGBlockDesc& B = C.blk[b];
        const int m = (int)npts(B);
        const double* M = minv + moff[b];
        for (int r = threadIdx.x; r < m; r += blockDim.x) {
            double acc = 0.0;
            if (!masked)
                for (int c = 0; c < m; c++) acc += M[(long long)r * m + c] * (double)C.b[B.off + c];
            C.x[B.off + r] = (T)acc;
        }
        xcur[last] = C.x;
        __syncthreads();
    }
    for (int l = last - 1; l >= 0; l--) {
        const MGLevelDev<T>& L = tl.L[l];
        const MGLevelDev<T>& C = tl.L[l + 1];
        const MGBlockDesc& B = L.blk[b];
        const MGBlockDesc& cb = C.blk[b];
        const long long n = npts(B);
        T* x = xcur[l];
        T* t = tcur[l];
        const T* xc = xcur[l + 1];
        for (long long q = threadIdx.x; q < n; q += blockDim.x) {
            const long long p = B.off + q;
            if (L.dinv[p] == T(0) || masked) { x[p] = T(0); continue; }
            int i, j, k;
            mg_ijk(q, B.n1, B.n2, i, j, k);
            x[p] += alpha * xc[cb.off + (i >> 1) + (long long)(j >> 1) * cb.n1 + (long long)(k >> 1) * cb.n1 * cb.n2];
        }
        __syncthreads();
        for (int s = 0; s < nu2; s++) {
            sweep(L, x, t);
            T* w = x; x = t; t = w;
        }
        xcur[l] = x;
    }
    // the level above reads the tail's top level from its x array
    const MGLevelDev<T>& L0 = tl.L[0];
    if (xcur[0] != L0.x) {
        const MGBlockDesc& B = L0.blk[b];
        const long long n = npts(B);
        for (long long q = threadIdx.x; q < n; q += blockDim.x) L0.x[B.off + q] = xcur[0][B.off + q];
    }
}

// ---------------------------------------------------------------------------
// Level-0 kernels on node tiles.  Level 0 of every block is the global unknown
// vector itself, and its 7-point operators are the self couplings of the rows
// of qms_operator.cu, so they read the same staged node coefficients instead
// of stored per-point links:
//   KIND 0: x = omega D^-1 b                      (first sweep, zero guess)
//   KIND 1: x_out = x_in + omega D^-1 (b - A x_in)
//   KIND 3: the first two sweeps from a zero guess in one pass (scaled b only): the
//           first sweep is x_1 = omega isc b pointwise (the diagonal cancels against
//           the row scaling), so b's tile is staged in x_in's place and scaled on use
//   KIND 2: b_c = sum over each 2x2x2 aggregate of (b - A x_in)  (restriction
//           fused with the residual; pairs in i via lane shuffles, in j via
//           shared memory, in k in registers -- no atomics, fixed order)
// b is scaled pointwise by the row scaling of the outer system when bscale is
// given; that scaling is the operator diagonal, formed here from the coefficients.
// x_in is staged in shared memory by cp.async two planes ahead (four
// components, +-1 halo in i and j); b is fetched into registers one plane ahead.
// The kernels are instruction-bound at this arithmetic intensity, so the
// Dirichlet tests are split into a per-thread (i, j) part and a per-plane k
// part, row indices advance by one add per plane, and D^-1 is a fast
// reciprocal in FP32 (a preconditioner needs no correctly rounded divide).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T mg_rcp(T d) {
    if constexpr (sizeof(T) == 4) return __fdividef(1.0f, d);
    else return T(1) / d;
}

// QS selects the blocks a cycle works on: 0 all four, 1 the three A blocks, 2 the V block
// (then only the three conductivities are staged).  xmap / cmap cover exactly those blocks /
// arrays; b, xout and the rows stay those of the whole padded vector, bc that of the level-1
// view of the same blocks.
template <int QS> struct MG0Set {
    static constexpr int NQ = QS == 0 ? 4 : (QS == 1 ? 3 : 1), Q0 = QS == 2 ? 3 : 0;
    static constexpr int NC = QS == 2 ? 3 : 6, C0 = QS == 2 ? 3 : 0;
    static constexpr bool A = QS != 2, V = QS != 1;
};

// Coefficient tiles of the level-0 kernels: bf16 in an FP32 hierarchy (a preconditioner needs
// no more than its ~3 significant digits, and the six node coefficients are 40 % of a sweep's
// DRAM traffic in FP32), the hierarchy's own type in FP64.
template <typename T> struct MG0Coef { using type = T; };
template <> struct MG0Coef<float> { using type = __nv_bfloat16; };
__device__ __forceinline__ float mg_cf(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ double mg_cf(double v) { return v; }

template <typename T, int KIND, int QS>
__global__ void __launch_bounds__(OTX * OTY, sizeof(T) == 4 ? QMS_STENCIL_MINB : 2)
mg0_tiled(QGrid g, QStepPar<T> P, T vshift, T omega, int mask_v, const T* __restrict__ b, int scaled,
          const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap cmap, T* __restrict__ xout,
          MGLevelDev<T> C, T* __restrict__ bc, unsigned* __restrict__ err) {
    using S = MG0Set<QS>;
    using CT = typename MG0Coef<T>::type;
    using TL = PLTiles<T, S::NQ, S::NC, CT>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* xsm = reinterpret_cast<T*>(smem_raw);                  // [4 slots][NQ][PLXY][PLX]
    CT* csm = reinterpret_cast<CT*>(smem_raw + 4 * TL::XSLOT * sizeof(T));   // [3 slots][NC][PLCY][CX]
    __shared__ __align__(8) uint64_t xbar[4], cbar[3];
    __shared__ T red[KIND == 2 ? S::NQ : 1][OTY][OTX];
    constexpr bool STAGE = KIND != 0;
    const int tid = threadIdx.x + OTX * threadIdx.y;
    const int i0 = blockIdx.x * OTX + 1, j0 = blockIdx.y * OTY + 1, k0 = blockIdx.z * OKB + 1;
    const int li = threadIdx.x + 1, lj = threadIdx.y + 1;
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    const bool inij = i <= g.Nx && j <= g.Ny;
    const int kend = min(k0 + OKB - 1, g.Nz);
    const QPL L = qms_pl(g);
    const int cx = i0 - 1, cy = j0 - 2;
    auto issue_x = [&](int kk) {
        const int sl = kk & 3;
        mbar_expect_tx(&xbar[sl], TL::XBYTES);
        tma_load_4d(xsm + sl * TL::XSLOT, &xmap, cx, cy, kk - 1, 0, &xbar[sl]);
    };
    auto issue_c = [&](int kk) {
        const int sl = kk % 3;
        mbar_expect_tx(&cbar[sl], TL::CBYTES);
        tma_load_4d(csm + sl * TL::CSLOT, &cmap, cx, cy, kk - 1, 0, &cbar[sl]);
    };
    auto xpar = [&](int kk) { return (unsigned)(((kk - (k0 - 1)) >> 2) & 1); };
    auto cpar = [&](int kk) { return (unsigned)(((kk - (k0 - 1)) / 3) & 1); };
    if (tid == 0) {
        for (int q = 0; q < 4; q++) mbar_init(&xbar[q], 1);
        for (int q = 0; q < 3; q++) mbar_init(&cbar[q], 1);
        fence_mbar_init();
        if (STAGE) {
            issue_x(k0 - 1);
            issue_x(k0);
            issue_x(k0 + 1);
        }
        issue_c(k0 - 1);
        issue_c(k0);
    }
    __syncthreads();
    bool ok = mbar_wait(&cbar[(k0 - 1) % 3], cpar(k0 - 1), err);
    if (STAGE) ok = ok && mbar_wait(&xbar[(k0 - 1) & 3], xpar(k0 - 1), err) && mbar_wait(&xbar[k0 & 3], xpar(k0), err);
    // per-thread parts of the component predicates (qFixX/Y/Z/V without their k terms)
    const bool exX = inij && i <= g.xs, exY = inij && j <= g.ys;
    const bool fxA = i <= 2 || i >= g.Nx - 1, fyA = j <= 2 || j >= g.Ny - 1;
    const bool fijX = fyA || i == 1 || i == g.xs;
    const bool fijY = fxA || j == 1 || j == g.ys;
    const bool fijZ = fxA || fyA;
    const bool fijV = fxA || fyA || mask_v;
    // node offset at plane k0 (padded layout); block q's row is q * comp + node
    long long nd = inij ? qms_pl_node(g, L, i, j, k0) : 0;
    const long long plane = (long long)g.Ny * L.P;
    const T iscV = scaled ? T(1) / (T(1) + vshift) : T(1);
    T acc[4] = {T(0), T(0), T(0), T(0)};
    // right-hand side of this thread's four rows, fetched one plane ahead so that the loads
    // are in flight while the previous plane is computed.  The row scaling of the outer
    // system is the operator's diagonal, which is this level's diagonal d divided by dscale
    // (1 + vshift on V, 1 on A): it is formed from the staged coefficients, not read.
    T bn0 = T(0), bn1 = T(0), bn2 = T(0), bn3 = T(0);
    auto fetch_b = [&](int kk, long long n) {
        if (S::A) {
            bn0 = exX ? __ldg(b + n) : T(0);
            bn1 = exY ? __ldg(b + L.comp + n) : T(0);
            bn2 = inij && kk <= g.zs ? __ldg(b + 2 * L.comp + n) : T(0);
        }
        if (S::V) bn3 = inij && !mask_v ? __ldg(b + 3 * L.comp + n) : T(0);
    };
    fetch_b(k0, nd);
    for (int k = k0; k <= kend; k++) {
        const T b0 = bn0, b1 = bn1, b2 = bn2, b3 = bn3;
        if (k < kend) fetch_b(k + 1, nd + plane);
        if (!__syncthreads_and(ok)) break;         // slots of plane k-2 free; uniform stop on a lost copy
        if (tid == 0) {
            fence_proxy_async();
            if (STAGE && k + 2 <= kend + 1) issue_x(k + 2);
            if (k < kend) issue_c(k + 1);
        }
        ok = mbar_wait(&cbar[k % 3], cpar(k), err);
        if (STAGE) ok = ok && mbar_wait(&xbar[(k + 1) & 3], xpar(k + 1), err);
        const T* xm = xsm + ((k - 1) & 3) * TL::XSLOT;
        const T* x0 = xsm + (k & 3) * TL::XSLOT;
        const T* xp = xsm + ((k + 1) & 3) * TL::XSLOT;
        const CT* cprv = csm + ((k - 1) % 3) * TL::CSLOT;
        const CT* ccur = csm + (k % 3) * TL::CSLOT;
        const bool kfA = k <= 2 || k >= g.Nz - 1;       // k terms of qFixX / qFixY / qFixV
        const bool kfZ = k == 1 || k == g.zs;           // k term of qFixZ
#define CF(q, dk, dj, di) \
    ((T)mg_cf((dk < 0 ? cprv : ccur)[((q) - S::C0) * PLCY * TL::CX + (lj + (dj)) * TL::CX + li + (di)]))
#define XS(q, sl, dj, di) (sl)[((q) - S::Q0) * PLXY * PLX + (lj + (dj)) * PLX + li + (di)]
        T r[4] = {T(0), T(0), T(0), T(0)};
        // one component: links (wxp, wxm, wyp, wym, wzp, wzm), extra diagonal
        auto point = [&](int q, bool exists, bool fixed, long long row, T bq, T wxp, T wxm, T wyp, T wym, T wzp,
                         T wzm, T dextra, T dscale, T isc) {
            if (!exists) return;
            if (fixed) {
                if (KIND != 2) xout[row] = T(0);
                return;
            }
            const T d = (wxp + wxm + wyp + wym + wzp + wzm + dextra) * dscale;
            const T bv = scaled ? bq * d * isc : bq;
            if (KIND == 0) {
                xout[row] = omega * bv * mg_rcp(d);
                return;
            }
            const T xs = XS(q, x0, 0, 0);
            // difference form (rounding scales with the variation of x): d - sum(w) is the mass
            // term, or the diagonal shift of V
            const T Axs = wxp * (xs - XS(q, x0, 0, 1)) + wxm * (xs - XS(q, x0, 0, -1)) + wyp * (xs - XS(q, x0, 1, 0)) +
                          wym * (xs - XS(q, x0, -1, 0)) + wzp * (xs - XS(q, xp, 0, 0)) + wzm * (xs - XS(q, xm, 0, 0)) +
                          (dextra * dscale + (wxp + wxm + wyp + wym + wzp + wzm) * (dscale - T(1))) * xs;
            // KIND 3: the staged values are b; x_1 = c b with c = omega isc, and A x_1 = c A b
            const T cq = KIND == 3 ? omega * isc : T(1);
            const T xc = cq * xs, Ax = cq * Axs;
            if (KIND == 2) r[q - S::Q0] = bv - Ax;
            else xout[row] = xc + omega * (bv - Ax) * mg_rcp(d);
        };
        if constexpr (S::A) {
        point(0, exX, fijX || kfA, nd, b0,
              CF(0, 0, 0, 0) * P.idx2, CF(0, 0, 0, -1) * P.idx2, CF(2, 0, 0, 0) * P.idy2,
              CF(2, 0, -1, 0) * P.idy2, CF(1, 0, 0, 0) * P.idz2, CF(1, -1, 0, 0) * P.idz2,
              CF(3, 0, 0, 0) * P.idt, T(1), T(1));
        point(1, exY, fijY || kfA, L.comp + nd, b1,
              CF(2, 0, 0, 0) * P.idx2, CF(2, 0, 0, -1) * P.idx2, CF(1, 0, 0, 0) * P.idy2,
              CF(1, 0, -1, 0) * P.idy2, CF(0, 0, 0, 0) * P.idz2, CF(0, -1, 0, 0) * P.idz2,
              CF(4, 0, 0, 0) * P.idt, T(1), T(1));
        point(2, inij && k <= g.zs, fijZ || kfZ, 2 * L.comp + nd, b2,
              CF(1, 0, 0, 0) * P.idx2, CF(1, 0, 0, -1) * P.idx2, CF(0, 0, 0, 0) * P.idy2,
              CF(0, 0, -1, 0) * P.idy2, CF(2, 0, 0, 0) * P.idz2, CF(2, -1, 0, 0) * P.idz2,
              CF(5, 0, 0, 0) * P.idt, T(1), T(1));
        }
        if constexpr (S::V) {
            const T fl = P.sigfloor;
            point(3, inij, fijV || kfA, 3 * L.comp + nd, b3,
                  fmax(CF(3, 0, 0, 0), fl) * P.idx2, fmax(CF(3, 0, 0, -1), fl) * P.idx2,
                  fmax(CF(4, 0, 0, 0), fl) * P.idy2, fmax(CF(4, 0, -1, 0), fl) * P.idy2,
                  fmax(CF(5, 0, 0, 0), fl) * P.idz2, fmax(CF(5, -1, 0, 0), fl) * P.idz2, T(0), T(1) + vshift, iscV);
        }
#undef CF
#undef XS
        nd += plane;
        if (KIND == 2) {
#pragma unroll
            for (int q = 0; q < S::NQ; q++) {
                r[q] += __shfl_xor_sync(0xffffffffu, r[q], 1);            // i pairs (2p+1, 2p+2)
                red[q][threadIdx.y][threadIdx.x] = r[q];
            }
            __syncthreads();
            if (!(threadIdx.x & 1) && !(threadIdx.y & 1)) {
                const bool first = ((k - k0) & 1) == 0;                    // k pairs (odd, even)
#pragma unroll
                for (int q = 0; q < S::NQ; q++) {
                    const T v = red[q][threadIdx.y][threadIdx.x] + red[q][threadIdx.y + 1][threadIdx.x];
                    acc[q] = first ? v : acc[q] + v;
                }
                if (!first || k == kend) {
                    const int I = (i - 1) >> 1, J = (j - 1) >> 1, K = (k - 1) >> 1;
#pragma unroll
                    for (int q = 0; q < S::NQ; q++) {
                        const MGBlockDesc& cb = C.blk[q];
                        if (I < cb.n1 && J < cb.n2 && K < cb.n3)
                            bc[cb.off + I + (long long)J * cb.n1 + (long long)K * cb.n1 * cb.n2] =
                                (mask_v && q + S::Q0 == 3) ? T(0) : acc[q];
                    }
                }
            }
        }
    }
}

// level 0: x += alpha P x_c on the active points (the Dirichlet points of every component,
// and V when masked, stay zero); one thread per node (i, j, k), its (up to) four unknowns
// in the padded layout
// (C and xc: the level-1 view of the blocks of QS)
template <typename T, int QS>
__global__ void mg0_prolong(QGrid g, int mask_v, T* __restrict__ x, MGLevelDev<T> C, const T* __restrict__ xc,
                            T alpha) {
    using S = MG0Set<QS>;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const int I = (i - 1) >> 1, J = (j - 1) >> 1, K = (k - 1) >> 1;
    auto coarse = [&](int q) {
        const MGBlockDesc& cb = C.blk[q - S::Q0];
        return xc[cb.off + I + (long long)J * cb.n1 + (long long)K * cb.n1 * cb.n2];
    };
    const QPL L = qms_pl(g);
    const long long nd = qms_pl_node(g, L, i, j, k);
    if (S::A) {
        if (i <= g.xs && !qFixX(g, i, j, k)) x[nd] += alpha * coarse(0);
        if (j <= g.ys && !qFixY(g, i, j, k)) x[L.comp + nd] += alpha * coarse(1);
        if (k <= g.zs && !qFixZ(g, i, j, k)) x[2 * L.comp + nd] += alpha * coarse(2);
    }
    if (S::V && !mask_v && !qFixV(g, i, j, k)) x[3 * L.comp + nd] += alpha * coarse(3);
}

template <typename T, int KIND, int QS = 0>
static size_t mg0_smem() {
    return PLTiles<T, MG0Set<QS>::NQ, MG0Set<QS>::NC, typename MG0Coef<T>::type>::SMEM;
}

// raise the dynamic shared-memory limit of the level-0 kernels once per device
template <typename T>
static void mg0_prepare() {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
#define ATTR(K, Q) \
    cudaFuncSetAttribute(mg0_tiled<T, K, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mg0_smem<T, K, Q>())
    ATTR(0, 0); ATTR(1, 0); ATTR(2, 0);
    ATTR(0, 1); ATTR(1, 1); ATTR(2, 1); ATTR(3, 1);
    ATTR(0, 2); ATTR(1, 2); ATTR(2, 2); ATTR(3, 2);
#undef ATTR
    done.fetch_or(bit, std::memory_order_acq_rel);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Cyclic Jacobi eigen-decomposition of a symmetric m x m matrix (row-major, in
// place): on return A's diagonal holds the eigenvalues and V the eigenvectors
// (columns).
static void sym_eig_jacobi(int m, std::vector<double>& A, std::vector<double>& V) {
    V.assign((size_t)m * m, 0.0);
    for (int q = 0; q < m; q++) V[(size_t)q * m + q] = 1.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int p = 0; p < m; p++)
            for (int q = 0; q < m; q++) {
                double a = A[(size_t)p * m + q];
                tot += a * a;
                if (p != q) off += a * a;
            }
        if (off <= 1e-30 * tot) break;
        for (int p = 0; p < m - 1; p++)
            for (int q = p + 1; q < m; q++) {
                const double apq = A[(size_t)p * m + q];
                if (std::fabs(apq) < 1e-300) continue;
                const double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < m; k++) {       // columns p, q
                    double akp = A[(size_t)k * m + p], akq = A[(size_t)k * m + q];
                    A[(size_t)k * m + p] = c * akp - sn * akq;
                    A[(size_t)k * m + q] = sn * akp + c * akq;
                }
                for (int k = 0; k < m; k++) {       // rows p, q
                    double apk = A[(size_t)p * m + k], aqk = A[(size_t)q * m + k];
                    A[(size_t)p * m + k] = c * apk - sn * aqk;
                    A[(size_t)q * m + k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < m; k++) {
                    double vkp = V[(size_t)k * m + p], vkq = V[(size_t)k * m + q];
                    V[(size_t)k * m + p] = c * vkp - sn * vkq;
                    V[(size_t)k * m + q] = sn * vkp + c * vkq;
                }
            }
    }
}
#define CKM(call)                                                                        \
    do {                                                                                 \
        cudaError_t _e = (call);                                                         \
        if (_e != cudaSuccess) {                                                         \
            err = std::string(#call) + ": " + cudaGetErrorString(_e);                    \
            return -2;                                                                   \
        }                                                                                \
    } while (0)

static inline unsigned nblk(long long n) { return (unsigned)((n + 255) / 256); }

template <typename T>
QmsMG<T>::~QmsMG() { release(); }

template <typename T>
void QmsMG<T>::release() {
    for (auto& L : lv) {
        T* ps[] = {L.w1, L.w2, L.w3, L.dg, L.dinv, L.x, L.b, L.t, L.mass};
        for (T* p : ps) if (p) cudaFree(p);
    }
    lv.clear();
    views[1].clear();
    views[2].clear();
    if (dminv) cudaFree(dminv);
    if (dmoff) cudaFree(dmoff);
    dminv = nullptr; dmoff = nullptr;
}

template <typename T>
int QmsMG<T>::levels_for(const QGrid& g, int min_coarse) {
    int dims[4][3] = {{g.xs, g.Ny, g.Nz}, {g.Nx, g.ys, g.Nz}, {g.Nx, g.Ny, g.zs}, {g.Nx, g.Ny, g.Nz}};
    int n = 0;
    for (;;) {
        n++;
        int mx = 0;
        for (int b = 0; b < 4; b++) mx = std::max({mx, dims[b][0], dims[b][1], dims[b][2]});
        if (mx <= min_coarse || n >= 12) return n;
        for (int b = 0; b < 4; b++) for (int a = 0; a < 3; a++) dims[b][a] = (dims[b][a] + 1) / 2;
    }
}

template <typename T>
size_t QmsMG<T>::bytes_for(const QGrid& g, int min_coarse, bool tiled) {
    // every level stores 9 values per point; a tiled level 0 (stored node coefficients,
    // more than one level) stores none: its x/b are the Krylov vectors and the caller's temporary
    long long dims[4][3] = {{g.xs, g.Ny, g.Nz}, {g.Nx, g.ys, g.Nz}, {g.Nx, g.Ny, g.zs}, {g.Nx, g.Ny, g.Nz}};
    size_t total = 0;
    for (int l = 0; l < 16; l++) {
        long long pts = 0, mx = 0;
        for (int b = 0; b < 4; b++) {
            pts += dims[b][0] * dims[b][1] * dims[b][2];
            mx = std::max({mx, dims[b][0], dims[b][1], dims[b][2]});
        }
        if (mx <= min_coarse) {
            total += (size_t)pts * 9 * sizeof(T);
            total += (size_t)4 * pts * pts * 8 / 4 + 1024;
            break;
        }
        if (!(tiled && l == 0)) total += (size_t)pts * 9 * sizeof(T);
        for (int b = 0; b < 4; b++) for (int a = 0; a < 3; a++) dims[b][a] = (dims[b][a] + 1) / 2;
    }
    return total;
}

template <typename T>
int QmsMG<T>::build(const QGrid& g, const QCoef<T>& c, const QStepPar<T>& P, T vshift, cudaStream_t st) {
    release();
    // level sizes
    int dims[4][3] = {{g.xs, g.Ny, g.Nz}, {g.Nx, g.ys, g.Nz}, {g.Nx, g.Ny, g.zs}, {g.Nx, g.Ny, g.Nz}};
    for (;;) {
        MGLevelDev<T> L{};
        L.nb = 4;
        long long off = 0;
        int mx = 0;
        for (int b = 0; b < 4; b++) {
            L.blk[b].n1 = dims[b][0]; L.blk[b].n2 = dims[b][1]; L.blk[b].n3 = dims[b][2];
            L.blk[b].off = off;
            off += (long long)dims[b][0] * dims[b][1] * dims[b][2];
            mx = std::max({mx, dims[b][0], dims[b][1], dims[b][2]});
        }
        L.total = off;
        lv.push_back(L);
        if (mx <= min_coarse || (int)lv.size() >= max_levels) break;
        for (int b = 0; b < 4; b++) for (int a = 0; a < 3; a++) dims[b][a] = (dims[b][a] + 1) / 2;
    }
    // With stored node coefficients level 0 runs on node tiles (mg0_tiled) and level 1 is
    // coarsened straight from the coefficients: level 0 keeps no arrays.
    tiled0 = lv.size() > 1 && c.nc != nullptr;
    if (!tiled0) {
        err = "multigrid needs at least two levels and stored node coefficients";
        release();
        return -1;
    }
    for (size_t l = tiled0 ? 1 : 0; l < lv.size(); l++) {
        MGLevelDev<T>& L = lv[l];
        const size_t bytes = L.total * sizeof(T);
        CKM(cudaMalloc(&L.w1, bytes)); CKM(cudaMalloc(&L.w2, bytes)); CKM(cudaMalloc(&L.w3, bytes));
        CKM(cudaMalloc(&L.dg, bytes)); CKM(cudaMalloc(&L.dinv, bytes)); CKM(cudaMalloc(&L.t, bytes));
        CKM(cudaMalloc(&L.mass, bytes));
        if (l > 0) { CKM(cudaMalloc(&L.x, bytes)); CKM(cudaMalloc(&L.b, bytes)); }
    }
    g0 = g; c0 = c; P0 = P; vshift0 = vshift;
    g0block = dim3(OTX, OTY, 1);
    g0grid = dim3((g.Nx + OTX - 1) / OTX, (g.Ny + OTY - 1) / OTY, (g.Nz + OKB - 1) / OKB);
    const double ncut = vcut > 0.0 ? vcut : (sizeof(T) == 8 ? 1e-9 : 1e-5);
    mg_coarsen_fine<<<nblk(lv[1].total), 256, 0, st>>>(g, c, P, vshift, lv[0], lv[1], ncut);
    mg_mask_links<<<nblk(lv[1].total), 256, 0, st>>>(lv[1]);
    for (size_t l = tiled0 ? 2 : 1; l < lv.size(); l++) {
        mg_coarsen<<<nblk(lv[l].total), 256, 0, st>>>(lv[l - 1], lv[l], ncut);
        mg_mask_links<<<nblk(lv[l].total), 256, 0, st>>>(lv[l]);
    }
    CKM(cudaGetLastError());
    // coarsest level: dense inverse per block in FP64 on the host
    MGLevelDev<T>& C = lv.back();
    std::vector<T> w1(C.total), w2(C.total), w3(C.total), dg(C.total), dinv(C.total), mass(C.total);
    CKM(cudaMemcpyAsync(mass.data(), C.mass, C.total * sizeof(T), cudaMemcpyDeviceToHost, st));
    CKM(cudaMemcpyAsync(w1.data(), C.w1, C.total * sizeof(T), cudaMemcpyDeviceToHost, st));
    CKM(cudaMemcpyAsync(w2.data(), C.w2, C.total * sizeof(T), cudaMemcpyDeviceToHost, st));
    CKM(cudaMemcpyAsync(w3.data(), C.w3, C.total * sizeof(T), cudaMemcpyDeviceToHost, st));
    CKM(cudaMemcpyAsync(dg.data(), C.dg, C.total * sizeof(T), cudaMemcpyDeviceToHost, st));
    CKM(cudaMemcpyAsync(dinv.data(), C.dinv, C.total * sizeof(T), cudaMemcpyDeviceToHost, st));
    CKM(cudaStreamSynchronize(st));
    std::vector<long long> moff(C.nb);
    long long mtot = 0;
    for (int b = 0; b < C.nb; b++) {
        long long m = (long long)C.blk[b].n1 * C.blk[b].n2 * C.blk[b].n3;
        moff[b] = mtot;
        mtot += m * m;
    }
    std::vector<double> minv(mtot, 0.0);
    for (int b = 0; b < C.nb; b++) {
        const MGBlockDesc& B = C.blk[b];
        const int m = B.n1 * B.n2 * B.n3;
        std::vector<double> A((size_t)m * m, 0.0), Inv((size_t)m * m, 0.0);
        for (int r = 0; r < m; r++) {
            long long t = B.off + r;
            Inv[(size_t)r * m + r] = 1.0;
            if (dinv[t] == T(0)) { A[(size_t)r * m + r] = 1.0; continue; }
            A[(size_t)r * m + r] = dg[t];
            int i = r % B.n1, j = (r / B.n1) % B.n2, k = r / (B.n1 * B.n2);
            auto link = [&](int nb, T w) { if (w != T(0)) A[(size_t)r * m + nb] -= w; };
            if (i > 0) link(r - 1, w1[t - 1]);
            if (i + 1 < B.n1) link(r + 1, w1[t]);
            if (j > 0) link(r - B.n1, w2[t - B.n1]);
            if (j + 1 < B.n2) link(r + B.n1, w2[t]);
            if (k > 0) link(r - B.n1 * B.n2, w3[t - (long long)B.n1 * B.n2]);
            if (k + 1 < B.n3) link(r + B.n1 * B.n2, w3[t]);
        }
        if (b == C.nb - 1) {
            // V block: pseudo-inverse.  An isolated conductor's potential is pinned only by the
            // 1e-12 S/m floor; on the coarsest grid that is an eigenvalue ~1e-19 of the operator
            // scaled by the summed level-0 diagonals of each point (its stiffness).  Inverting it
            // would amplify round-off without bound, so eigenvalues at or below the cut are
            // dropped (the mode does not enter A or H), and so are the near-null points the
            // coarsening already took out (inactive rows).  Scaling by the point's own Galerkin
            // diagonal instead would hide the mode: a body that collapsed into one point has a
            // diagonal of pure rounding noise and an eigenvalue near 1 in that scaling.
            std::vector<double> dsq(m);
            for (int r = 0; r < m; r++) {
                const long long t = B.off + r;
                dsq[r] = dinv[t] == T(0) ? 1.0 : 1.0 / std::sqrt(std::fabs((double)mass[t]));
            }
            for (int r = 0; r < m; r++)
                for (int q = 0; q < m; q++) A[(size_t)r * m + q] *= dsq[r] * dsq[q];
            for (int r = 0; r < m; r++)             // symmetrise round-off
                for (int q = r + 1; q < m; q++) {
                    double av = 0.5 * (A[(size_t)r * m + q] + A[(size_t)q * m + r]);
                    A[(size_t)r * m + q] = A[(size_t)q * m + r] = av;
                }
            std::vector<double> Q;
            sym_eig_jacobi(m, A, Q);
            for (int r = 0; r < m; r++)
                for (int q = 0; q < m; q++) {
                    double acc = 0.0;
                    for (int e = 0; e < m; e++) {
                        const double lam = A[(size_t)e * m + e];
                        if (lam > ncut) acc += Q[(size_t)r * m + e] * Q[(size_t)q * m + e] / lam;
                    }
                    const bool off_r = dinv[B.off + r] == T(0), off_q = dinv[B.off + q] == T(0);
                    Inv[(size_t)r * m + q] = off_r || off_q ? 0.0 : dsq[r] * acc * dsq[q];
                }
            std::memcpy(&minv[moff[b]], Inv.data(), sizeof(double) * (size_t)m * m);
            continue;
        }
        // A blocks: Gauss-Jordan with partial pivoting
        for (int col = 0; col < m; col++) {
            int piv = col;
            for (int r = col + 1; r < m; r++)
                if (std::fabs(A[(size_t)r * m + col]) > std::fabs(A[(size_t)piv * m + col])) piv = r;
            if (A[(size_t)piv * m + col] == 0.0) { err = "singular coarsest-level operator"; return -1; }
            if (piv != col)
                for (int q = 0; q < m; q++) {
                    std::swap(A[(size_t)piv * m + q], A[(size_t)col * m + q]);
                    std::swap(Inv[(size_t)piv * m + q], Inv[(size_t)col * m + q]);
                }
            const double p = 1.0 / A[(size_t)col * m + col];
            for (int q = 0; q < m; q++) { A[(size_t)col * m + q] *= p; Inv[(size_t)col * m + q] *= p; }
            for (int r = 0; r < m; r++) {
                if (r == col) continue;
                const double f = A[(size_t)r * m + col];
                if (f == 0.0) continue;
                for (int q = 0; q < m; q++) {
                    A[(size_t)r * m + q] -= f * A[(size_t)col * m + q];
                    Inv[(size_t)r * m + q] -= f * Inv[(size_t)col * m + q];
                }
            }
        }
        std::memcpy(&minv[moff[b]], Inv.data(), sizeof(double) * (size_t)m * m);
    }
    CKM(cudaMalloc(&dminv, std::max<long long>(mtot, 1) * 8));
    CKM(cudaMalloc(&dmoff, C.nb * sizeof(long long)));
    CKM(cudaMemcpyAsync(dminv, minv.data(), mtot * 8, cudaMemcpyHostToDevice, st));
    CKM(cudaMemcpyAsync(dmoff, moff.data(), C.nb * sizeof(long long), cudaMemcpyHostToDevice, st));
    CKM(cudaStreamSynchronize(st));
    // views of the three A blocks and of the V block, for cycles on one side of the A-V
    // coupling: same arrays, block table and pointers restricted to those blocks
    views[1].assign(lv.begin(), lv.end());
    views[2].assign(lv.begin(), lv.end());
    for (size_t l = 0; l < lv.size(); l++) {
        const long long o = lv[l].blk[3].off;
        MGLevelDev<T>& A = views[1][l];
        A.nb = 3;
        A.total = o;
        MGLevelDev<T>& V = views[2][l];
        V.nb = 1;
        V.blk[0] = lv[l].blk[3];
        V.blk[0].off = 0;
        V.total = lv[l].total - o;
        T** ps[] = {&V.w1, &V.w2, &V.w3, &V.dg, &V.dinv, &V.x, &V.b, &V.t, &V.mass};
        for (T** q : ps)
            if (*q) *q += o;
    }
    return 0;
}

// z = MG(r): level-0 right-hand side b0 (scaled pointwise by `bscale` when given),
// result in x0; t0 is a level-0 temporary.  Returns the number of kernel launches.
template <typename T>
int QmsMG<T>::vcycle(const T* b0, bool scaled, T* x0, const CUtensorMap& x0map, T* t0, const CUtensorMap& t0map,
                     const CUtensorMap& cmap, bool mask_v, unsigned* err, cudaStream_t st, int qs,
                     const CUtensorMap* b0map) {
    if (qs == 1) return vcycle_q<1>(b0, scaled, x0, x0map, t0, t0map, cmap, mask_v, err, st, b0map);
    if (qs == 2) return vcycle_q<2>(b0, scaled, x0, x0map, t0, t0map, cmap, mask_v, err, st, b0map);
    return vcycle_q<0>(b0, scaled, x0, x0map, t0, t0map, cmap, mask_v, err, st, nullptr);
}

template <typename T>
template <int QS>
int QmsMG<T>::vcycle_q(const T* b0, bool scaled, T* x0, const CUtensorMap& x0map, T* t0, const CUtensorMap& t0map,
                       const CUtensorMap& cmap, bool mask_v, unsigned* err, cudaStream_t st,
                       const CUtensorMap* b0map) {
    int launches = 0;
    std::vector<MGLevelDev<T>>& lv = QS == 0 ? this->lv : views[QS];   // levels >= 1 of the cycle's blocks
    const long long* dmo = dmoff + (QS == 2 ? 3 : 0);                    // their dense coarsest inverses
    const int nl = (int)lv.size();
    const int mv = (QS == 0 && mask_v) ? 1 : 0;
    // sweeps on each side: the V-block cycle may use its own count
    const int n1 = (QS == 2 && nu_v > 0) ? nu_v : nu1, n2 = (QS == 2 && nu_v > 0) ? nu_v : nu2;
    const int sc = scaled ? 1 : 0;
    mg0_prepare<T>();
    struct Buf { T* p; const CUtensorMap* m; };
    // level-0 sweeps: KIND 0 writes XO from b; KIND 1 reads XI (tile copies) and writes XO;
    // KIND 2 reads XI and writes the level-1 right-hand side
#define MG0(KIND, XI, XO, BC)                                                                                     \
    mg0_tiled<T, KIND, QS><<<g0grid, g0block, mg0_smem<T, KIND, QS>(), st>>>(g0, P0, vshift0, omega, mv, b0, sc,  \
                                                                              *(XI).m, \
                                                                       cmap, (XO), lv[1], (BC), err)
    // level 0: nu1 + nu2 sweeps alternate between x0 and t0 (the prolongation is in place);
    // start in t0 when that count is even so that the last write lands in x0
    Buf x{x0, &x0map}, t{t0, &t0map};
    if ((n1 + n2) % 2 == 0) std::swap(x, t);
    int s = 1;
    if (b0map && scaled && QS != 0 && n1 >= 2) {
        // the first two sweeps in one pass, from b's tiles (KIND 3), into the buffer the second
        // sweep writes
        Buf bb{const_cast<T*>(b0), b0map};
        MG0(3, bb, t.p, nullptr);
        std::swap(x, t);
        launches++;
        s = 2;
    } else {
        MG0(0, x, x.p, nullptr);
        launches++;
    }
    // the A-block sweeps are the largest single kernel of a transient step: optionally timed,
    // with their algorithmic bytes (x and b read, x written, one material byte per cell)
    const double asweep_bytes = 3.0 * sizeof(T) * (double)g0.oV + (double)g0.xs * g0.ys * g0.zs;
    auto sweep = [&](Buf& xi, T* xo) {
        void* tok = (QS == 1 && prof) ? prof->begin(MGPROF_A_SWEEP, asweep_bytes) : nullptr;
        MG0(1, xi, xo, nullptr);
        if (tok) prof->end(tok);
    };
    for (; s < n1; s++) {
        sweep(x, t.p);
        std::swap(x, t);
        launches++;
    }
    MG0(2, x, nullptr, lv[1].b);
    launches++;
    // levels >= 1: nu_coarse sweeps on each side when set
    const int nuc1 = (QS == 2 && nu_v > 0) ? nu_v : (nu_coarse > 0 ? nu_coarse : nu1);
    const int nuc2 = (QS == 2 && nu_v > 0) ? nu_v : (nu_coarse > 0 ? nu_coarse : nu2);
    // coarse tail: from level lt on, every level has at most tail_points points per block and
    // the whole sub-cycle runs as one launch (one CTA per block)
    auto maxpts = [](const MGLevelDev<T>& L) {
        long long m = 0;
        for (int q = 0; q < L.nb; q++) m = std::max(m, (long long)L.blk[q].n1 * L.blk[q].n2 * L.blk[q].n3);
        return m;
    };
    int lt = nl - 1;
    if (tail_points > 0)
        while (lt > 1 && maxpts(lv[lt - 1]) <= tail_points && nl - (lt - 1) <= MG_TAIL_MAX_LEVELS) lt--;
    for (int l = 1; l < nl; l++) {
        MGLevelDev<T>& L = lv[l];
        if (l == lt && tail_points > 0) {
            MGTail<T> tl{};
            tl.nl = nl - lt;
            for (int q = 0; q < tl.nl; q++) tl.L[q] = lv[lt + q];
            mg_tail<T><<<L.nb, 1024, 0, st>>>(tl, dminv, dmo, omega, alpha, nuc1, nuc2, mv);
            launches++;
            break;
        }
        if (l == nl - 1) {
            mg_dense<<<L.nb, 256, 0, st>>>(L, dminv, dmo, L.b, L.x, mv);
            launches++;
            break;
        }
        T* xl = L.x;
        T* tl = L.t;
        mg_smooth0<<<nblk(L.total), 256, 0, st>>>(L, L.b, nullptr, omega, xl, mv);
        launches++;
        for (int s = 1; s < nuc1; s++) {
            mg_smooth<<<nblk(L.total), 256, 0, st>>>(L, L.b, nullptr, omega, xl, tl, mv);
            std::swap(xl, tl);
            launches++;
        }
        L.x = xl;
        L.t = tl;
        mg_restrict<<<nblk(lv[l + 1].total), 256, 0, st>>>(L, L.b, nullptr, xl, lv[l + 1], lv[l + 1].b, mv);
        launches++;
    }
    for (int l = lt - 1; l >= 1; l--) {
        MGLevelDev<T>& L = lv[l];
        T* xl = L.x;
        T* tl = L.t;
        mg_prolong<<<nblk(L.total), 256, 0, st>>>(L, xl, xl, lv[l + 1], lv[l + 1].x, alpha);
        launches++;
        for (int s = 0; s < nuc2; s++) {
            mg_smooth<<<nblk(L.total), 256, 0, st>>>(L, L.b, nullptr, omega, xl, tl, mv);
            std::swap(xl, tl);
            launches++;
        }
        L.x = xl;
        L.t = tl;
    }
    mg0_prolong<T, QS><<<qms_node_grid(g0), qms_node_block(), 0, st>>>(g0, mv, x.p, lv[1], lv[1].x, alpha);
    launches++;
    for (int s = 0; s < n2; s++) {
        sweep(x, t.p);
        std::swap(x, t);
        launches++;
    }
#undef MG0
    return launches;
}

template struct QmsMG<float>;
template struct QmsMG<double>;

// ---------------------------------------------------------------------------
// conductor-region coarse space of the V block
// ---------------------------------------------------------------------------
namespace {

// s[r] = sum over the V rows of region r of b * bscale (FP64, fixed order: one CTA per region)
template <typename T>
__global__ void qk_region_sums(const int* __restrict__ ptr, const int* __restrict__ rows, const T* __restrict__ b,
                               const float* __restrict__ bscale, double* __restrict__ s) {
    __shared__ double sh[32];
    const int r = blockIdx.x;
    double acc = 0.0;
    for (int e = ptr[r] + threadIdx.x; e < ptr[r + 1]; e += blockDim.x) {
        const int row = rows[e];
        acc += (double)b[row] * (bscale ? (double)bscale[row] : 1.0);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) s[r] = v;
    }
}

// y = K^+ s (one CTA)
__global__ void qk_region_solve(int K, const double* __restrict__ Kp, const double* __restrict__ s,
                                double* __restrict__ y) {
    for (int r = threadIdx.x; r < K; r += blockDim.x) {
        double acc = 0.0;
        for (int c = 0; c < K; c++) acc += Kp[(long long)r * K + c] * s[c];
        y[r] = acc;
    }
}

// z[row] += y[region of row]
template <typename T>
__global__ void qk_region_scatter(int total, const int* __restrict__ rows, const int* __restrict__ rid,
                                  const double* __restrict__ y, T* __restrict__ z) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < total) z[rows[e]] += (T)y[rid[e]];
}

}  // namespace

QmsRegions::~QmsRegions() { release(); }

void QmsRegions::release() {
    void* ps[] = {ptr, rows, rid, Kp, s, y};
    for (void* p : ps) if (p) cudaFree(p);
    ptr = rows = rid = nullptr;
    Kp = s = y = nullptr;
    K = 0;
}

int QmsRegions::build(const QGrid& g, const uint8_t* slots, const double* rows6, int nmat, double vshift,
                      double cut, cudaStream_t st) {
    release();
    const int xs = g.xs, ys = g.ys, zs = g.zs, Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
    const long long ncell = (long long)xs * ys * zs;
    // per-slot conductivity per axis and its maximum (slot 0: vacuum)
    std::vector<double> sax(3 * (nmat + 1), 0.0), smax(nmat + 1, 0.0);
    for (int r = 0; r < nmat; r++)
        for (int a = 0; a < 3; a++) {
            sax[3 * (r + 1) + a] = rows6[r * 6 + 3 + a];
            smax[r + 1] = std::max(smax[r + 1], rows6[r * 6 + 3 + a]);
        }
    auto cid = [&](int i, int j, int k) { return (long long)(i - 1) + (long long)(j - 1) * xs + (long long)(k - 1) * xs * ys; };
    auto is_cond = [&](long long c) { return smax[slots[c]] > 1.0; };
    // connected bodies: union-find over conductor cells of one slot (6-neighbours)
    std::vector<int> par(ncell, -1);                 // ncell < 2^31 (checked at creation)
    auto find = [&](long long a) -> long long {
        while (par[a] != a) { par[a] = par[par[a]]; a = par[a]; }
        return a;
    };
    for (int k = 1; k <= zs; k++)
        for (int j = 1; j <= ys; j++)
            for (int i = 1; i <= xs; i++) {
                const long long c = cid(i, j, k);
                if (!is_cond(c)) continue;
                par[c] = (int)c;
                const long long nb[3] = {i > 1 ? cid(i - 1, j, k) : -1, j > 1 ? cid(i, j - 1, k) : -1,
                                         k > 1 ? cid(i, j, k - 1) : -1};
                for (long long q : nb)
                    if (q >= 0 && par[q] >= 0 && slots[q] == slots[c]) {
                        const long long ra = find(c), rb = find(q);
                        if (ra != rb) par[std::max(ra, rb)] = (int)std::min(ra, rb);
                    }
            }
    // region of each active V node: body of its incident conductor cell with the largest sigma
    const long long Nn = g.Nn;
    std::vector<int> nreg(Nn, -1);
    std::vector<long long> roots;                   // region index -> body root
    std::vector<long long> count;
    std::map<long long, int> rmap;
    for (int k = 1; k <= Nz; k++)
        for (int j = 1; j <= Ny; j++)
            for (int i = 1; i <= Nx; i++) {
                if (qFixV(g, i, j, k)) continue;
                double best = -1.0;
                long long broot = -1;
                for (int ck = k - 1; ck <= k; ck++)
                    for (int cj = j - 1; cj <= j; cj++)
                        for (int ci = i - 1; ci <= i; ci++) {
                            if (ci < 1 || cj < 1 || ck < 1 || ci > xs || cj > ys || ck > zs) continue;
                            const long long c = cid(ci, cj, ck);
                            if (!is_cond(c)) continue;
                            const long long rt = find(c);
                            const double sv = smax[slots[c]];
                            if (sv > best || (sv == best && rt < broot)) { best = sv; broot = rt; }
                        }
                if (broot < 0) continue;
                auto it = rmap.find(broot);
                int r;
                if (it == rmap.end()) {
                    r = (int)roots.size();
                    rmap[broot] = r;
                    roots.push_back(broot);
                    count.push_back(0);
                } else {
                    r = it->second;
                }
                count[r]++;
                nreg[(i - 1) + (long long)(j - 1) * Nx + (long long)(k - 1) * Nx * Ny] = r;
            }
    int nr = (int)roots.size();
    if (nr == 0) return 0;
    // keep at most QMS_REGION_MAX regions (the largest; ties by first appearance)
    std::vector<int> order(nr), newid(nr, -1);
    for (int r = 0; r < nr; r++) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return count[a] > count[b]; });
    const int Kr = std::min(nr, QMS_REGION_MAX);
    std::vector<int> keep(order.begin(), order.begin() + Kr);
    std::sort(keep.begin(), keep.end());
    for (int q = 0; q < Kr; q++) newid[keep[q]] = q;
    for (long long p = 0; p < Nn; p++)
        if (nreg[p] >= 0) nreg[p] = newid[nreg[p]];
    // Galerkin matrix W^T A_V W from the links crossing region boundaries (no cancellation):
    // link weight max(sigma_edge, floor) / h^2, sigma_edge the mean of the four cells around it
    const double floor_s = (double)1.0e-12f;
    const double ih2[3] = {1.0 / (g.dx * g.dx), 1.0 / (g.dy * g.dy), 1.0 / (g.dz * g.dz)};
    std::vector<double> Km((size_t)Kr * Kr, 0.0);
    std::vector<double> Tr(Kr, 0.0);              // sum of the V-operator diagonal over each region
    auto sig_edge = [&](int a, int i, int j, int k) {
        // edge from node (i,j,k) along axis a: cells with that axis index i/j/k and the other two
        // indices in {n-1, n}
        double acc = 0.0;
        for (int u = 0; u < 2; u++)
            for (int v = 0; v < 2; v++) {
                int ci = i, cj = j, ck = k;
                if (a == 0) { cj = j - 1 + u; ck = k - 1 + v; }
                else if (a == 1) { ci = i - 1 + u; ck = k - 1 + v; }
                else { ci = i - 1 + u; cj = j - 1 + v; }
                if (ci < 1 || cj < 1 || ck < 1 || ci > xs || cj > ys || ck > zs) continue;
                acc += sax[3 * slots[cid(ci, cj, ck)] + a];
            }
        return 0.25 * acc;
    };
    for (int k = 1; k <= Nz; k++)
        for (int j = 1; j <= Ny; j++)
            for (int i = 1; i <= Nx; i++) {
                const long long p = (i - 1) + (long long)(j - 1) * Nx + (long long)(k - 1) * Nx * Ny;
                for (int a = 0; a < 3; a++) {
                    const int i2 = i + (a == 0), j2 = j + (a == 1), k2 = k + (a == 2);
                    if (i2 > Nx || j2 > Ny || k2 > Nz) continue;
                    const long long q = (i2 - 1) + (long long)(j2 - 1) * Nx + (long long)(k2 - 1) * Nx * Ny;
                    const int R = nreg[p], S = nreg[q];
                    if (R < 0 && S < 0) continue;
                    const double w = std::max(sig_edge(a, i, j, k), floor_s) * ih2[a];
                    if (R >= 0) Tr[R] += (1.0 + vshift) * w;
                    if (S >= 0) Tr[S] += (1.0 + vshift) * w;
                    if (vshift != 0.0) {
                        if (R >= 0) Km[(size_t)R * Kr + R] += vshift * w;
                        if (S >= 0) Km[(size_t)S * Kr + S] += vshift * w;
                    }
                    if (R == S) continue;
                    if (R >= 0) Km[(size_t)R * Kr + R] += w;
                    if (S >= 0) Km[(size_t)S * Kr + S] += w;
                    if (R >= 0 && S >= 0) {
                        Km[(size_t)R * Kr + S] -= w;
                        Km[(size_t)S * Kr + R] -= w;
                    }
                }
            }
    // pseudo-inverse, scaled by each region's own stiffness T_R (the sum of the V-operator
    // diagonal over its nodes), so that its eigenvalues compare with those of the row-scaled
    // fine operator: the constant of an isolated conductor (coupled only through the floor)
    // lands near 1e-19 and is dropped, a body attached to others through a few edges keeps
    // its small but resolvable eigenvalue.  `cut` bounds the amplification 1/lambda to what
    // the inner vectors' precision carries.
    std::vector<double> dsq(Kr), A((size_t)Kr * Kr), Q;
    for (int r = 0; r < Kr; r++) dsq[r] = Tr[r] > 0 ? 1.0 / std::sqrt(Tr[r]) : 0.0;
    for (int r = 0; r < Kr; r++)
        for (int c = 0; c < Kr; c++) A[(size_t)r * Kr + c] = Km[(size_t)r * Kr + c] * dsq[r] * dsq[c];
    sym_eig_jacobi(Kr, A, Q);
    std::vector<double> Kpi((size_t)Kr * Kr, 0.0);
    int kept = 0;
    for (int e = 0; e < Kr; e++) {
        const double lam = A[(size_t)e * Kr + e];
        if (!(lam > cut)) continue;
        kept++;
        for (int r = 0; r < Kr; r++)
            for (int c = 0; c < Kr; c++)
                Kpi[(size_t)r * Kr + c] += Q[(size_t)r * Kr + e] * Q[(size_t)c * Kr + e] / lam;
    }
    if (kept == 0) return 0;                          // only null modes: nothing to add
    for (int r = 0; r < Kr; r++)
        for (int c = 0; c < Kr; c++) Kpi[(size_t)r * Kr + c] *= dsq[r] * dsq[c];
    // node lists, region by region
    std::vector<int> hptr(Kr + 1, 0), hrows, hrid;
    for (long long p = 0; p < Nn; p++)
        if (nreg[p] >= 0) hptr[nreg[p] + 1]++;
    for (int r = 0; r < Kr; r++) hptr[r + 1] += hptr[r];
    hrows.resize(hptr[Kr]);
    hrid.resize(hptr[Kr]);
    std::vector<int> fill(hptr.begin(), hptr.end() - 1);
    const QPL L = qms_pl(g);                        // rows in the inner solver's padded layout
    for (long long p = 0; p < Nn; p++)
        if (nreg[p] >= 0) {
            const int r = nreg[p];
            const int i = (int)(p % Nx) + 1, j = (int)((p / Nx) % Ny) + 1, k = (int)(p / ((long long)Nx * Ny)) + 1;
            hrows[fill[r]] = (int)(3 * L.comp + qms_pl_node(g, L, i, j, k));
            hrid[fill[r]] = r;
            fill[r]++;
        }
    const int total = hptr[Kr];
    if (cudaMalloc(&ptr, (Kr + 1) * sizeof(int)) != cudaSuccess || cudaMalloc(&rows, total * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&rid, total * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&Kp, (size_t)Kr * Kr * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&s, Kr * sizeof(double)) != cudaSuccess || cudaMalloc(&y, Kr * sizeof(double)) != cudaSuccess) {
        err = "out of device memory (region coarse space)";
        release();
        return -1;
    }
    cudaMemcpyAsync(ptr, hptr.data(), (Kr + 1) * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(rows, hrows.data(), total * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(rid, hrid.data(), total * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(Kp, Kpi.data(), (size_t)Kr * Kr * sizeof(double), cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {   // the host vectors go out of scope
        err = "region coarse space upload failed";
        release();
        return -1;
    }
    K = Kr;
    total_entries = total;
    return 0;
}

template <typename T>
void QmsRegions::apply(const T* b, const float* bscale, T* z, cudaStream_t st, long long& launches) {
    if (K == 0) return;
    qk_region_sums<T><<<K, 256, 0, st>>>(ptr, rows, b, bscale, s);
    qk_region_solve<<<1, 256, 0, st>>>(K, Kp, s, y);
    const int total = total_entries;
    qk_region_scatter<T><<<(total + 255) / 256, 256, 0, st>>>(total, rows, rid, y, z);
    launches += 3;
}
template void QmsRegions::apply<float>(const float*, const float*, float*, cudaStream_t, long long&);
template void QmsRegions::apply<double>(const double*, const float*, double*, cudaStream_t, long long&);
