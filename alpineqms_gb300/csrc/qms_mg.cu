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

#include <cmath>
#include <cstring>
#include <vector>

namespace {

template <typename T>
__device__ __forceinline__ int find_block(const MGLevelDev<T>& L, long long t) {
    int b = 0;
#pragma unroll
    for (int q = 1; q < MG_MAX_BLOCKS; q++)
        if (q < L.nb && t >= L.blk[q].off) b = q;
    return b;
}

// ---------------------------------------------------------------- fine level
template <typename T>
__global__ void mg_fine_coef(QGrid g, QCoef<T> c, QStepPar<T> P, T vshift, MGLevelDev<T> L) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.total) return;
    const int b = find_block(L, t);
    const MGBlockDesc& B = L.blk[b];
    long long q = t - B.off;
    const int i = (int)(q % B.n1) + 1;
    const int j = (int)((q / B.n1) % B.n2) + 1;
    const int k = (int)(q / ((long long)B.n1 * B.n2)) + 1;
    T w1 = 0, w2 = 0, w3 = 0, d = 1;
    bool active;
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
    L.w1[t] = w1; L.w2[t] = w2; L.w3[t] = w3;
    L.dg[t] = d;                              // diagonal (including links to Dirichlet points)
    L.dinv[t] = active ? T(1) / d : T(0);     // 0 marks an inactive (Dirichlet) point
}

// -------------------------------------------------------------- coarsening
// coarse point (I,J,K) aggregates fine points (2I..2I+1, 2J..2J+1, 2K..2K+1) (0-based)
template <typename T>
__global__ void mg_coarsen(MGLevelDev<T> F, MGLevelDev<T> C) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.total) return;
    const int b = find_block(C, t);
    const MGBlockDesc& cb = C.blk[b];
    const MGBlockDesc& fb = F.blk[b];
    long long q = t - cb.off;
    const int I = (int)(q % cb.n1), J = (int)((q / cb.n1) % cb.n2), K = (int)(q / ((long long)cb.n1 * cb.n2));
    double d = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0;
    bool any = false;
    const long long s1 = 1, s2 = fb.n1, s3 = (long long)fb.n1 * fb.n2;
    for (int dk = 0; dk < 2; dk++) for (int dj = 0; dj < 2; dj++) for (int di = 0; di < 2; di++) {
        int i = 2 * I + di, j = 2 * J + dj, k = 2 * K + dk;
        if (i >= fb.n1 || j >= fb.n2 || k >= fb.n3) continue;
        long long f = fb.off + i + (long long)j * s2 + (long long)k * s3;
        if (F.dinv[f] == T(0)) continue;
        any = true;
        d += F.dg[f];
        // +x link of f: internal if di == 0, crossing to I+1 if di == 1
        if (i + 1 < fb.n1 && F.dinv[f + s1] != T(0)) {
            if (di == 0) d -= 2.0 * F.w1[f];
            else w1 += F.w1[f];
        }
        if (j + 1 < fb.n2 && F.dinv[f + s2] != T(0)) {
            if (dj == 0) d -= 2.0 * F.w2[f];
            else w2 += F.w2[f];
        }
        if (k + 1 < fb.n3 && F.dinv[f + s3] != T(0)) {
            if (dk == 0) d -= 2.0 * F.w3[f];
            else w3 += F.w3[f];
        }
    }
    C.w1[t] = I + 1 < cb.n1 ? (T)w1 : T(0);
    C.w2[t] = J + 1 < cb.n2 ? (T)w2 : T(0);
    C.w3[t] = K + 1 < cb.n3 ? (T)w3 : T(0);
    C.dg[t] = any ? (T)d : T(1);
    C.dinv[t] = any && d > 0.0 ? (T)(1.0 / d) : T(0);
}

// a crossing link is only kept if both aggregates are active
template <typename T>
__global__ void mg_mask_links(MGLevelDev<T> C) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.total) return;
    const int b = find_block(C, t);
    const MGBlockDesc& cb = C.blk[b];
    long long q = t - cb.off;
    const int I = (int)(q % cb.n1), J = (int)((q / cb.n1) % cb.n2), K = (int)(q / ((long long)cb.n1 * cb.n2));
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
    const int i = (int)(q % B.n1), j = (int)((q / B.n1) % B.n2), k = (int)(q / ((long long)B.n1 * B.n2));
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
    const int I = (int)(q % cb.n1), J = (int)((q / cb.n1) % cb.n2), K = (int)(q / ((long long)cb.n1 * cb.n2));
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
    const int i = (int)(q % fb.n1), j = (int)((q / fb.n1) % fb.n2), k = (int)(q / ((long long)fb.n1 * fb.n2));
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
        T* ps[] = {L.w1, L.w2, L.w3, L.dg, L.dinv, L.x, L.b, L.t};
        for (T* p : ps) if (p) cudaFree(p);
    }
    lv.clear();
    if (dminv) cudaFree(dminv);
    if (dmoff) cudaFree(dmoff);
    dminv = nullptr; dmoff = nullptr;
}

template <typename T>
size_t QmsMG<T>::bytes_for(const QGrid& g, int min_coarse) {
    // every level stores 8 floats per point (level 0 shares x/b with the Krylov vectors but keeps a temp)
    long long dims[4][3] = {{g.xs, g.Ny, g.Nz}, {g.Nx, g.ys, g.Nz}, {g.Nx, g.Ny, g.zs}, {g.Nx, g.Ny, g.Nz}};
    size_t total = 0;
    for (int l = 0; l < 16; l++) {
        long long pts = 0, mx = 0;
        for (int b = 0; b < 4; b++) {
            pts += dims[b][0] * dims[b][1] * dims[b][2];
            mx = std::max({mx, dims[b][0], dims[b][1], dims[b][2]});
        }
        total += (size_t)pts * 8 * sizeof(T);
        if (mx <= min_coarse) {
            total += (size_t)4 * pts * pts * 8 / 4 + 1024;
            break;
        }
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
    for (size_t l = 0; l < lv.size(); l++) {
        MGLevelDev<T>& L = lv[l];
        const size_t bytes = L.total * sizeof(T);
        CKM(cudaMalloc(&L.w1, bytes)); CKM(cudaMalloc(&L.w2, bytes)); CKM(cudaMalloc(&L.w3, bytes));
        CKM(cudaMalloc(&L.dg, bytes)); CKM(cudaMalloc(&L.dinv, bytes)); CKM(cudaMalloc(&L.t, bytes));
        if (l > 0) { CKM(cudaMalloc(&L.x, bytes)); CKM(cudaMalloc(&L.b, bytes)); }
    }
    mg_fine_coef<<<nblk(lv[0].total), 256, 0, st>>>(g, c, P, vshift, lv[0]);
    for (size_t l = 1; l < lv.size(); l++) {
        mg_coarsen<<<nblk(lv[l].total), 256, 0, st>>>(lv[l - 1], lv[l]);
        mg_mask_links<<<nblk(lv[l].total), 256, 0, st>>>(lv[l]);
    }
    CKM(cudaGetLastError());
    // coarsest level: dense inverse per block in FP64 on the host
    MGLevelDev<T>& C = lv.back();
    std::vector<T> w1(C.total), w2(C.total), w3(C.total), dg(C.total), dinv(C.total);
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
            // 1e-12 S/m floor; on the coarsest grid that is an eigenvalue ~1e-19 of the
            // diagonally scaled operator.  Inverting it would amplify round-off without bound,
            // so eigenvalues below 1e-9 are dropped (the mode does not enter A or H).
            std::vector<double> dsq(m);
            for (int r = 0; r < m; r++) dsq[r] = 1.0 / std::sqrt(std::fabs(A[(size_t)r * m + r]));
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
                        if (lam > 1e-9) acc += Q[(size_t)r * m + e] * Q[(size_t)q * m + e] / lam;
                    }
                    Inv[(size_t)r * m + q] = dsq[r] * acc * dsq[q];
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
    return 0;
}

// z = MG(r): level-0 right-hand side b0 (scaled pointwise by `bscale` when given),
// result in x0; t0 is a level-0 temporary.  Returns the number of kernel launches.
template <typename T>
int QmsMG<T>::vcycle(const T* b0, const float* bscale, T* x0, T* t0, bool mask_v, cudaStream_t st) {
    int launches = 0;
    const int nl = (int)lv.size();
    const int mv = mask_v ? 1 : 0;
    for (int l = 0; l < nl; l++) {
        MGLevelDev<T>& L = lv[l];
        const T* b = l == 0 ? b0 : L.b;
        const float* bs = l == 0 ? bscale : nullptr;
        T* x = l == 0 ? x0 : L.x;
        T* t = l == 0 ? t0 : L.t;
        if (l == nl - 1) {
            mg_dense<<<L.nb, 256, 0, st>>>(L, dminv, dmoff, b, x, mv);
            launches++;
            break;
        }
        // pre-smoothing: nu1 Jacobi sweeps from zero; keep the result in x
        mg_smooth0<<<nblk(L.total), 256, 0, st>>>(L, b, bs, omega, x, mv);
        launches++;
        for (int s = 1; s < nu1; s++) {
            mg_smooth<<<nblk(L.total), 256, 0, st>>>(L, b, bs, omega, x, t, mv);
            std::swap(x, t);
            launches++;
        }
        if (l == 0) { cur_x0 = x; cur_t0 = t; }
        else { L.x = x; L.t = t; }
        mg_restrict<<<nblk(lv[l + 1].total), 256, 0, st>>>(L, b, bs, x, lv[l + 1], lv[l + 1].b, mv);
        launches++;
    }
    for (int l = nl - 2; l >= 0; l--) {
        MGLevelDev<T>& L = lv[l];
        const T* b = l == 0 ? b0 : L.b;
        const float* bs = l == 0 ? bscale : nullptr;
        T* x = l == 0 ? cur_x0 : L.x;
        T* t = l == 0 ? cur_t0 : L.t;
        // on level 0 the result must land in x0: the nu2 sweeps alternate buffers, so
        // prolongate out of place when the parity would end in the temporary
        const bool flip = l == 0 && (((nu2 % 2 == 0) ? x : t) != x0);
        if (flip) {
            mg_prolong<<<nblk(L.total), 256, 0, st>>>(L, x, t, lv[l + 1], lv[l + 1].x, alpha);
            std::swap(x, t);
        } else {
            mg_prolong<<<nblk(L.total), 256, 0, st>>>(L, x, x, lv[l + 1], lv[l + 1].x, alpha);
        }
        launches++;
        for (int s = 0; s < nu2; s++) {
            mg_smooth<<<nblk(L.total), 256, 0, st>>>(L, b, bs, omega, x, t, mv);
            std::swap(x, t);
            launches++;
        }
        if (l > 0) { L.x = x; L.t = t; }
    }
    return launches;
}

template struct QmsMG<float>;
template struct QmsMG<double>;
