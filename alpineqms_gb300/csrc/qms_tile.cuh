// qms_tile.cuh -- shared-memory tiles of node coefficients for the stencil kernels.
//
// A CTA of OTX x OTY threads owns a column of nodes (i, j) and marches along k
// over OKB planes.  The six face/edge coefficients of every node (1/mu_x,
// 1/mu_y, 1/mu_z, sigma_x, sigma_y, sigma_z) that the rows of plane k need
// (planes k-1 and k, with a -1 halo in i and j) are staged in a three-plane ring.
#pragma once
#include "qms_common.cuh"
#include "qms_tma.cuh"

#define OTX 32
#define OTY 8
#define OKB 16
// resident CTAs per SM the FP32 stencil kernels are compiled for (caps registers at 64)
#ifndef QMS_STENCIL_MINB
#define QMS_STENCIL_MINB 4
#endif

// three-plane ring: planes k-1 and k are read while plane k+1 is filled, so a
// single barrier per plane separates the fill of one plane from its first use
template <typename T>
struct TileCoef {
    T c[3][6][OTY + 1][OTX + 1];
};
__device__ __forceinline__ int tslot(int k) { return k % 3; }

// x tiles: the four unknown components of planes k-1, k, k+1 (and k+2 in flight) with a
// +-1 halo in i and j, staged by cp.async (zero-filled outside each component's grid)
#define XTX (OTX + 2)
#define XTY (OTY + 2)
template <typename T>
struct XTile {
    T v[4][4][XTY][XTX];          // [slot][component][j][i]
};
__device__ __forceinline__ int xslot(int k) { return k & 3; }

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 8 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// commits any copies still pending in this thread and waits for all of them
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Per-thread staging plan of the x tiles: every thread copies the same (li, lj)
// positions of each component on every plane, so the global offsets of those
// positions on plane 1 are formed once and a plane costs one multiply-add, a
// range test and a cp.async per element.  A plane of one component is
// XTX*XTY = 340 elements: two per thread, the second only for the first 84.
struct XStager {
    int goff[4][2];                  // offset in x of (i, j, k = 1); -1 outside the component
    int soff[2];                     // position in a component plane of the tile
    __device__ __forceinline__ void init(const QGrid& g, int i0, int j0) {
        const int tid = threadIdx.x + OTX * threadIdx.y;
#pragma unroll
        for (int e = 0; e < 2; e++) {
            const int q = tid + OTX * OTY * e;
            const bool ok = q < XTX * XTY;
            const int li = q % XTX, lj = q / XTX;
            const int i = i0 - 1 + li, j = j0 - 1 + lj;
            soff[e] = ok ? lj * XTX + li : -1;
            const int n1[4] = {g.xs, g.Nx, g.Nx, g.Nx}, n2[4] = {g.Ny, g.ys, g.Ny, g.Ny};
            const long long off[4] = {0, g.oY, g.oZ, g.oV};
#pragma unroll
            for (int c = 0; c < 4; c++)
                goff[c][e] = ok && i >= 1 && j >= 1 && i <= n1[c] && j <= n2[c]
                                 ? (int)(off[c] + (i - 1) + (long long)(j - 1) * n1[c]) : -1;
        }
    }
    // issue the copies of plane kk of the four components into slot xslot(kk)
    template <typename T>
    __device__ __forceinline__ void load(const QGrid& g, const T* __restrict__ x, XTile<T>& xt, int kk) const {
        const int sl = xslot(kk);
        const int n3[4] = {g.Nz, g.Nz, g.zs, g.Nz};
        const int pl[4] = {g.xs * g.Ny, g.Nx * g.ys, g.Nx * g.Ny, g.Nx * g.Ny};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const bool kin = kk >= 1 && kk <= n3[c];
            T* dst = &xt.v[sl][c][0][0];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                if (soff[e] < 0) continue;
                const bool v = kin && goff[c][e] >= 0;
                const T* src = v ? x + goff[c][e] + (long long)(kk - 1) * pl[c] : x;
                cp_async_elem(dst + soff[e], src, v);
            }
        }
    }
};

// The same for the node-coefficient tiles (six SoA arrays of Nn nodes, -1 halo):
// (OTX+1)*(OTY+1) = 297 nodes a plane, two per thread, the second for the first 41.
struct CStager {
    int noff[2];                     // node index of (i, j, k = 1); -1 outside the grid
    int soff[2];
    __device__ __forceinline__ void init(const QGrid& g, int i0, int j0) {
        const int tid = threadIdx.x + OTX * threadIdx.y;
#pragma unroll
        for (int e = 0; e < 2; e++) {
            const int q = tid + OTX * OTY * e;
            const bool ok = q < (OTX + 1) * (OTY + 1);
            const int li = q % (OTX + 1), lj = q / (OTX + 1);
            const int i = i0 - 1 + li, j = j0 - 1 + lj;
            soff[e] = ok ? lj * (OTX + 1) + li : -1;
            // node coefficients are stored in the padded layout ([6][Nz][Ny][P], column i)
            noff[e] = ok && i >= 1 && j >= 1 && i <= g.Nx && j <= g.Ny ? i + (j - 1) * qms_pl(g).P : -1;
        }
    }
    // plane k of the six coefficients into slot tslot(k): cp.async from the stored node
    // coefficients, or formed in place from the material slots when none are stored
    template <typename T>
    __device__ __forceinline__ void load(const QCoef<T>& c, TileCoef<T>& tc, int k) const {
        const int sl = tslot(k);
        if (c.nc) {
            const bool kin = k >= 1 && k <= c.g.Nz;
            const QPL L = qms_pl(c.g);
            const long long N = L.comp;
            const long long kb = (long long)(k - 1) * c.g.Ny * L.P;
#pragma unroll
            for (int e = 0; e < 2; e++) {
                if (soff[e] < 0) continue;
                const bool v = kin && noff[e] >= 0;
                const T* src = v ? c.nc + noff[e] + kb : c.nc;
#pragma unroll
                for (int q = 0; q < 6; q++) cp_async_elem(&tc.c[sl][q][0][0] + soff[e], v ? src + q * N : src, v);
            }
        } else {
#pragma unroll
            for (int e = 0; e < 2; e++) {
                if (soff[e] < 0) continue;
                const int li = soff[e] % (OTX + 1), lj = soff[e] / (OTX + 1);
                T v0 = 0, v1 = 0, v2 = 0, v3 = 0, v4 = 0, v5 = 0;
                if (noff[e] >= 0 && k >= 1 && k <= c.g.Nz) {
                    const int P = qms_pl(c.g).P;
                    const int i = noff[e] % P, j = noff[e] / P + 1;
                    v0 = c.imux(i, j, k); v1 = c.imuy(i, j, k); v2 = c.imuz(i, j, k);
                    v3 = c.sgx(i, j, k); v4 = c.sgy(i, j, k); v5 = c.sgz(i, j, k);
                }
                tc.c[sl][0][lj][li] = v0; tc.c[sl][1][lj][li] = v1; tc.c[sl][2][lj][li] = v2;
                tc.c[sl][3][lj][li] = v3; tc.c[sl][4][lj][li] = v4; tc.c[sl][5][lj][li] = v5;
            }
        }
    }
};
