// qms_operator.cu -- matrix-free Yee A-V operator (the production replacement
// of the CSR matrix handed to PARDISO, 3D/QMS_3D.f90:1316, F:2196, F:2201).
//
// One thread per node (i,j) of a tile, marching in k, evaluates the (up to) four rows living there:
// the Ax row (i <= xs), Ay row (j <= ys), Az row (k <= zs) and the V row, with
// the same entries as the assembled CSR (F:476-607, F:650-781, F:824-955,
// F:1014-1285 and the transient additions F:1475-1504, F:1624-1681,
// F:1772-1857, F:1925-2126).  Face 1/mu and edge sigma are formed on the fly
// from the uint8 material slots (qms_common.cuh), so the only HBM traffic is
// the input vector, the output vector and one byte per cell.
//
// Modes:
//   QOP_APPLY   y = M x                       (Dirichlet rows: y = x)
//   QOP_SCALED  y = D^-1 M x, D = diag(M)     (Dirichlet rows: y = x)
//   QOP_RESID   r = D^-1 (b - M x)            (FP64; Dirichlet rows: b - x)
// Optional fused reductions (block partials, FP64):
//   APPLY/SCALED: [0] += y . w, [1] += y . y    (w may be null -> skip)
//   RESID:        [0] += |r_A|^2, [1] += |r_V|^2, [2] += |x_A|^2, [3] += |x_V|^2
#include "qms_internal.h"
#include <algorithm>
#include <type_traits>

enum QOpMode { QOP_APPLY = 0, QOP_SCALED = 1, QOP_RESID = 2 };

// ---------------------------------------------------------------------------
// A CTA of OTX x OTY threads owns a column
// of nodes (i, j) and marches along k over OKB planes.  The six face/edge
// coefficients of every node (1/mu_x, 1/mu_y, 1/mu_z, sigma_x, sigma_y,
// sigma_z), which the rows of plane k need for planes k-1 and k and with a
// -1 halo in i and j, are formed once per node into a two-plane shared-memory
// ring instead of once per use (each coefficient is used by up to 8 rows).
// Unknowns are read through L1; index arithmetic is 32-bit within a block.
// ---------------------------------------------------------------------------
#define OTX 32
#define OTY 8
#define OKB 16

template <typename T>
struct TileCoef {
    T c[2][6][OTY + 1][OTX + 1];
};

template <typename T>
__device__ __forceinline__ void tile_fill_plane(const QCoef<T>& c, TileCoef<T>& tc, int slot, int i0, int j0, int k) {
    const int tid = threadIdx.x + OTX * threadIdx.y;
    for (int q = tid; q < (OTX + 1) * (OTY + 1); q += OTX * OTY) {
        const int li = q % (OTX + 1), lj = q / (OTX + 1);
        const int i = i0 - 1 + li, j = j0 - 1 + lj;
        T v0 = 0, v1 = 0, v2 = 0, v3 = 0, v4 = 0, v5 = 0;
        if (i >= 1 && j >= 1 && k >= 1 && i <= c.g.Nx && j <= c.g.Ny && k <= c.g.Nz) {
            v0 = c.imux(i, j, k); v1 = c.imuy(i, j, k); v2 = c.imuz(i, j, k);
            v3 = c.sgx(i, j, k); v4 = c.sgy(i, j, k); v5 = c.sgz(i, j, k);
        }
        tc.c[slot][0][lj][li] = v0; tc.c[slot][1][lj][li] = v1; tc.c[slot][2][lj][li] = v2;
        tc.c[slot][3][lj][li] = v3; tc.c[slot][4][lj][li] = v4; tc.c[slot][5][lj][li] = v5;
    }
}

template <typename T, bool ADV, int MODE>
__global__ void __launch_bounds__(OTX * OTY)
qk_operator_t(QGrid g, QCoef<T> c, QStepPar<T> P, const T* __restrict__ x, const T* __restrict__ b,
              T* __restrict__ y, const T* __restrict__ w, double* __restrict__ partials) {
    __shared__ TileCoef<T> tc;
    const int i0 = blockIdx.x * OTX + 1, j0 = blockIdx.y * OTY + 1, k0 = blockIdx.z * OKB + 1;
    const int li = threadIdx.x + 1, lj = threadIdx.y + 1;   // position in the coefficient tile
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    const bool inij = i <= g.Nx && j <= g.Ny;
    // block bases and 32-bit strides of the four unknown blocks
    const T* __restrict__ xX = x;
    const T* __restrict__ xY = x + g.oY;
    const T* __restrict__ xZ = x + g.oZ;
    const T* __restrict__ xV = x + g.oV;
    const int sXj = g.xs, sXk = g.xs * g.Ny;      // Ax: (xs, Ny, Nz)
    const int sYj = g.Nx, sYk = g.Nx * g.ys;      // Ay: (Nx, ys, Nz)
    const int sZj = g.Nx, sZk = g.Nx * g.Ny;      // Az: (Nx, Ny, zs); V: (Nx, Ny, Nz)
    using RT = typename std::conditional<MODE == QOP_RESID, double, float>::type;
    RT red0 = 0, red1 = 0, red2 = 0, red3 = 0;
    auto emit = [&](long long row, T acc, T diag, bool is_a) {
        T out;
        if (MODE == QOP_APPLY) out = acc;
        else if (MODE == QOP_SCALED) out = acc / diag;
        else out = (b[row] - acc) / diag;
        y[row] = out;
        if (partials) {
            if (MODE == QOP_RESID) {
                RT o = (RT)out, xv = (RT)__ldg(x + row);
                if (is_a) { red0 += o * o; red2 += xv * xv; }
                else { red1 += o * o; red3 += xv * xv; }
            } else {
                if (w) red0 += (RT)(out * w[row]);
                red1 += (RT)(out * out);
            }
        }
    };
    tile_fill_plane(c, tc, (k0 - 1) & 1, i0, j0, k0 - 1);
    const int kend = min(k0 + OKB - 1, g.Nz);
    for (int k = k0; k <= kend; k++) {
        const int cur = k & 1, prv = (k - 1) & 1;
        tile_fill_plane(c, tc, cur, i0, j0, k);
        __syncthreads();
#define CF(q, s, dj, di) tc.c[s][q][lj + (dj)][li + (di)]
        if (inij) {
            // ---------------------------------------------------------------- Ax
            if (i <= g.xs) {
                const int o = (i - 1) + (j - 1) * sXj + (k - 1) * sXk;
                const long long row = o;
                if (qFixX(g, i, j, k)) {
                    emit(row, __ldg(xX + o), T(1), true);
                } else {
                    const T s = CF(3, cur, 0, 0);
                    const T my_km = CF(1, prv, 0, 0), my_k = CF(1, cur, 0, 0);
                    const T mz_jm = CF(2, cur, -1, 0), mz_j = CF(2, cur, 0, 0);
                    const T mx_im = CF(0, cur, 0, -1), mx_i = CF(0, cur, 0, 0);
                    const T svy = ADV ? s * P.vy : T(0), svz = ADV ? s * P.vz : T(0);
                    const T d = (mz_j + mz_jm) * P.idy2 + (my_k + my_km) * P.idz2 + (mx_i + mx_im) * P.idx2 + s * P.idt;
                    const int oy = (i - 1) + (j - 1) * sYj + (k - 1) * sYk;
                    const int oz = (i - 1) + (j - 1) * sZj + (k - 1) * sZk;
                    T acc = d * __ldg(xX + o);
                    acc += (-my_km * P.idz2 + svz * P.i2dz) * __ldg(xX + o - sXk);
                    acc += (-mz_jm * P.idy2 + svy * P.i2dy) * __ldg(xX + o - sXj);
                    acc += (-mx_im * P.idx2) * __ldg(xX + o - 1);
                    acc += (-mx_i * P.idx2) * __ldg(xX + o + 1);
                    acc += (-mz_j * P.idy2 - svy * P.i2dy) * __ldg(xX + o + sXj);
                    acc += (-my_k * P.idz2 - svz * P.i2dz) * __ldg(xX + o + sXk);
                    acc += (mz_jm * P.idxdy - svy * P.i2dx) * __ldg(xY + oy - sYj);
                    acc += (-mz_jm * P.idxdy + svy * P.i2dx) * __ldg(xY + oy - sYj + 1);
                    acc += (-mz_j * P.idxdy - svy * P.i2dx) * __ldg(xY + oy);
                    acc += (mz_j * P.idxdy + svy * P.i2dx) * __ldg(xY + oy + 1);
                    acc += (my_km * P.idxdz - svz * P.i2dx) * __ldg(xZ + oz - sZk);
                    acc += (-my_km * P.idxdz + svz * P.i2dx) * __ldg(xZ + oz - sZk + 1);
                    acc += (-my_k * P.idxdz - svz * P.i2dx) * __ldg(xZ + oz);
                    acc += (my_k * P.idxdz + svz * P.i2dx) * __ldg(xZ + oz + 1);
                    acc += s * P.idx * (__ldg(xV + oz + 1) - __ldg(xV + oz));
                    emit(row, acc, d, true);
                }
            }
            // ---------------------------------------------------------------- Ay
            if (j <= g.ys) {
                const int o = (i - 1) + (j - 1) * sYj + (k - 1) * sYk;
                const long long row = g.oY + o;
                if (qFixY(g, i, j, k)) {
                    emit(row, __ldg(xY + o), T(1), true);
                } else {
                    const T s = CF(4, cur, 0, 0);
                    const T mz_im = CF(2, cur, 0, -1), mz_i = CF(2, cur, 0, 0);
                    const T mx_km = CF(0, prv, 0, 0), mx_k = CF(0, cur, 0, 0);
                    const T my_jm = CF(1, cur, -1, 0), my_j = CF(1, cur, 0, 0);
                    const T svx = ADV ? s * P.vx : T(0), svz = ADV ? s * P.vz : T(0);
                    const T d = (mz_i + mz_im) * P.idx2 + (mx_k + mx_km) * P.idz2 + (my_j + my_jm) * P.idy2 + s * P.idt;
                    const int ox = (i - 1) + (j - 1) * sXj + (k - 1) * sXk;
                    const int oz = (i - 1) + (j - 1) * sZj + (k - 1) * sZk;
                    T acc = d * __ldg(xY + o);
                    acc += (mz_im * P.idxdy - svx * P.i2dy) * __ldg(xX + ox - 1);
                    acc += (-mz_i * P.idxdy - svx * P.i2dy) * __ldg(xX + ox);
                    acc += (-mz_im * P.idxdy + svx * P.i2dy) * __ldg(xX + ox + sXj - 1);
                    acc += (mz_i * P.idxdy + svx * P.i2dy) * __ldg(xX + ox + sXj);
                    acc += (-mx_km * P.idz2 + svz * P.i2dz) * __ldg(xY + o - sYk);
                    acc += (-my_jm * P.idy2) * __ldg(xY + o - sYj);
                    acc += (-mz_im * P.idx2 + svx * P.i2dx) * __ldg(xY + o - 1);
                    acc += (-mz_i * P.idx2 - svx * P.i2dx) * __ldg(xY + o + 1);
                    acc += (-my_j * P.idy2) * __ldg(xY + o + sYj);
                    acc += (-mx_k * P.idz2 - svz * P.i2dz) * __ldg(xY + o + sYk);
                    acc += (mx_km * P.idydz - svz * P.i2dy) * __ldg(xZ + oz - sZk);
                    acc += (-mx_km * P.idydz + svz * P.i2dy) * __ldg(xZ + oz - sZk + sZj);
                    acc += (-mx_k * P.idydz - svz * P.i2dy) * __ldg(xZ + oz);
                    acc += (mx_k * P.idydz + svz * P.i2dy) * __ldg(xZ + oz + sZj);
                    acc += s * P.idy * (__ldg(xV + oz + sZj) - __ldg(xV + oz));
                    emit(row, acc, d, true);
                }
            }
            // ---------------------------------------------------------------- Az
            if (k <= g.zs) {
                const int o = (i - 1) + (j - 1) * sZj + (k - 1) * sZk;
                const long long row = g.oZ + o;
                if (qFixZ(g, i, j, k)) {
                    emit(row, __ldg(xZ + o), T(1), true);
                } else {
                    const T s = CF(5, cur, 0, 0);
                    const T my_im = CF(1, cur, 0, -1), my_i = CF(1, cur, 0, 0);
                    const T mx_jm = CF(0, cur, -1, 0), mx_j = CF(0, cur, 0, 0);
                    const T mz_km = CF(2, prv, 0, 0), mz_k = CF(2, cur, 0, 0);
                    const T svx = ADV ? s * P.vx : T(0), svy = ADV ? s * P.vy : T(0);
                    const T d = (my_i + my_im) * P.idx2 + (mx_j + mx_jm) * P.idy2 + (mz_k + mz_km) * P.idz2 + s * P.idt;
                    const int ox = (i - 1) + (j - 1) * sXj + (k - 1) * sXk;
                    const int oy = (i - 1) + (j - 1) * sYj + (k - 1) * sYk;
                    T acc = d * __ldg(xZ + o);
                    acc += (my_im * P.idxdz - svx * P.i2dz) * __ldg(xX + ox - 1);
                    acc += (-my_i * P.idxdz - svx * P.i2dz) * __ldg(xX + ox);
                    acc += (-my_im * P.idxdz + svx * P.i2dz) * __ldg(xX + ox + sXk - 1);
                    acc += (my_i * P.idxdz + svx * P.i2dz) * __ldg(xX + ox + sXk);
                    acc += (mx_jm * P.idydz - svy * P.i2dz) * __ldg(xY + oy - sYj);
                    acc += (-mx_j * P.idydz - svy * P.i2dz) * __ldg(xY + oy);
                    acc += (-mx_jm * P.idydz + svy * P.i2dz) * __ldg(xY + oy - sYj + sYk);
                    acc += (mx_j * P.idydz + svy * P.i2dz) * __ldg(xY + oy + sYk);
                    acc += (-mz_km * P.idz2) * __ldg(xZ + o - sZk);
                    acc += (-mx_jm * P.idy2 + svy * P.i2dy) * __ldg(xZ + o - sZj);
                    acc += (-my_im * P.idx2 + svx * P.i2dx) * __ldg(xZ + o - 1);
                    acc += (-my_i * P.idx2 - svx * P.i2dx) * __ldg(xZ + o + 1);
                    acc += (-mx_j * P.idy2 - svy * P.i2dy) * __ldg(xZ + o + sZj);
                    acc += (-mz_k * P.idz2) * __ldg(xZ + o + sZk);
                    acc += s * P.idz * (__ldg(xV + o + sZk) - __ldg(xV + o));
                    emit(row, acc, d, true);
                }
            }
            // ---------------------------------------------------------------- V
            {
                const int o = (i - 1) + (j - 1) * sZj + (k - 1) * sZk;
                const long long row = g.oV + o;
                if (qFixV(g, i, j, k)) {
                    emit(row, __ldg(xV + o), T(1), false);
                } else {
                    const T sx0 = CF(3, cur, 0, 0), sx1 = CF(3, cur, 0, -1);
                    const T sy0 = CF(4, cur, 0, 0), sy1 = CF(4, cur, -1, 0);
                    const T sz0 = CF(5, cur, 0, 0), sz1 = CF(5, prv, 0, 0);
                    const T fx0 = fmax(sx0, P.sigfloor), fx1 = fmax(sx1, P.sigfloor);
                    const T fy0 = fmax(sy0, P.sigfloor), fy1 = fmax(sy1, P.sigfloor);
                    const T fz0 = fmax(sz0, P.sigfloor), fz1 = fmax(sz1, P.sigfloor);
                    const T d = (fx0 + fx1) * P.idx2 + (fy0 + fy1) * P.idy2 + (fz0 + fz1) * P.idz2;
                    const int ox = (i - 1) + (j - 1) * sXj + (k - 1) * sXk;
                    const int oy = (i - 1) + (j - 1) * sYj + (k - 1) * sYk;
                    T acc = d * __ldg(xV + o);
                    acc -= fz1 * P.idz2 * __ldg(xV + o - sZk);
                    acc -= fy1 * P.idy2 * __ldg(xV + o - sZj);
                    acc -= fx1 * P.idx2 * __ldg(xV + o - 1);
                    acc -= fx0 * P.idx2 * __ldg(xV + o + 1);
                    acc -= fy0 * P.idy2 * __ldg(xV + o + sZj);
                    acc -= fz0 * P.idz2 * __ldg(xV + o + sZk);
                    const T axm = __ldg(xX + ox - 1), ax0 = __ldg(xX + ox);
                    const T aym = __ldg(xY + oy - sYj), ay0 = __ldg(xY + oy);
                    const T azm = __ldg(xZ + o - sZk), az0 = __ldg(xZ + o);
                    acc += P.idt * ((sx0 * ax0 - sx1 * axm) * P.idx + (sy0 * ay0 - sy1 * aym) * P.idy +
                                    (sz0 * az0 - sz1 * azm) * P.idz);
                    if (ADV) {
                        const T vx = P.vx, vy = P.vy, vz = P.vz;
                        acc += (sx1 * vz * P.i2dxdz - sz1 * vx * P.i2dz2) * __ldg(xX + ox - 1 - sXk);
                        acc += (-sx0 * vz * P.i2dxdz - sz1 * vx * P.i2dz2) * __ldg(xX + ox - sXk);
                        acc += (sx1 * vy * P.i2dxdy - sy1 * vx * P.i2dy2) * __ldg(xX + ox - 1 - sXj);
                        acc += (-sx0 * vy * P.i2dxdy - sy1 * vx * P.i2dy2) * __ldg(xX + ox - sXj);
                        acc += ((sy0 + sy1) * vx * P.i2dy2 + (sz0 + sz1) * vx * P.i2dz2) * (axm + ax0);
                        acc += (-sx1 * vy * P.i2dxdy - sy0 * vx * P.i2dy2) * __ldg(xX + ox - 1 + sXj);
                        acc += (sx0 * vy * P.i2dxdy - sy0 * vx * P.i2dy2) * __ldg(xX + ox + sXj);
                        acc += (-sx1 * vz * P.i2dxdz - sz0 * vx * P.i2dz2) * __ldg(xX + ox - 1 + sXk);
                        acc += (sx0 * vz * P.i2dxdz - sz0 * vx * P.i2dz2) * __ldg(xX + ox + sXk);

                        acc += (sy1 * vz * P.i2dydz - sz1 * vy * P.i2dz2) * __ldg(xY + oy - sYj - sYk);
                        acc += (-sy0 * vz * P.i2dydz - sz1 * vy * P.i2dz2) * __ldg(xY + oy - sYk);
                        acc += (-sx1 * vy * P.i2dx2 + sy1 * vx * P.i2dxdy) * __ldg(xY + oy - sYj - 1);
                        acc += ((sx0 + sx1) * vy * P.i2dx2 + (sz0 + sz1) * vy * P.i2dz2) * (aym + ay0);
                        acc += (-sx0 * vy * P.i2dx2 - sy1 * vx * P.i2dxdy) * __ldg(xY + oy - sYj + 1);
                        acc += (-sx1 * vy * P.i2dx2 - sy0 * vx * P.i2dxdy) * __ldg(xY + oy - 1);
                        acc += (-sx0 * vy * P.i2dx2 + sy0 * vx * P.i2dxdy) * __ldg(xY + oy + 1);
                        acc += (-sy1 * vz * P.i2dydz - sz0 * vy * P.i2dz2) * __ldg(xY + oy - sYj + sYk);
                        acc += (sy0 * vz * P.i2dydz - sz0 * vy * P.i2dz2) * __ldg(xY + oy + sYk);

                        acc += (-sy1 * vz * P.i2dy2 + sz1 * vy * P.i2dydz) * __ldg(xZ + o - sZj - sZk);
                        acc += (-sx1 * vz * P.i2dx2 + sz1 * vx * P.i2dxdz) * __ldg(xZ + o - 1 - sZk);
                        acc += ((sx0 + sx1) * vz * P.i2dx2 + (sy0 + sy1) * vz * P.i2dy2) * (azm + az0);
                        acc += (-sx0 * vz * P.i2dx2 - sz1 * vx * P.i2dxdz) * __ldg(xZ + o + 1 - sZk);
                        acc += (-sy0 * vz * P.i2dy2 - sz1 * vy * P.i2dydz) * __ldg(xZ + o + sZj - sZk);
                        acc += (-sy1 * vz * P.i2dy2 - sz0 * vy * P.i2dydz) * __ldg(xZ + o - sZj);
                        acc += (-sx1 * vz * P.i2dx2 - sz0 * vx * P.i2dxdz) * __ldg(xZ + o - 1);
                        acc += (-sx0 * vz * P.i2dx2 + sz0 * vx * P.i2dxdz) * __ldg(xZ + o + 1);
                        acc += (-sy0 * vz * P.i2dy2 + sz0 * vy * P.i2dydz) * __ldg(xZ + o + sZj);
                    }
                    emit(row, acc, d, false);
                }
            }
        }
#undef CF
        __syncthreads();
    }
    if (partials) {
        __shared__ double sh[32];
        const long long bid = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
        const long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
        double s0 = qBlockSum(red0, sh);
        if (qLinTid() == 0) partials[bid] = s0;
        double s1 = qBlockSum(red1, sh);
        if (qLinTid() == 0) partials[nb + bid] = s1;
        if (MODE == QOP_RESID) {
            double s2 = qBlockSum(red2, sh);
            if (qLinTid() == 0) partials[2 * nb + bid] = s2;
            double s3 = qBlockSum(red3, sh);
            if (qLinTid() == 0) partials[3 * nb + bid] = s3;
        }
    }
}

// Diagonal of the (steady or transient) operator, FP32, for the Jacobi
// preconditioner of the inner PCG.  Dirichlet rows get 1.
__global__ void qk_diag(QGrid g, QCoef<float> c, QStepPar<float> P, float* __restrict__ dg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > g.Nx || j > g.Ny || k > g.Nz) return;
    if (i <= g.xs) {
        float d = 1.f;
        if (!qFixX(g, i, j, k))
            d = (c.imuz(i, j, k) + c.imuz(i, j - 1, k)) * P.idy2 + (c.imuy(i, j, k) + c.imuy(i, j, k - 1)) * P.idz2 +
                (c.imux(i, j, k) + c.imux(i - 1, j, k)) * P.idx2 + c.sgx(i, j, k) * P.idt;
        dg[qAX(g, i, j, k)] = d;
    }
    if (j <= g.ys) {
        float d = 1.f;
        if (!qFixY(g, i, j, k))
            d = (c.imuz(i, j, k) + c.imuz(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j, k - 1)) * P.idz2 +
                (c.imuy(i, j, k) + c.imuy(i, j - 1, k)) * P.idy2 + c.sgy(i, j, k) * P.idt;
        dg[qAY(g, i, j, k)] = d;
    }
    if (k <= g.zs) {
        float d = 1.f;
        if (!qFixZ(g, i, j, k))
            d = (c.imuy(i, j, k) + c.imuy(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j - 1, k)) * P.idy2 +
                (c.imuz(i, j, k) + c.imuz(i, j, k - 1)) * P.idz2 + c.sgz(i, j, k) * P.idt;
        dg[qAZ(g, i, j, k)] = d;
    }
    {
        float d = 1.f;
        if (!qFixV(g, i, j, k)) {
            const float f = P.sigfloor;
            d = (fmaxf(c.sgx(i, j, k), f) + fmaxf(c.sgx(i - 1, j, k), f)) * P.idx2 +
                (fmaxf(c.sgy(i, j, k), f) + fmaxf(c.sgy(i, j - 1, k), f)) * P.idy2 +
                (fmaxf(c.sgz(i, j, k), f) + fmaxf(c.sgz(i, j, k - 1), f)) * P.idz2;
        }
        dg[qV(g, i, j, k)] = d;
    }
}

// CSR SpMV (1-based ia int64 / ja int32 as produced by the assembly kernel): y = A x.
__global__ void qk_csr_spmv(long long n, const long long* __restrict__ ia, const int32_t* __restrict__ ja,
                            const double* __restrict__ a, const double* __restrict__ x, double* __restrict__ y) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double acc = 0.0;
    for (long long e = ia[r] - 1; e < ia[r + 1] - 1; e++) acc += a[e] * x[ja[e] - 1];
    y[r] = acc;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static dim3 op_block() { return dim3(32, 4, 2); }
static dim3 op_grid(const QGrid& g) { return dim3((g.Nx + 31) / 32, (g.Ny + 3) / 4, (g.Nz + 1) / 2); }
static dim3 opt_block() { return dim3(OTX, OTY, 1); }
static dim3 opt_grid(const QGrid& g) { return dim3((g.Nx + OTX - 1) / OTX, (g.Ny + OTY - 1) / OTY, (g.Nz + OKB - 1) / OKB); }

// number of CTAs (= partial sums per reduction) of an operator launch
long long qms_op_num_blocks(const QGrid& g) {
    dim3 t = opt_grid(g);
    return (long long)t.x * t.y * t.z;
}

template <typename T>
void qms_launch_operator(const QGrid& g, const QCoef<T>& c, const QStepPar<T>& P, bool adv, int mode, const T* x,
                         const T* b, T* y, const T* w, double* partials, cudaStream_t st) {
    dim3 bs = opt_block(), gs = opt_grid(g);
#define L(ADV, MODE) qk_operator_t<T, ADV, MODE><<<gs, bs, 0, st>>>(g, c, P, x, b, y, w, partials)
    if (adv) {
        if (mode == QOP_APPLY) L(true, QOP_APPLY);
        else if (mode == QOP_SCALED) L(true, QOP_SCALED);
        else L(true, QOP_RESID);
    } else {
        if (mode == QOP_APPLY) L(false, QOP_APPLY);
        else if (mode == QOP_SCALED) L(false, QOP_SCALED);
        else L(false, QOP_RESID);
    }
#undef L
}

template void qms_launch_operator<float>(const QGrid&, const QCoef<float>&, const QStepPar<float>&, bool, int,
                                         const float*, const float*, float*, const float*, double*, cudaStream_t);
template void qms_launch_operator<double>(const QGrid&, const QCoef<double>&, const QStepPar<double>&, bool, int,
                                          const double*, const double*, double*, const double*, double*, cudaStream_t);

void qms_launch_diag(const QGrid& g, const QCoef<float>& c, const QStepPar<float>& P, float* dg, cudaStream_t st) {
    qk_diag<<<op_grid(g), op_block(), 0, st>>>(g, c, P, dg);
}

void qms_launch_csr_spmv(long long n, const long long* ia, const int32_t* ja, const double* a, const double* x,
                         double* y, cudaStream_t st) {
    qk_csr_spmv<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, ia, ja, a, x, y);
}
