// qms_op_rows.cuh -- the rows of the Yee A-V operator at one node (the same entries as the
// assembled CSR: F:476-607, F:650-781, F:824-955, F:1014-1285 and the transient additions
// F:1475-1504, F:1624-1681, F:1772-1857, F:1925-2126), shared by the stencil kernels.
//
// Each row is evaluated in difference form: every coupling pair acts on a difference of
// unknowns, so rounding scales with the variation of x rather than with x itself.
//   xs(q, dk, dj, di): unknown block q at (i + di, j + dj, k + dk), dk in {-1, 0, 1}
//   cf(q, dk, dj, di): node coefficient q (1/mu_x,y,z, sigma_x,y,z) at (i + di, j + dj, k + dk),
//                      dk in {-1, 0}
//   emit(row, acc, diag, is_a, x_row): the row's value M x, its diagonal and its own unknown
// fij*/kf*: the (i, j) and k parts of the Dirichlet predicates qFixX/Y/Z/V.
// VM: which velocity components may be nonzero (bit 0 x, 1 y, 2 z; 0 = no advection term);
// the terms of components outside VM are left out at compile time (they are exact zeros).
#pragma once
#include "qms_common.cuh"

template <typename T, int VM, typename XS, typename CF, typename EMIT>
__device__ __forceinline__ void qms_op_node(const QGrid& g, const QStepPar<T>& P, int i, int j, int k, bool fijX,
                                            bool fijY, bool fijZ, bool kfA, bool kfZ, long long rX, long long rY,
                                            long long rZ, long long rV, XS xs, CF cf, EMIT emit) {
        constexpr bool HX = (VM & 1) != 0, HY = (VM & 2) != 0, HZ = (VM & 4) != 0;
        // ---------------------------------------------------------------- Ax
        if (i <= g.xs) {
            const long long row = rX;
            if (fijX || kfA) {
                emit(row, xs(0, 0, 0, 0), T(1), true, xs(0, 0, 0, 0));
            } else {
                const T s = cf(3, 0, 0, 0);
                const T my_km = cf(1, -1, 0, 0), my_k = cf(1, 0, 0, 0);
                const T mz_jm = cf(2, 0, -1, 0), mz_j = cf(2, 0, 0, 0);
                const T mx_im = cf(0, 0, 0, -1), mx_i = cf(0, 0, 0, 0);
                const T svy = HY ? s * P.vy : T(0), svz = HZ ? s * P.vz : T(0);
                const T d = (mz_j + mz_jm) * P.idy2 + (my_k + my_km) * P.idz2 + (mx_i + mx_im) * P.idx2 + s * P.idt;
                // difference form: every coupling pair is applied to a difference of unknowns,
                // so the rounding error scales with the variation of x, not with x itself
                const T X0 = xs(0, 0, 0, 0);
                T acc = s * P.idt * X0;
                acc += my_km * P.idz2 * (X0 - xs(0, -1, 0, 0)) + my_k * P.idz2 * (X0 - xs(0, 1, 0, 0));
                acc += mz_jm * P.idy2 * (X0 - xs(0, 0, -1, 0)) + mz_j * P.idy2 * (X0 - xs(0, 0, 1, 0));
                acc += mx_im * P.idx2 * (X0 - xs(0, 0, 0, -1)) + mx_i * P.idx2 * (X0 - xs(0, 0, 0, 1));
                if constexpr (HZ) acc += svz * P.i2dz * (xs(0, -1, 0, 0) - xs(0, 1, 0, 0));
                if constexpr (HY) acc += svy * P.i2dy * (xs(0, 0, -1, 0) - xs(0, 0, 1, 0));
                acc += (HY ? mz_jm * P.idxdy - svy * P.i2dx : mz_jm * P.idxdy) * (xs(1, 0, -1, 0) - xs(1, 0, -1, 1));
                acc += (HY ? mz_j * P.idxdy + svy * P.i2dx : mz_j * P.idxdy) * (xs(1, 0, 0, 1) - xs(1, 0, 0, 0));
                acc += (HZ ? my_km * P.idxdz - svz * P.i2dx : my_km * P.idxdz) * (xs(2, -1, 0, 0) - xs(2, -1, 0, 1));
                acc += (HZ ? my_k * P.idxdz + svz * P.i2dx : my_k * P.idxdz) * (xs(2, 0, 0, 1) - xs(2, 0, 0, 0));
                acc += s * P.idx * (xs(3, 0, 0, 1) - xs(3, 0, 0, 0));
                emit(row, acc, d, true, xs(0, 0, 0, 0));
            }
        }
        // ---------------------------------------------------------------- Ay
        if (j <= g.ys) {
            const long long row = rY;
            if (fijY || kfA) {
                emit(row, xs(1, 0, 0, 0), T(1), true, xs(1, 0, 0, 0));
            } else {
                const T s = cf(4, 0, 0, 0);
                const T mz_im = cf(2, 0, 0, -1), mz_i = cf(2, 0, 0, 0);
                const T mx_km = cf(0, -1, 0, 0), mx_k = cf(0, 0, 0, 0);
                const T my_jm = cf(1, 0, -1, 0), my_j = cf(1, 0, 0, 0);
                const T svx = HX ? s * P.vx : T(0), svz = HZ ? s * P.vz : T(0);
                const T d = (mz_i + mz_im) * P.idx2 + (mx_k + mx_km) * P.idz2 + (my_j + my_jm) * P.idy2 + s * P.idt;
                const T Y0 = xs(1, 0, 0, 0);
                T acc = s * P.idt * Y0;
                acc += mx_km * P.idz2 * (Y0 - xs(1, -1, 0, 0)) + mx_k * P.idz2 * (Y0 - xs(1, 1, 0, 0));
                acc += my_jm * P.idy2 * (Y0 - xs(1, 0, -1, 0)) + my_j * P.idy2 * (Y0 - xs(1, 0, 1, 0));
                acc += mz_im * P.idx2 * (Y0 - xs(1, 0, 0, -1)) + mz_i * P.idx2 * (Y0 - xs(1, 0, 0, 1));
                if constexpr (HZ) acc += svz * P.i2dz * (xs(1, -1, 0, 0) - xs(1, 1, 0, 0));
                if constexpr (HX) acc += svx * P.i2dx * (xs(1, 0, 0, -1) - xs(1, 0, 0, 1));
                acc += (HX ? mz_im * P.idxdy - svx * P.i2dy : mz_im * P.idxdy) * (xs(0, 0, 0, -1) - xs(0, 0, 1, -1));
                acc += (HX ? mz_i * P.idxdy + svx * P.i2dy : mz_i * P.idxdy) * (xs(0, 0, 1, 0) - xs(0, 0, 0, 0));
                acc += (HZ ? mx_km * P.idydz - svz * P.i2dy : mx_km * P.idydz) * (xs(2, -1, 0, 0) - xs(2, -1, 1, 0));
                acc += (HZ ? mx_k * P.idydz + svz * P.i2dy : mx_k * P.idydz) * (xs(2, 0, 1, 0) - xs(2, 0, 0, 0));
                acc += s * P.idy * (xs(3, 0, 1, 0) - xs(3, 0, 0, 0));
                emit(row, acc, d, true, xs(1, 0, 0, 0));
            }
        }
        // ---------------------------------------------------------------- Az
        if (k <= g.zs) {
            const long long row = rZ;
            if (fijZ || kfZ) {
                emit(row, xs(2, 0, 0, 0), T(1), true, xs(2, 0, 0, 0));
            } else {
                const T s = cf(5, 0, 0, 0);
                const T my_im = cf(1, 0, 0, -1), my_i = cf(1, 0, 0, 0);
                const T mx_jm = cf(0, 0, -1, 0), mx_j = cf(0, 0, 0, 0);
                const T mz_km = cf(2, -1, 0, 0), mz_k = cf(2, 0, 0, 0);
                const T svx = HX ? s * P.vx : T(0), svy = HY ? s * P.vy : T(0);
                const T d = (my_i + my_im) * P.idx2 + (mx_j + mx_jm) * P.idy2 + (mz_k + mz_km) * P.idz2 + s * P.idt;
                const T Z0 = xs(2, 0, 0, 0);
                T acc = s * P.idt * Z0;
                acc += mz_km * P.idz2 * (Z0 - xs(2, -1, 0, 0)) + mz_k * P.idz2 * (Z0 - xs(2, 1, 0, 0));
                acc += mx_jm * P.idy2 * (Z0 - xs(2, 0, -1, 0)) + mx_j * P.idy2 * (Z0 - xs(2, 0, 1, 0));
                acc += my_im * P.idx2 * (Z0 - xs(2, 0, 0, -1)) + my_i * P.idx2 * (Z0 - xs(2, 0, 0, 1));
                if constexpr (HY) acc += svy * P.i2dy * (xs(2, 0, -1, 0) - xs(2, 0, 1, 0));
                if constexpr (HX) acc += svx * P.i2dx * (xs(2, 0, 0, -1) - xs(2, 0, 0, 1));
                acc += (HX ? my_im * P.idxdz - svx * P.i2dz : my_im * P.idxdz) * (xs(0, 0, 0, -1) - xs(0, 1, 0, -1));
                acc += (HX ? my_i * P.idxdz + svx * P.i2dz : my_i * P.idxdz) * (xs(0, 1, 0, 0) - xs(0, 0, 0, 0));
                acc += (HY ? mx_jm * P.idydz - svy * P.i2dz : mx_jm * P.idydz) * (xs(1, 0, -1, 0) - xs(1, 1, -1, 0));
                acc += (HY ? mx_j * P.idydz + svy * P.i2dz : mx_j * P.idydz) * (xs(1, 1, 0, 0) - xs(1, 0, 0, 0));
                acc += s * P.idz * (xs(3, 1, 0, 0) - xs(3, 0, 0, 0));
                emit(row, acc, d, true, xs(2, 0, 0, 0));
            }
        }
        // ---------------------------------------------------------------- V
        {
            const long long row = rV;
            if (fijZ || kfA) {
                emit(row, xs(3, 0, 0, 0), T(1), false, xs(3, 0, 0, 0));
            } else {
                const T sx0 = cf(3, 0, 0, 0), sx1 = cf(3, 0, 0, -1);
                const T sy0 = cf(4, 0, 0, 0), sy1 = cf(4, 0, -1, 0);
                const T sz0 = cf(5, 0, 0, 0), sz1 = cf(5, -1, 0, 0);
                const T fx0 = fmax(sx0, P.sigfloor), fx1 = fmax(sx1, P.sigfloor);
                const T fy0 = fmax(sy0, P.sigfloor), fy1 = fmax(sy1, P.sigfloor);
                const T fz0 = fmax(sz0, P.sigfloor), fz1 = fmax(sz1, P.sigfloor);
                const T d = (fx0 + fx1) * P.idx2 + (fy0 + fy1) * P.idy2 + (fz0 + fz1) * P.idz2;
                const T V0 = xs(3, 0, 0, 0);
                T acc = fz1 * P.idz2 * (V0 - xs(3, -1, 0, 0)) + fz0 * P.idz2 * (V0 - xs(3, 1, 0, 0));
                acc += fy1 * P.idy2 * (V0 - xs(3, 0, -1, 0)) + fy0 * P.idy2 * (V0 - xs(3, 0, 1, 0));
                acc += fx1 * P.idx2 * (V0 - xs(3, 0, 0, -1)) + fx0 * P.idx2 * (V0 - xs(3, 0, 0, 1));
                const T axm = xs(0, 0, 0, -1), ax0 = xs(0, 0, 0, 0);
                const T aym = xs(1, 0, -1, 0), ay0 = xs(1, 0, 0, 0);
                const T azm = xs(2, -1, 0, 0), az0 = xs(2, 0, 0, 0);
                // div(sigma A) / dt: s0 a0 - s1 a1 = s0 (a0 - a1) + (s0 - s1) a1 (exact inside a body)
                acc += P.idt * ((sx0 * (ax0 - axm) + (sx0 - sx1) * axm) * P.idx +
                                (sy0 * (ay0 - aym) + (sy0 - sy1) * aym) * P.idy +
                                (sz0 * (az0 - azm) + (sz0 - sz1) * azm) * P.idz);
                // div(sigma v x curl A), grouped by velocity component into differences
                const T vx = P.vx, vy = P.vy, vz = P.vz;
                // Ax neighbours
                const T SA = axm + ax0;
                if constexpr (HZ)
                    acc += vz * P.i2dxdz * (sx1 * (xs(0, -1, 0, -1) - xs(0, 1, 0, -1)) +
                                             sx0 * (xs(0, 1, 0, 0) - xs(0, -1, 0, 0)));
                if constexpr (HY)
                    acc += vy * P.i2dxdy * (sx1 * (xs(0, 0, -1, -1) - xs(0, 0, 1, -1)) +
                                             sx0 * (xs(0, 0, 1, 0) - xs(0, 0, -1, 0)));
                if constexpr (HX) {
                    acc += vx * P.i2dy2 * (sy1 * (SA - (xs(0, 0, -1, -1) + xs(0, 0, -1, 0))) +
                                           sy0 * (SA - (xs(0, 0, 1, -1) + xs(0, 0, 1, 0))));
                    acc += vx * P.i2dz2 * (sz1 * (SA - (xs(0, -1, 0, -1) + xs(0, -1, 0, 0))) +
                                           sz0 * (SA - (xs(0, 1, 0, -1) + xs(0, 1, 0, 0))));
                }
                // Ay neighbours
                const T SB = aym + ay0;
                if constexpr (HZ)
                    acc += vz * P.i2dydz * (sy1 * (xs(1, -1, -1, 0) - xs(1, 1, -1, 0)) +
                                             sy0 * (xs(1, 1, 0, 0) - xs(1, -1, 0, 0)));
                if constexpr (HX)
                    acc += vx * P.i2dxdy * (sy1 * (xs(1, 0, -1, -1) - xs(1, 0, -1, 1)) +
                                             sy0 * (xs(1, 0, 0, 1) - xs(1, 0, 0, -1)));
                if constexpr (HY) {
                    acc += vy * P.i2dx2 * (sx1 * (SB - (xs(1, 0, -1, -1) + xs(1, 0, 0, -1))) +
                                           sx0 * (SB - (xs(1, 0, -1, 1) + xs(1, 0, 0, 1))));
                    acc += vy * P.i2dz2 * (sz1 * (SB - (xs(1, -1, -1, 0) + xs(1, -1, 0, 0))) +
                                           sz0 * (SB - (xs(1, 1, -1, 0) + xs(1, 1, 0, 0))));
                }
                // Az neighbours
                const T SC = azm + az0;
                if constexpr (HY)
                    acc += vy * P.i2dydz * (sz1 * (xs(2, -1, -1, 0) - xs(2, -1, 1, 0)) +
                                             sz0 * (xs(2, 0, 1, 0) - xs(2, 0, -1, 0)));
                if constexpr (HX)
                    acc += vx * P.i2dxdz * (sz1 * (xs(2, -1, 0, -1) - xs(2, -1, 0, 1)) +
                                             sz0 * (xs(2, 0, 0, 1) - xs(2, 0, 0, -1)));
                if constexpr (HZ) {
                    acc += vz * P.i2dx2 * (sx1 * (SC - (xs(2, -1, 0, -1) + xs(2, 0, 0, -1))) +
                                           sx0 * (SC - (xs(2, -1, 0, 1) + xs(2, 0, 0, 1))));
                    acc += vz * P.i2dy2 * (sy1 * (SC - (xs(2, -1, -1, 0) + xs(2, 0, -1, 0))) +
                                           sy0 * (SC - (xs(2, -1, 1, 0) + xs(2, 0, 1, 0))));
                }
                emit(row, acc, d, false, xs(3, 0, 0, 0));
            }
        }
}
