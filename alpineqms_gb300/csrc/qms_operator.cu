// qms_operator.cu -- matrix-free Yee A-V operator (the production replacement
// of the CSR matrix handed to PARDISO, 3D/QMS_3D.f90:1316, F:2196, F:2201).
//
// One thread per node (i,j,k) evaluates the (up to) four rows living there:
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
#include <type_traits>

enum QOpMode { QOP_APPLY = 0, QOP_SCALED = 1, QOP_RESID = 2 };

template <typename T, bool ADV, int MODE>
__global__ void __launch_bounds__(256)
qk_operator(QGrid g, QCoef<T> c, QStepPar<T> P, const T* __restrict__ x, const T* __restrict__ b,
            T* __restrict__ y, const T* __restrict__ w, double* __restrict__ partials) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    const bool in = i <= g.Nx && j <= g.Ny && k <= g.Nz;
    // per-thread partial sums: FP64 for the FP64 residual, FP32 otherwise
    using RT = typename std::conditional<MODE == QOP_RESID, double, float>::type;
    RT red0 = 0, red1 = 0, red2 = 0, red3 = 0;
#define X(idx) __ldg(x + (idx))
    auto emit = [&](long long row, T acc, T diag, bool is_a) {
        T out;
        if (MODE == QOP_APPLY) out = acc;
        else if (MODE == QOP_SCALED) out = acc / diag;
        else out = (b[row] - acc) / diag;
        y[row] = out;
        if (partials) {
            if (MODE == QOP_RESID) {
                RT o = (RT)out, xv = (RT)X(row);
                if (is_a) { red0 += o * o; red2 += xv * xv; }
                else { red1 += o * o; red3 += xv * xv; }
            } else {
                if (w) red0 += (RT)(out * w[row]);
                red1 += (RT)(out * out);
            }
        }
    };
    if (in) {
        // ------------------------------------------------------------ Ax row
        if (i <= g.xs) {
            const long long row = qAX(g, i, j, k);
            if (qFixX(g, i, j, k)) {
                emit(row, X(row), T(1), true);
            } else {
                const T s = c.sgx(i, j, k);
                const T my_km = c.imuy(i, j, k - 1), my_k = c.imuy(i, j, k);
                const T mz_jm = c.imuz(i, j - 1, k), mz_j = c.imuz(i, j, k);
                const T mx_im = c.imux(i - 1, j, k), mx_i = c.imux(i, j, k);
                const T svy = ADV ? s * P.vy : T(0), svz = ADV ? s * P.vz : T(0);
                const T d = (mz_j + mz_jm) * P.idy2 + (my_k + my_km) * P.idz2 + (mx_i + mx_im) * P.idx2 + s * P.idt;
                T acc = d * X(row);
                acc += (-my_km * P.idz2 + svz * P.i2dz) * X(qAX(g, i, j, k - 1));
                acc += (-mz_jm * P.idy2 + svy * P.i2dy) * X(qAX(g, i, j - 1, k));
                acc += (-mx_im * P.idx2) * X(row - 1);
                acc += (-mx_i * P.idx2) * X(row + 1);
                acc += (-mz_j * P.idy2 - svy * P.i2dy) * X(qAX(g, i, j + 1, k));
                acc += (-my_k * P.idz2 - svz * P.i2dz) * X(qAX(g, i, j, k + 1));
                acc += (mz_jm * P.idxdy - svy * P.i2dx) * X(qAY(g, i, j - 1, k));
                acc += (-mz_jm * P.idxdy + svy * P.i2dx) * X(qAY(g, i + 1, j - 1, k));
                acc += (-mz_j * P.idxdy - svy * P.i2dx) * X(qAY(g, i, j, k));
                acc += (mz_j * P.idxdy + svy * P.i2dx) * X(qAY(g, i + 1, j, k));
                acc += (my_km * P.idxdz - svz * P.i2dx) * X(qAZ(g, i, j, k - 1));
                acc += (-my_km * P.idxdz + svz * P.i2dx) * X(qAZ(g, i + 1, j, k - 1));
                acc += (-my_k * P.idxdz - svz * P.i2dx) * X(qAZ(g, i, j, k));
                acc += (my_k * P.idxdz + svz * P.i2dx) * X(qAZ(g, i + 1, j, k));
                acc += s * P.idx * (X(qV(g, i + 1, j, k)) - X(qV(g, i, j, k)));
                emit(row, acc, d, true);
            }
        }
        // ------------------------------------------------------------ Ay row
        if (j <= g.ys) {
            const long long row = qAY(g, i, j, k);
            if (qFixY(g, i, j, k)) {
                emit(row, X(row), T(1), true);
            } else {
                const T s = c.sgy(i, j, k);
                const T mz_im = c.imuz(i - 1, j, k), mz_i = c.imuz(i, j, k);
                const T mx_km = c.imux(i, j, k - 1), mx_k = c.imux(i, j, k);
                const T my_jm = c.imuy(i, j - 1, k), my_j = c.imuy(i, j, k);
                const T svx = ADV ? s * P.vx : T(0), svz = ADV ? s * P.vz : T(0);
                const T d = (mz_i + mz_im) * P.idx2 + (mx_k + mx_km) * P.idz2 + (my_j + my_jm) * P.idy2 + s * P.idt;
                T acc = d * X(row);
                acc += (mz_im * P.idxdy - svx * P.i2dy) * X(qAX(g, i - 1, j, k));
                acc += (-mz_i * P.idxdy - svx * P.i2dy) * X(qAX(g, i, j, k));
                acc += (-mz_im * P.idxdy + svx * P.i2dy) * X(qAX(g, i - 1, j + 1, k));
                acc += (mz_i * P.idxdy + svx * P.i2dy) * X(qAX(g, i, j + 1, k));
                acc += (-mx_km * P.idz2 + svz * P.i2dz) * X(qAY(g, i, j, k - 1));
                acc += (-my_jm * P.idy2) * X(qAY(g, i, j - 1, k));
                acc += (-mz_im * P.idx2 + svx * P.i2dx) * X(row - 1);
                acc += (-mz_i * P.idx2 - svx * P.i2dx) * X(row + 1);
                acc += (-my_j * P.idy2) * X(qAY(g, i, j + 1, k));
                acc += (-mx_k * P.idz2 - svz * P.i2dz) * X(qAY(g, i, j, k + 1));
                acc += (mx_km * P.idydz - svz * P.i2dy) * X(qAZ(g, i, j, k - 1));
                acc += (-mx_km * P.idydz + svz * P.i2dy) * X(qAZ(g, i, j + 1, k - 1));
                acc += (-mx_k * P.idydz - svz * P.i2dy) * X(qAZ(g, i, j, k));
                acc += (mx_k * P.idydz + svz * P.i2dy) * X(qAZ(g, i, j + 1, k));
                acc += s * P.idy * (X(qV(g, i, j + 1, k)) - X(qV(g, i, j, k)));
                emit(row, acc, d, true);
            }
        }
        // ------------------------------------------------------------ Az row
        if (k <= g.zs) {
            const long long row = qAZ(g, i, j, k);
            if (qFixZ(g, i, j, k)) {
                emit(row, X(row), T(1), true);
            } else {
                const T s = c.sgz(i, j, k);
                const T my_im = c.imuy(i - 1, j, k), my_i = c.imuy(i, j, k);
                const T mx_jm = c.imux(i, j - 1, k), mx_j = c.imux(i, j, k);
                const T mz_km = c.imuz(i, j, k - 1), mz_k = c.imuz(i, j, k);
                const T svx = ADV ? s * P.vx : T(0), svy = ADV ? s * P.vy : T(0);
                const T d = (my_i + my_im) * P.idx2 + (mx_j + mx_jm) * P.idy2 + (mz_k + mz_km) * P.idz2 + s * P.idt;
                T acc = d * X(row);
                acc += (my_im * P.idxdz - svx * P.i2dz) * X(qAX(g, i - 1, j, k));
                acc += (-my_i * P.idxdz - svx * P.i2dz) * X(qAX(g, i, j, k));
                acc += (-my_im * P.idxdz + svx * P.i2dz) * X(qAX(g, i - 1, j, k + 1));
                acc += (my_i * P.idxdz + svx * P.i2dz) * X(qAX(g, i, j, k + 1));
                acc += (mx_jm * P.idydz - svy * P.i2dz) * X(qAY(g, i, j - 1, k));
                acc += (-mx_j * P.idydz - svy * P.i2dz) * X(qAY(g, i, j, k));
                acc += (-mx_jm * P.idydz + svy * P.i2dz) * X(qAY(g, i, j - 1, k + 1));
                acc += (mx_j * P.idydz + svy * P.i2dz) * X(qAY(g, i, j, k + 1));
                acc += (-mz_km * P.idz2) * X(qAZ(g, i, j, k - 1));
                acc += (-mx_jm * P.idy2 + svy * P.i2dy) * X(qAZ(g, i, j - 1, k));
                acc += (-my_im * P.idx2 + svx * P.i2dx) * X(row - 1);
                acc += (-my_i * P.idx2 - svx * P.i2dx) * X(row + 1);
                acc += (-mx_j * P.idy2 - svy * P.i2dy) * X(qAZ(g, i, j + 1, k));
                acc += (-mz_k * P.idz2) * X(qAZ(g, i, j, k + 1));
                acc += s * P.idz * (X(qV(g, i, j, k + 1)) - X(qV(g, i, j, k)));
                emit(row, acc, d, true);
            }
        }
        // ------------------------------------------------------------- V row
        {
            const long long row = qV(g, i, j, k);
            if (qFixV(g, i, j, k)) {
                emit(row, X(row), T(1), false);
            } else {
                const T sx0 = c.sgx(i, j, k), sx1 = c.sgx(i - 1, j, k);
                const T sy0 = c.sgy(i, j, k), sy1 = c.sgy(i, j - 1, k);
                const T sz0 = c.sgz(i, j, k), sz1 = c.sgz(i, j, k - 1);
                const T fx0 = fmax(sx0, P.sigfloor), fx1 = fmax(sx1, P.sigfloor);
                const T fy0 = fmax(sy0, P.sigfloor), fy1 = fmax(sy1, P.sigfloor);
                const T fz0 = fmax(sz0, P.sigfloor), fz1 = fmax(sz1, P.sigfloor);
                const T d = (fx0 + fx1) * P.idx2 + (fy0 + fy1) * P.idy2 + (fz0 + fz1) * P.idz2;
                T acc = d * X(row);
                acc -= fz1 * P.idz2 * X(qV(g, i, j, k - 1));
                acc -= fy1 * P.idy2 * X(qV(g, i, j - 1, k));
                acc -= fx1 * P.idx2 * X(row - 1);
                acc -= fx0 * P.idx2 * X(row + 1);
                acc -= fy0 * P.idy2 * X(qV(g, i, j + 1, k));
                acc -= fz0 * P.idz2 * X(qV(g, i, j, k + 1));
                // (1/dt) div(sigma A): F:1973-1985, F:2033-2054, F:2093-2126
                const T axm = X(qAX(g, i - 1, j, k)), ax0 = X(qAX(g, i, j, k));
                const T aym = X(qAY(g, i, j - 1, k)), ay0 = X(qAY(g, i, j, k));
                const T azm = X(qAZ(g, i, j, k - 1)), az0 = X(qAZ(g, i, j, k));
                acc += P.idt * ((sx0 * ax0 - sx1 * axm) * P.idx + (sy0 * ay0 - sy1 * aym) * P.idy +
                                (sz0 * az0 - sz1 * azm) * P.idz);
                if (ADV) {
                    // div(sigma v x curl A): F:1014-1230
                    const T vx = P.vx, vy = P.vy, vz = P.vz;
                    acc += (sx1 * vz * P.i2dxdz - sz1 * vx * P.i2dz2) * X(qAX(g, i - 1, j, k - 1));
                    acc += (-sx0 * vz * P.i2dxdz - sz1 * vx * P.i2dz2) * X(qAX(g, i, j, k - 1));
                    acc += (sx1 * vy * P.i2dxdy - sy1 * vx * P.i2dy2) * X(qAX(g, i - 1, j - 1, k));
                    acc += (-sx0 * vy * P.i2dxdy - sy1 * vx * P.i2dy2) * X(qAX(g, i, j - 1, k));
                    const T cx = (sy0 + sy1) * vx * P.i2dy2 + (sz0 + sz1) * vx * P.i2dz2;
                    acc += cx * (axm + ax0);
                    acc += (-sx1 * vy * P.i2dxdy - sy0 * vx * P.i2dy2) * X(qAX(g, i - 1, j + 1, k));
                    acc += (sx0 * vy * P.i2dxdy - sy0 * vx * P.i2dy2) * X(qAX(g, i, j + 1, k));
                    acc += (-sx1 * vz * P.i2dxdz - sz0 * vx * P.i2dz2) * X(qAX(g, i - 1, j, k + 1));
                    acc += (sx0 * vz * P.i2dxdz - sz0 * vx * P.i2dz2) * X(qAX(g, i, j, k + 1));

                    acc += (sy1 * vz * P.i2dydz - sz1 * vy * P.i2dz2) * X(qAY(g, i, j - 1, k - 1));
                    acc += (-sy0 * vz * P.i2dydz - sz1 * vy * P.i2dz2) * X(qAY(g, i, j, k - 1));
                    acc += (-sx1 * vy * P.i2dx2 + sy1 * vx * P.i2dxdy) * X(qAY(g, i - 1, j - 1, k));
                    const T cy = (sx0 + sx1) * vy * P.i2dx2 + (sz0 + sz1) * vy * P.i2dz2;
                    acc += cy * (aym + ay0);
                    acc += (-sx0 * vy * P.i2dx2 - sy1 * vx * P.i2dxdy) * X(qAY(g, i + 1, j - 1, k));
                    acc += (-sx1 * vy * P.i2dx2 - sy0 * vx * P.i2dxdy) * X(qAY(g, i - 1, j, k));
                    acc += (-sx0 * vy * P.i2dx2 + sy0 * vx * P.i2dxdy) * X(qAY(g, i + 1, j, k));
                    acc += (-sy1 * vz * P.i2dydz - sz0 * vy * P.i2dz2) * X(qAY(g, i, j - 1, k + 1));
                    acc += (sy0 * vz * P.i2dydz - sz0 * vy * P.i2dz2) * X(qAY(g, i, j, k + 1));

                    acc += (-sy1 * vz * P.i2dy2 + sz1 * vy * P.i2dydz) * X(qAZ(g, i, j - 1, k - 1));
                    acc += (-sx1 * vz * P.i2dx2 + sz1 * vx * P.i2dxdz) * X(qAZ(g, i - 1, j, k - 1));
                    const T cz = (sx0 + sx1) * vz * P.i2dx2 + (sy0 + sy1) * vz * P.i2dy2;
                    acc += cz * (azm + az0);
                    acc += (-sx0 * vz * P.i2dx2 - sz1 * vx * P.i2dxdz) * X(qAZ(g, i + 1, j, k - 1));
                    acc += (-sy0 * vz * P.i2dy2 - sz1 * vy * P.i2dydz) * X(qAZ(g, i, j + 1, k - 1));
                    acc += (-sy1 * vz * P.i2dy2 - sz0 * vy * P.i2dydz) * X(qAZ(g, i, j - 1, k));
                    acc += (-sx1 * vz * P.i2dx2 - sz0 * vx * P.i2dxdz) * X(qAZ(g, i - 1, j, k));
                    acc += (-sx0 * vz * P.i2dx2 + sz0 * vx * P.i2dxdz) * X(qAZ(g, i + 1, j, k));
                    acc += (-sy0 * vz * P.i2dy2 + sz0 * vy * P.i2dydz) * X(qAZ(g, i, j + 1, k));
                }
                emit(row, acc, d, false);
            }
        }
    }
#undef X
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

long long qms_op_num_blocks(const QGrid& g) {
    dim3 gs = op_grid(g);
    return (long long)gs.x * gs.y * gs.z;
}

template <typename T>
void qms_launch_operator(const QGrid& g, const QCoef<T>& c, const QStepPar<T>& P, bool adv, int mode, const T* x,
                         const T* b, T* y, const T* w, double* partials, cudaStream_t st) {
    dim3 bs = op_block(), gs = op_grid(g);
#define L(ADV, MODE) qk_operator<T, ADV, MODE><<<gs, bs, 0, st>>>(g, c, P, x, b, y, w, partials)
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
