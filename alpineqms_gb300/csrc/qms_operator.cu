// qms_operator.cu -- matrix-free Yee A-V operator (the production replacement
// of the CSR matrix handed to PARDISO, 3D/QMS_3D.f90:1316, F:2196, F:2201).
//
// One thread per node (i,j) of a tile, marching in k, evaluates the (up to) four rows living there:
// the Ax row (i <= xs), Ay row (j <= ys), Az row (k <= zs) and the V row, with
// the same entries as the assembled CSR (F:476-607, F:650-781, F:824-955,
// F:1014-1285 and the transient additions F:1475-1504, F:1624-1681,
// F:1772-1857, F:1925-2126).  Face 1/mu and edge sigma come from the six stored
// node coefficients (or are formed on the fly from the uint8 material slots when
// none are stored), so the HBM traffic per node is the four inputs, the four
// outputs and the six coefficients.  The four unknown components of three
// k-planes (plus one in flight) sit in shared memory, staged by cp.async, so
// every neighbour read of the 17/37-point rows is a shared-memory read.
//
// Modes:
//   QOP_APPLY   y = M x                       (Dirichlet rows: y = x)
//   QOP_SCALED  y = D^-1 M x, D = diag(M)     (Dirichlet rows: y = x)
//   QOP_RESID   r = D^-1 (b - M x)            (FP64; Dirichlet rows: b - x)
// Optional fused reductions (block partials, FP64):
//   APPLY/SCALED: [0] += y . w, [1] += y . y    (w may be null -> skip)
//   RESID:        [0] += |r_A|^2, [1] += |r_V|^2, [2] += |x_A|^2, [3] += |x_V|^2
#include "qms_internal.h"
#include "qms_tile.cuh"
#include "qms_op_rows.cuh"
#include <algorithm>
#include <atomic>
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
// D^-1 of the scaled FP32 operator: a fast divide (the inner solver only needs the
// same operator on every application, which any deterministic rounding gives); FP64 exact
template <typename T>
__device__ __forceinline__ T op_div(T a, T d) {
    if constexpr (sizeof(T) == 4) return __fdividef(a, d);
    else return a / d;
}

// VM: the velocity components the advection term may use (qms_op_rows.cuh)
template <typename T, int VM, int MODE>
__global__ void __launch_bounds__(OTX * OTY, sizeof(T) == 4 ? QMS_STENCIL_MINB : 2)
qk_operator_t(QGrid g, QCoef<T> c, QStepPar<T> P, const T* __restrict__ x, const T* __restrict__ b,
              T* __restrict__ y, const T* __restrict__ w, double* __restrict__ partials) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileCoef<T>& tc = *reinterpret_cast<TileCoef<T>*>(smem_raw);
    XTile<T>& xt = *reinterpret_cast<XTile<T>*>(smem_raw + sizeof(TileCoef<T>));
    const int i0 = blockIdx.x * OTX + 1, j0 = blockIdx.y * OTY + 1, k0 = blockIdx.z * OKB + 1;
    const int li = threadIdx.x + 1, lj = threadIdx.y + 1;   // position in the coefficient tile
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    const bool inij = i <= g.Nx && j <= g.Ny;
    // 32-bit strides of the four unknown blocks (row indices of this thread's unknowns)
    // (i, j) parts of the Dirichlet predicates qFixX/Y/Z/V; their k parts are per plane
    const bool fxA = i <= 2 || i >= g.Nx - 1, fyA = j <= 2 || j >= g.Ny - 1;
    const bool fijX = fyA || i == 1 || i == g.xs, fijY = fxA || j == 1 || j == g.ys, fijZ = fxA || fyA;
    const int sXj = g.xs, sXk = g.xs * g.Ny;      // Ax: (xs, Ny, Nz)
    const int sYj = g.Nx, sYk = g.Nx * g.ys;      // Ay: (Nx, ys, Nz)
    const int sZj = g.Nx, sZk = g.Nx * g.Ny;      // Az: (Nx, Ny, zs); V: (Nx, Ny, Nz)
    using RT = typename std::conditional<MODE == QOP_RESID, double, float>::type;
    RT red0 = 0, red1 = 0, red2 = 0, red3 = 0;
    auto emit = [&](long long row, T acc, T diag, bool is_a, T xc_center) {
        T out;
        if (MODE == QOP_APPLY) out = acc;
        else if (MODE == QOP_SCALED) out = op_div(acc, diag);
        else out = (b[row] - acc) / diag;
        y[row] = out;
        if (partials) {
            if (MODE == QOP_RESID) {
                RT o = (RT)out, xv = (RT)xc_center;
                if (is_a) { red0 += o * o; red2 += xv * xv; }
                else { red1 += o * o; red3 += xv * xv; }
            } else {
                if (w) red0 += (RT)(out * w[row]);
                red1 += (RT)(out * out);
            }
        }
    };
    XStager xsg;
    CStager csg;
    xsg.init(g, i0, j0);
    csg.init(g, i0, j0);
    xsg.load(g, x, xt, k0 - 1);
    xsg.load(g, x, xt, k0);
    xsg.load(g, x, xt, k0 + 1);
    csg.load(c, tc, k0 - 1);
    csg.load(c, tc, k0);
    const int kend = min(k0 + OKB - 1, g.Nz);
    // rows of this thread's four unknowns at plane k0 (32-bit: n_dims < 2^31 is checked at creation)
    int rX = (i - 1) + (j - 1) * sXj + (k0 - 1) * sXk;
    int rY = (int)g.oY + (i - 1) + (j - 1) * sYj + (k0 - 1) * sYk;
    int rZ = (int)g.oZ + (i - 1) + (j - 1) * sZj + (k0 - 1) * sZk;
    int rV = (int)g.oV + (i - 1) + (j - 1) * sZj + (k0 - 1) * sZk;
    for (int k = k0; k <= kend; k++) {
        const bool kfA = k <= 2 || k >= g.Nz - 1;       // k terms of qFixX / qFixY / qFixV
        const bool kfZ = k == 1 || k == g.zs;           // k term of qFixZ
        cp_async_wait_all();
        __syncthreads();                       // planes k-1..k+1 of x and k-1..k of the coefficients ready
        if (k + 2 <= kend + 1) xsg.load(g, x, xt, k + 2);   // x plane k+2 into the slot of plane k-2
        if (k < kend) csg.load(c, tc, k + 1);                // coefficients of plane k+1 into that of k-2
        const int cur = tslot(k), prv = tslot(k - 1);
        const int xm = xslot(k - 1), x0 = xslot(k), xp = xslot(k + 1);
        if (inij) {
            auto xsf = [&](int comp, int dk, int dj, int di) -> T {
                return xt.v[dk < 0 ? xm : (dk > 0 ? xp : x0)][comp][lj + dj][li + di];
            };
            auto cff = [&](int q, int dk, int dj, int di) -> T { return tc.c[dk < 0 ? prv : cur][q][lj + dj][li + di]; };
            qms_op_node<T, VM>(g, P, i, j, k, fijX, fijY, fijZ, kfA, kfZ, rX, rY, rZ, rV, xsf, cff, emit);
        }
        rX += sXk; rY += sYk; rZ += sZk; rV += sZk;
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

// The six node coefficients, formed once per geometry from the material slots.
template <typename T>
__global__ void qk_node_coef(QGrid g, QCoef<T> c, T* __restrict__ nc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
    if (i > g.Nx) return;
    const QPL L = qms_pl(g);
    const long long t = qms_pl_node(g, L, i, j, k);
    nc[t] = c.imux(i, j, k);
    nc[L.comp + t] = c.imuy(i, j, k);
    nc[2 * L.comp + t] = c.imuz(i, j, k);
    nc[3 * L.comp + t] = c.sgx(i, j, k);
    nc[4 * L.comp + t] = c.sgy(i, j, k);
    nc[5 * L.comp + t] = c.sgz(i, j, k);
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

// The operator's tiles exceed the 48 KB default of dynamic shared memory in FP64: raise the
// limit of all six instances once per device (before any stream capture of a launch).
template <typename T>
static void qms_operator_prepare() {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    const int shm = (int)(sizeof(TileCoef<T>) + sizeof(XTile<T>));
    for (auto f : {qk_operator_t<T, 0, QOP_APPLY>, qk_operator_t<T, 0, QOP_SCALED>, qk_operator_t<T, 0, QOP_RESID>,
                   qk_operator_t<T, 7, QOP_APPLY>, qk_operator_t<T, 7, QOP_SCALED>, qk_operator_t<T, 7, QOP_RESID>,
                   qk_operator_t<T, 1, QOP_RESID>, qk_operator_t<T, 2, QOP_RESID>, qk_operator_t<T, 4, QOP_RESID>})
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
    done.fetch_or(bit, std::memory_order_acq_rel);
}

template <typename T>
void qms_launch_operator(const QGrid& g, const QCoef<T>& c, const QStepPar<T>& P, bool adv, int mode, const T* x,
                         const T* b, T* y, const T* w, double* partials, cudaStream_t st) {
    dim3 bs = opt_block(), gs = opt_grid(g);
    const size_t shm = sizeof(TileCoef<T>) + sizeof(XTile<T>);
    qms_operator_prepare<T>();
#define L(VM, MODE) qk_operator_t<T, VM, MODE><<<gs, bs, shm, st>>>(g, c, P, x, b, y, w, partials)
    // the residual (the FP64 anchor of every solve) also has one instantiation per velocity axis
    const int m = (P.vx != T(0) ? 1 : 0) | (P.vy != T(0) ? 2 : 0) | (P.vz != T(0) ? 4 : 0);
    if (adv) {
        if (mode == QOP_APPLY) L(7, QOP_APPLY);
        else if (mode == QOP_SCALED) L(7, QOP_SCALED);
        else if (m == 1) L(1, QOP_RESID);
        else if (m == 2) L(2, QOP_RESID);
        else if (m == 4) L(4, QOP_RESID);
        else L(7, QOP_RESID);
    } else {
        if (mode == QOP_APPLY) L(0, QOP_APPLY);
        else if (mode == QOP_SCALED) L(0, QOP_SCALED);
        else L(0, QOP_RESID);
    }
#undef L
}

template void qms_launch_operator<float>(const QGrid&, const QCoef<float>&, const QStepPar<float>&, bool, int,
                                         const float*, const float*, float*, const float*, double*, cudaStream_t);
template void qms_launch_operator<double>(const QGrid&, const QCoef<double>&, const QStepPar<double>&, bool, int,
                                          const double*, const double*, double*, const double*, double*, cudaStream_t);

template <typename T>
void qms_launch_node_coef(const QGrid& g, const QCoef<T>& c, T* nc, cudaStream_t st) {
    QCoef<T> c0 = c;
    c0.nc = nullptr;
    // padding between and around the nodes stays zero
    cudaMemsetAsync(nc, 0, 6 * qms_pl(g).comp * sizeof(T), st);
    qk_node_coef<T><<<dim3((g.Nx + 127) / 128, g.Ny, g.Nz), 128, 0, st>>>(g, c0, nc);
}
template void qms_launch_node_coef<float>(const QGrid&, const QCoef<float>&, float*, cudaStream_t);
template void qms_launch_node_coef<double>(const QGrid&, const QCoef<double>&, double*, cudaStream_t);

void qms_launch_diag(const QGrid& g, const QCoef<float>& c, const QStepPar<float>& P, float* dg, cudaStream_t st) {
    qk_diag<<<op_grid(g), op_block(), 0, st>>>(g, c, P, dg);
}

void qms_launch_csr_spmv(long long n, const long long* ia, const int32_t* ja, const double* a, const double* x,
                         double* y, cudaStream_t st) {
    qk_csr_spmv<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, ia, ja, a, x, y);
}
