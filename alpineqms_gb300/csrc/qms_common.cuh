// qms_common.cuh -- grid descriptor, unknown numbering and on-the-fly Yee
// coefficients shared by every kernel of libqms_gb300.
//
// Unknown vector layout (the reference's x_vec, 3D/QMS_3D.f90:172-176,
// F:455-457, F:628-631, F:802-805, F:976-979), i fastest:
//   [ Ax : xs*Ny*Nz | Ay : Nx*ys*Nz | Az : Nx*Ny*zs | V : Nx*Ny*Nz ]
// with N* = *s + 1 nodes.  All (i,j,k) below are 1-based like the reference.
//
// Materials live in HBM as one uint8 slot per cell (0 = vacuum, r = table
// row r) plus a per-slot table; face permeabilities (harmonic mean across the
// face normal, F:261-263) and edge conductivities (mean of the 4 cells around
// the edge, F:264-266) are formed on the fly from the slots.  As in the
// reference they are only formed for 2 <= i <= xs, 2 <= j <= ys, 2 <= k <= zs
// (F:258-260); elsewhere they keep the vacuum values mu0 / 0.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define QMS_MU0 1.25663706E-6
#define QMS_MAX_SLOTS 256

struct QGrid {
    int xs, ys, zs;
    int Nx, Ny, Nz;
    long long Nn;                 // Nx*Ny*Nz
    long long oY, oZ, oV, n;      // block offsets and n_dims
    long long nAx, nAy, nAz;      // block sizes
    double dx, dy, dz;
};

static inline QGrid qms_make_grid(int xs, int ys, int zs, double dx, double dy, double dz) {
    QGrid g;
    g.xs = xs; g.ys = ys; g.zs = zs;
    g.Nx = xs + 1; g.Ny = ys + 1; g.Nz = zs + 1;
    g.Nn = (long long)g.Nx * g.Ny * g.Nz;
    g.nAx = (long long)xs * g.Ny * g.Nz;
    g.nAy = (long long)g.Nx * ys * g.Nz;
    g.nAz = (long long)g.Nx * g.Ny * zs;
    g.oY = g.nAx;
    g.oZ = g.nAx + g.nAy;
    g.oV = g.nAx + g.nAy + g.nAz;
    g.n = g.oV + g.Nn;
    g.dx = dx; g.dy = dy; g.dz = dz;
    return g;
}

// 0-based positions in the unknown vector (1-based i, j, k)
__host__ __device__ __forceinline__ long long qAX(const QGrid& g, int i, int j, int k) {
    return (long long)(i - 1) + (long long)(j - 1) * g.xs + (long long)(k - 1) * g.xs * g.Ny;
}
__host__ __device__ __forceinline__ long long qAY(const QGrid& g, int i, int j, int k) {
    return g.oY + (long long)(i - 1) + (long long)(j - 1) * g.Nx + (long long)(k - 1) * g.Nx * g.ys;
}
__host__ __device__ __forceinline__ long long qAZ(const QGrid& g, int i, int j, int k) {
    return g.oZ + (long long)(i - 1) + (long long)(j - 1) * g.Nx + (long long)(k - 1) * g.Nx * g.Ny;
}
__host__ __device__ __forceinline__ long long qV(const QGrid& g, int i, int j, int k) {
    return g.oV + (long long)(i - 1) + (long long)(j - 1) * g.Nx + (long long)(k - 1) * g.Nx * g.Ny;
}
__host__ __device__ __forceinline__ long long qCELL(const QGrid& g, int i, int j, int k) {
    return (long long)(i - 1) + (long long)(j - 1) * g.xs + (long long)(k - 1) * g.xs * g.ys;
}

// Dirichlet predicates (F:361-396): two-layer shell
__host__ __device__ __forceinline__ bool qFixX(const QGrid& g, int i, int j, int k) {
    return j <= 2 || j >= g.Ny - 1 || k <= 2 || k >= g.Nz - 1 || i == 1 || i == g.xs;
}
__host__ __device__ __forceinline__ bool qFixY(const QGrid& g, int i, int j, int k) {
    return i <= 2 || i >= g.Nx - 1 || k <= 2 || k >= g.Nz - 1 || j == 1 || j == g.ys;
}
__host__ __device__ __forceinline__ bool qFixZ(const QGrid& g, int i, int j, int k) {
    return i <= 2 || i >= g.Nx - 1 || j <= 2 || j >= g.Ny - 1 || k == 1 || k == g.zs;
}
__host__ __device__ __forceinline__ bool qFixV(const QGrid& g, int i, int j, int k) {
    return i <= 2 || i >= g.Nx - 1 || j <= 2 || j >= g.Ny - 1 || k <= 2 || k >= g.Nz - 1;
}

// Per-slot material table.  mu[] = mu_r * mu0 (cell permeability, F:245-247),
// imu[] = 1 / (mu_r * mu0), sig[] = cell conductivity (F:248-250); index 3*slot + axis.
template <typename T>
struct QMatTable {
    T mu[3 * QMS_MAX_SLOTS];
    T imu[3 * QMS_MAX_SLOTS];
    T sig[3 * QMS_MAX_SLOTS];
};

// Face / edge coefficient evaluator used by the matrix-free kernels.
// Reciprocal face permeability: 1/Mu_face = 0.5*(1/mu_a + 1/mu_b), the exact
// reciprocal of the harmonic mean 2ab/(a+b) up to rounding.
template <typename T>
struct QCoef {
    QGrid g;
    const uint8_t* __restrict__ id;
    const QMatTable<T>* __restrict__ tab;
    T imu0;
    // optional: the six node coefficients (1/mu_x, 1/mu_y, 1/mu_z, sigma_x, sigma_y, sigma_z)
    // formed once per geometry, six arrays in the padded node layout of qms_tma.cuh
    const T* __restrict__ nc = nullptr;

    __device__ __forceinline__ int cell(int i, int j, int k) const { return __ldg(id + qCELL(g, i, j, k)); }
    __device__ __forceinline__ bool face(int i, int j, int k) const {
        return i >= 2 && i <= g.xs && j >= 2 && j <= g.ys && k >= 2 && k <= g.zs;
    }
    __device__ __forceinline__ T imux(int i, int j, int k) const {
        return face(i, j, k) ? T(0.5) * (tab->imu[3 * cell(i, j, k)] + tab->imu[3 * cell(i - 1, j, k)]) : imu0;
    }
    __device__ __forceinline__ T imuy(int i, int j, int k) const {
        return face(i, j, k) ? T(0.5) * (tab->imu[3 * cell(i, j, k) + 1] + tab->imu[3 * cell(i, j - 1, k) + 1]) : imu0;
    }
    __device__ __forceinline__ T imuz(int i, int j, int k) const {
        return face(i, j, k) ? T(0.5) * (tab->imu[3 * cell(i, j, k) + 2] + tab->imu[3 * cell(i, j, k - 1) + 2]) : imu0;
    }
    __device__ __forceinline__ T sgx(int i, int j, int k) const {
        if (!face(i, j, k)) return T(0);
        return (tab->sig[3 * cell(i, j, k)] + tab->sig[3 * cell(i, j, k - 1)] + tab->sig[3 * cell(i, j - 1, k)] +
                tab->sig[3 * cell(i, j - 1, k - 1)]) * T(0.25);
    }
    __device__ __forceinline__ T sgy(int i, int j, int k) const {
        if (!face(i, j, k)) return T(0);
        return (tab->sig[3 * cell(i, j, k) + 1] + tab->sig[3 * cell(i - 1, j, k) + 1] + tab->sig[3 * cell(i, j, k - 1) + 1] +
                tab->sig[3 * cell(i - 1, j, k - 1) + 1]) * T(0.25);
    }
    __device__ __forceinline__ T sgz(int i, int j, int k) const {
        if (!face(i, j, k)) return T(0);
        return (tab->sig[3 * cell(i, j, k) + 2] + tab->sig[3 * cell(i - 1, j, k) + 2] + tab->sig[3 * cell(i, j - 1, k) + 2] +
                tab->sig[3 * cell(i - 1, j - 1, k) + 2]) * T(0.25);
    }
};

// Step parameters of the operator: velocity, dt and the grid reciprocals.
template <typename T>
struct QStepPar {
    T vx, vy, vz;
    T idt;                 // 1/dt (0 for the steady form)
    T idx2, idy2, idz2;    // 1/h^2
    T idxdy, idxdz, idydz; // 1/(h_a h_b)
    T i2dx, i2dy, i2dz;    // 1/(2h)
    T idx, idy, idz;       // 1/h
    T i2dx2, i2dy2, i2dz2; // 1/(2h^2)
    T i2dxdy, i2dxdz, i2dydz;
    T sigfloor;            // (double)1.0e-12f, F:1237
};

template <typename T>
static inline QStepPar<T> qms_step_par(const QGrid& g, double vx, double vy, double vz, double dt, bool transient) {
    QStepPar<T> p;
    p.vx = (T)vx; p.vy = (T)vy; p.vz = (T)vz;
    p.idt = transient ? (T)(1.0 / dt) : (T)0;
    p.idx2 = (T)(1.0 / (g.dx * g.dx)); p.idy2 = (T)(1.0 / (g.dy * g.dy)); p.idz2 = (T)(1.0 / (g.dz * g.dz));
    p.idxdy = (T)(1.0 / (g.dx * g.dy)); p.idxdz = (T)(1.0 / (g.dx * g.dz)); p.idydz = (T)(1.0 / (g.dy * g.dz));
    p.i2dx = (T)(1.0 / (2.0 * g.dx)); p.i2dy = (T)(1.0 / (2.0 * g.dy)); p.i2dz = (T)(1.0 / (2.0 * g.dz));
    p.idx = (T)(1.0 / g.dx); p.idy = (T)(1.0 / g.dy); p.idz = (T)(1.0 / g.dz);
    p.i2dx2 = (T)(1.0 / (2.0 * g.dx * g.dx)); p.i2dy2 = (T)(1.0 / (2.0 * g.dy * g.dy)); p.i2dz2 = (T)(1.0 / (2.0 * g.dz * g.dz));
    p.i2dxdy = (T)(1.0 / (2.0 * g.dx * g.dy)); p.i2dxdz = (T)(1.0 / (2.0 * g.dx * g.dz)); p.i2dydz = (T)(1.0 / (2.0 * g.dy * g.dz));
    p.sigfloor = (T)(double)1.0e-12f;
    return p;
}

// ---------------------------------------------------------------------------
// block reductions (warp shuffles, then one warp over the warp partials)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T qWarpSum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ int qLinTid() {
    return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
}
__device__ __forceinline__ int qNumThreads() { return blockDim.x * blockDim.y * blockDim.z; }

// Sums `v` over the (1-, 2- or 3-D) block; the result is valid in linear
// thread 0.  Warp stage in T, cross-warp stage in double.  `sh` needs 32 doubles.
template <typename T>
__device__ __forceinline__ double qBlockSum(T v, double* sh) {
    const int tid = qLinTid();
    const int lane = tid & 31, wid = tid >> 5;
    const int nw = (qNumThreads() + 31) >> 5;
    v = qWarpSum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = (double)v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < nw ? sh[lane] : 0.0;
        r = qWarpSum(r);
    }
    return r;
}

// status bits written by kernels and read by the host
enum QStatusBits : unsigned {
    QMS_ST_BAD_MATERIAL = 1u,   // geometry ID outside the table
    QMS_ST_NAN = 2u,            // non-finite residual
    QMS_ST_NO_CONVERGENCE = 4u, // iteration limit reached
    QMS_ST_BREAKDOWN = 8u,      // Krylov breakdown (zero denominator)
    QMS_ST_TIMEOUT = 16u,       // a bounded wait for a tile copy gave up
};
