// qms_exact.cu -- kernels whose results must match the reference bit for bit.
// Compiled with -fmad=false so no FMA contraction changes the rounding of the
// source-order expressions of 3D/QMS_3D.f90; divisions are IEEE (no fast-math).
//
//   qk_assemble_csr  K1  CSR pattern + values + RHS      F:448-1312, F:1457-2191
//   qk_build_rhs     K7  right-hand side (+ Dirichlet values into x)  F:460-469,
//                        F:1465-1476, F:1614-1625, F:1762-1773, F:1910-1929
//   qk_hfield        K8  H at cell centres               F:1346-1376, F:2237-2267
//   qk_slice         K8  2-D slice of the H cubes        F:1380-1394, F:2276-2290
//   qk_ids_from_geom K9  float64 IDs -> uint8 slots      F:234-254
#include "qms_internal.h"
#include "qms_pl.h"

namespace {

constexpr double THIRD = (double)(1.0f / 3.0f);   // "1/3.0" is a default-real quotient (F:465)
constexpr double FLOOR = (double)1.0e-12f;         // "1.0e-12" default real (F:1237)

// Exact face / edge coefficients, formed like F:261-266 from cell values.
struct ExactCoef {
    QGrid g;
    const uint8_t* id;
    const QMatTable<double>* tab;
    __device__ int cell(int i, int j, int k) const { return id[qCELL(g, i, j, k)]; }
    __device__ bool face(int i, int j, int k) const {
        return i >= 2 && i <= g.xs && j >= 2 && j <= g.ys && k >= 2 && k <= g.zs;
    }
    __device__ double mux(int i, int j, int k) const {
        if (!face(i, j, k)) return QMS_MU0;
        double a = tab->mu[3 * cell(i, j, k)], b = tab->mu[3 * cell(i - 1, j, k)];
        return 2.0 * a * b / (a + b);
    }
    __device__ double muy(int i, int j, int k) const {
        if (!face(i, j, k)) return QMS_MU0;
        double a = tab->mu[3 * cell(i, j, k) + 1], b = tab->mu[3 * cell(i, j - 1, k) + 1];
        return 2.0 * a * b / (a + b);
    }
    __device__ double muz(int i, int j, int k) const {
        if (!face(i, j, k)) return QMS_MU0;
        double a = tab->mu[3 * cell(i, j, k) + 2], b = tab->mu[3 * cell(i, j, k - 1) + 2];
        return 2.0 * a * b / (a + b);
    }
    __device__ double sgx(int i, int j, int k) const {
        if (!face(i, j, k)) return 0.0;
        return (tab->sig[3 * cell(i, j, k)] + tab->sig[3 * cell(i, j, k - 1)] + tab->sig[3 * cell(i, j - 1, k)] +
                tab->sig[3 * cell(i, j - 1, k - 1)]) / 4.0;
    }
    __device__ double sgy(int i, int j, int k) const {
        if (!face(i, j, k)) return 0.0;
        return (tab->sig[3 * cell(i, j, k) + 1] + tab->sig[3 * cell(i - 1, j, k) + 1] + tab->sig[3 * cell(i, j, k - 1) + 1] +
                tab->sig[3 * cell(i - 1, j, k - 1) + 1]) / 4.0;
    }
    __device__ double sgz(int i, int j, int k) const {
        if (!face(i, j, k)) return 0.0;
        return (tab->sig[3 * cell(i, j, k) + 2] + tab->sig[3 * cell(i - 1, j, k) + 2] + tab->sig[3 * cell(i, j - 1, k) + 2] +
                tab->sig[3 * cell(i - 1, j - 1, k) + 2]) / 4.0;
    }
};

struct Excite {           // background field of this solve (already scaled by s(t))
    double B[3];
    double G[9];          // gxx gxy gxz gyx gyy gyz gzx gzy gzz
    double v[3];          // solve_v{x,y,z}
};

// Dirichlet lift values, F:464-465, F:638-639, F:812-813, F:986-991
__device__ double lift_ax(const Excite& e, double xq, double yq, double zq) {
    return 0.5 * e.B[1] * (zq) - 0.5 * e.B[2] * (yq) +
           THIRD * ((e.G[3] * xq + e.G[4] * yq + e.G[5] * zq) * zq - (e.G[6] * xq + e.G[7] * yq + e.G[8] * zq) * yq);
}
__device__ double lift_ay(const Excite& e, double xq, double yq, double zq) {
    return 0.5 * e.B[2] * (xq) - 0.5 * e.B[0] * (zq) +
           THIRD * ((e.G[6] * xq + e.G[7] * yq + e.G[8] * zq) * xq - (e.G[0] * xq + e.G[1] * yq + e.G[2] * zq) * zq);
}
__device__ double lift_az(const Excite& e, double xq, double yq, double zq) {
    return 0.5 * e.B[0] * yq - 0.5 * e.B[1] * xq +
           THIRD * ((e.G[0] * xq + e.G[1] * yq + e.G[2] * zq) * yq - (e.G[3] * xq + e.G[4] * yq + e.G[5] * zq) * xq);
}
__device__ double lift_v(const Excite& e, double xq, double yq, double zq) {
    const double vx = e.v[0], vy = e.v[1], vz = e.v[2];
    const double gx = e.G[0] * xq + e.G[1] * yq + e.G[2] * zq;
    const double gy = e.G[3] * xq + e.G[4] * yq + e.G[5] * zq;
    const double gz = e.G[6] * xq + e.G[7] * yq + e.G[8] * zq;
    return -1.0 * (vy * e.B[2] - vz * e.B[1]) * xq
           - 1.0 * (vz * e.B[0] - vx * e.B[2]) * yq
           - 1.0 * (vx * e.B[1] - vy * e.B[0]) * zq
           - 0.5 * (vy * gz - vz * gy) * xq
           - 0.5 * (vz * gx - vx * gz) * yq
           - 0.5 * (vx * gy - vy * gx) * zq;
}

// One Dirichlet value (comp 0..2: A x, y, z; 3: V) at node (i, j, k), out of line: only boundary
// threads of the node kernel call it, and inlined, its FP64 arithmetic would be if-converted
// into every thread (FP64 issue is scarce on GB300)
__device__ __noinline__ double lift_comp(const Excite& e, int comp, int i, int j, int k, double dx, double dy,
                                         double dz) {
    const double xq = (i - 1) * dx, yq = (j - 1) * dy, zq = (k - 1) * dz;
    if (comp == 0) return lift_ax(e, xq, yq, zq);
    if (comp == 1) return lift_ay(e, xq, yq, zq);
    if (comp == 2) return lift_az(e, xq, yq, zq);
    return lift_v(e, xq, yq, zq);
}

// number of interior rows before (i,j,k) in a block whose interior is the box
// [ilo,ihi]x[jlo,jhi]x[klo,khi] (F-order traversal, i fastest)
__device__ long long interior_before(int i, int j, int k, int ilo, int ihi, int jlo, int jhi, int klo, int khi) {
    long long wi = max(0, ihi - ilo + 1), wj = max(0, jhi - jlo + 1);
    long long cnt = (long long)max(0, min(k - 1, khi) - klo + 1) * wi * wj;
    if (k >= klo && k <= khi) {
        cnt += (long long)max(0, min(j - 1, jhi) - jlo + 1) * wi;
        if (j >= jlo && j <= jhi) cnt += max(0, min(i - 1, ihi) - ilo + 1);
    }
    return cnt;
}

struct CsrLayout {
    long long baseAy, baseAz, baseV, nnz;
};

__host__ __device__ inline long long box_count(int ilo, int ihi, int jlo, int jhi, int klo, int khi) {
    long long a = ihi - ilo + 1, b = jhi - jlo + 1, c = khi - klo + 1;
    if (a <= 0 || b <= 0 || c <= 0) return 0;
    return a * b * c;
}

}  // namespace

static CsrLayout qms_csr_layout(const QGrid& g) {
    CsrLayout L;
    long long iAx = box_count(2, g.xs - 1, 3, g.Ny - 2, 3, g.Nz - 2);
    long long iAy = box_count(3, g.Nx - 2, 2, g.ys - 1, 3, g.Nz - 2);
    long long iAz = box_count(3, g.Nx - 2, 3, g.Ny - 2, 2, g.zs - 1);
    long long iV = box_count(3, g.Nx - 2, 3, g.Ny - 2, 3, g.Nz - 2);
    L.baseAy = g.nAx + 16 * iAx;
    L.baseAz = L.baseAy + g.nAy + 16 * iAy;
    L.baseV = L.baseAz + g.nAz + 16 * iAz;
    L.nnz = L.baseV + g.Nn + 36 * iV;
    return L;
}

#define PUT(col, val) do { ja[p] = (int32_t)((col) + 1); a[p] = (val); p++; } while (0)

__global__ void qk_assemble_csr(QGrid g, const uint8_t* __restrict__ ids, const QMatTable<double>* __restrict__ tab,
                                Excite e, double dt, int tr, const double* __restrict__ xp, CsrLayout L,
                                long long* __restrict__ ia, int32_t* __restrict__ ja, double* __restrict__ a,
                                double* __restrict__ b) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n) return;
    if (r == 0) ia[g.n] = L.nnz + 1;
    ExactCoef c{g, ids, tab};
    const double dx = g.dx, dy = g.dy, dz = g.dz, vx = e.v[0], vy = e.v[1], vz = e.v[2];
    long long p;
    if (r < g.oY) {                                                   // Ax rows, F:448-615 / F:1457-1599
        long long q = r;
        int i = (int)(q % g.xs) + 1, j = (int)((q / g.xs) % g.Ny) + 1, k = (int)(q / ((long long)g.xs * g.Ny)) + 1;
        p = q + 16 * interior_before(i, j, k, 2, g.xs - 1, 3, g.Ny - 2, 3, g.Nz - 2);
        ia[r] = p + 1;
        if (qFixX(g, i, j, k)) {
            b[r] = lift_ax(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
            PUT(r, 1.0);
            return;
        }
        const double s = c.sgx(i, j, k);
        b[r] = tr ? (s / dt) * xp[qAX(g, i, j, k)] : 0.0;
        PUT(qAX(g, i, j, k - 1), -1.0 / c.muy(i, j, k - 1) / (dz * dz) + (s * vz) / (2.0 * dz));
        PUT(qAX(g, i, j - 1, k), -1.0 / c.muz(i, j - 1, k) / (dy * dy) + (s * vy) / (2.0 * dy));
        PUT(qAX(g, i - 1, j, k), -1.0 / c.mux(i - 1, j, k) / (dx * dx));
        {
            double w = (1.0 / c.muz(i, j, k) + 1.0 / c.muz(i, j - 1, k)) / (dy * dy)
                     + (1.0 / c.muy(i, j, k) + 1.0 / c.muy(i, j, k - 1)) / (dz * dz)
                     + (1.0 / c.mux(i, j, k) + 1.0 / c.mux(i - 1, j, k)) / (dx * dx);
            if (tr) w = w + s / dt;
            PUT(qAX(g, i, j, k), w);
        }
        PUT(qAX(g, i + 1, j, k), -1.0 / c.mux(i, j, k) / (dx * dx));
        PUT(qAX(g, i, j + 1, k), -1.0 / c.muz(i, j, k) / (dy * dy) - (s * vy) / (2.0 * dy));
        PUT(qAX(g, i, j, k + 1), -1.0 / c.muy(i, j, k) / (dz * dz) - (s * vz) / (2.0 * dz));
        PUT(qAY(g, i, j - 1, k), 1.0 / c.muz(i, j - 1, k) / (dx * dy) - (s * vy) / (2.0 * dx));
        PUT(qAY(g, i + 1, j - 1, k), -1.0 / c.muz(i, j - 1, k) / (dx * dy) + (s * vy) / (2.0 * dx));
        PUT(qAY(g, i, j, k), -1.0 / c.muz(i, j, k) / (dx * dy) - (s * vy) / (2.0 * dx));
        PUT(qAY(g, i + 1, j, k), 1.0 / c.muz(i, j, k) / (dx * dy) + (s * vy) / (2.0 * dx));
        PUT(qAZ(g, i, j, k - 1), 1.0 / c.muy(i, j, k - 1) / (dx * dz) - (s * vz) / (2.0 * dx));
        PUT(qAZ(g, i + 1, j, k - 1), -1.0 / c.muy(i, j, k - 1) / (dx * dz) + (s * vz) / (2.0 * dx));
        PUT(qAZ(g, i, j, k), -1.0 / c.muy(i, j, k) / (dx * dz) - (s * vz) / (2.0 * dx));
        PUT(qAZ(g, i + 1, j, k), 1.0 / c.muy(i, j, k) / (dx * dz) + (s * vz) / (2.0 * dx));
        PUT(qV(g, i, j, k), -c.sgx(i, j, k) / dx);
        PUT(qV(g, i + 1, j, k), c.sgx(i, j, k) / dx);
    } else if (r < g.oZ) {                                            // Ay rows, F:620-789 / F:1605-1748
        long long q = r - g.oY;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.ys) + 1, k = (int)(q / ((long long)g.Nx * g.ys)) + 1;
        p = L.baseAy + q + 16 * interior_before(i, j, k, 3, g.Nx - 2, 2, g.ys - 1, 3, g.Nz - 2);
        ia[r] = p + 1;
        if (qFixY(g, i, j, k)) {
            b[r] = lift_ay(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
            PUT(r, 1.0);
            return;
        }
        const double s = c.sgy(i, j, k);
        b[r] = tr ? (s / dt) * xp[qAY(g, i, j, k)] : 0.0;
        PUT(qAX(g, i - 1, j, k), 1.0 / c.muz(i - 1, j, k) / (dx * dy) - (s * vx) / (2.0 * dy));
        PUT(qAX(g, i, j, k), -1.0 / c.muz(i, j, k) / (dx * dy) - (s * vx) / (2.0 * dy));
        PUT(qAX(g, i - 1, j + 1, k), -1.0 / c.muz(i - 1, j, k) / (dx * dy) + (s * vx) / (2.0 * dy));
        PUT(qAX(g, i, j + 1, k), 1.0 / c.muz(i, j, k) / (dx * dy) + (s * vx) / (2.0 * dy));
        PUT(qAY(g, i, j, k - 1), -1.0 / c.mux(i, j, k - 1) / (dz * dz) + (s * vz) / (2.0 * dz));
        PUT(qAY(g, i, j - 1, k), -1.0 / c.muy(i, j - 1, k) / (dy * dy));
        PUT(qAY(g, i - 1, j, k), -1.0 / c.muz(i - 1, j, k) / (dx * dx) + (s * vx) / (2.0 * dx));
        {
            double w = (1.0 / c.muz(i, j, k) + 1.0 / c.muz(i - 1, j, k)) / (dx * dx)
                     + (1.0 / c.mux(i, j, k) + 1.0 / c.mux(i, j, k - 1)) / (dz * dz)
                     + (1.0 / c.muy(i, j, k) + 1.0 / c.muy(i, j - 1, k)) / (dy * dy);
            if (tr) w = w + s / dt;
            PUT(qAY(g, i, j, k), w);
        }
        PUT(qAY(g, i + 1, j, k), -1.0 / c.muz(i, j, k) / (dx * dx) - (s * vx) / (2.0 * dx));
        PUT(qAY(g, i, j + 1, k), -1.0 / c.muy(i, j, k) / (dy * dy));
        PUT(qAY(g, i, j, k + 1), -1.0 / c.mux(i, j, k) / (dz * dz) - (s * vz) / (2.0 * dz));
        PUT(qAZ(g, i, j, k - 1), 1.0 / c.mux(i, j, k - 1) / (dy * dz) - (s * vz) / (2.0 * dy));
        PUT(qAZ(g, i, j + 1, k - 1), -1.0 / c.mux(i, j, k - 1) / (dy * dz) + (s * vz) / (2.0 * dy));
        PUT(qAZ(g, i, j, k), -1.0 / c.mux(i, j, k) / (dy * dz) - (s * vz) / (2.0 * dy));
        PUT(qAZ(g, i, j + 1, k), 1.0 / c.mux(i, j, k) / (dy * dz) + (s * vz) / (2.0 * dy));
        PUT(qV(g, i, j, k), -c.sgy(i, j, k) / dy);
        PUT(qV(g, i, j + 1, k), c.sgy(i, j, k) / dy);
    } else if (r < g.oV) {                                            // Az rows, F:794-963 / F:1753-1896
        long long q = r - g.oZ;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.Ny) + 1, k = (int)(q / ((long long)g.Nx * g.Ny)) + 1;
        p = L.baseAz + q + 16 * interior_before(i, j, k, 3, g.Nx - 2, 3, g.Ny - 2, 2, g.zs - 1);
        ia[r] = p + 1;
        if (qFixZ(g, i, j, k)) {
            b[r] = lift_az(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
            PUT(r, 1.0);
            return;
        }
        const double s = c.sgz(i, j, k);
        b[r] = tr ? (s / dt) * xp[qAZ(g, i, j, k)] : 0.0;
        PUT(qAX(g, i - 1, j, k), 1.0 / c.muy(i - 1, j, k) / (dx * dz) - (s * vx) / (2.0 * dz));
        PUT(qAX(g, i, j, k), -1.0 / c.muy(i, j, k) / (dx * dz) - (s * vx) / (2.0 * dz));
        PUT(qAX(g, i - 1, j, k + 1), -1.0 / c.muy(i - 1, j, k) / (dx * dz) + (s * vx) / (2.0 * dz));
        PUT(qAX(g, i, j, k + 1), 1.0 / c.muy(i, j, k) / (dx * dz) + (s * vx) / (2.0 * dz));
        PUT(qAY(g, i, j - 1, k), 1.0 / c.mux(i, j - 1, k) / (dy * dz) - (s * vy) / (2.0 * dz));
        PUT(qAY(g, i, j, k), -1.0 / c.mux(i, j, k) / (dy * dz) - (s * vy) / (2.0 * dz));
        PUT(qAY(g, i, j - 1, k + 1), -1.0 / c.mux(i, j - 1, k) / (dy * dz) + (s * vy) / (2.0 * dz));
        PUT(qAY(g, i, j, k + 1), 1.0 / c.mux(i, j, k) / (dy * dz) + (s * vy) / (2.0 * dz));
        PUT(qAZ(g, i, j, k - 1), -1.0 / c.muz(i, j, k - 1) / (dz * dz));
        PUT(qAZ(g, i, j - 1, k), -1.0 / c.mux(i, j - 1, k) / (dy * dy) + (s * vy) / (2.0 * dy));
        PUT(qAZ(g, i - 1, j, k), -1.0 / c.muy(i - 1, j, k) / (dx * dx) + (s * vx) / (2.0 * dx));
        {
            double w = (1.0 / c.muy(i, j, k) + 1.0 / c.muy(i - 1, j, k)) / (dx * dx)
                     + (1.0 / c.mux(i, j, k) + 1.0 / c.mux(i, j - 1, k)) / (dy * dy)
                     + (1.0 / c.muz(i, j, k) + 1.0 / c.muz(i, j, k - 1)) / (dz * dz);
            if (tr) w = w + s / dt;
            PUT(qAZ(g, i, j, k), w);
        }
        PUT(qAZ(g, i + 1, j, k), -1.0 / c.muy(i, j, k) / (dx * dx) - (s * vx) / (2.0 * dx));
        PUT(qAZ(g, i, j + 1, k), -1.0 / c.mux(i, j, k) / (dy * dy) - (s * vy) / (2.0 * dy));
        PUT(qAZ(g, i, j, k + 1), -1.0 / c.muz(i, j, k) / (dz * dz));
        PUT(qV(g, i, j, k), -c.sgz(i, j, k) / dz);
        PUT(qV(g, i, j, k + 1), c.sgz(i, j, k) / dz);
    } else {                                                          // V rows, F:968-1293 / F:1901-2191
        long long q = r - g.oV;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.Ny) + 1, k = (int)(q / ((long long)g.Nx * g.Ny)) + 1;
        p = L.baseV + q + 36 * interior_before(i, j, k, 3, g.Nx - 2, 3, g.Ny - 2, 3, g.Nz - 2);
        ia[r] = p + 1;
        if (qFixV(g, i, j, k)) {
            b[r] = lift_v(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
            PUT(r, 1.0);
            return;
        }
        const double sx0 = c.sgx(i, j, k), sx1 = c.sgx(i - 1, j, k);
        const double sy0 = c.sgy(i, j, k), sy1 = c.sgy(i, j - 1, k);
        const double sz0 = c.sgz(i, j, k), sz1 = c.sgz(i, j, k - 1);
        if (tr) {
            b[r] = (sx0 * xp[qAX(g, i, j, k)] - sx1 * xp[qAX(g, i - 1, j, k)]) / (dt * dx)
                 + (sy0 * xp[qAY(g, i, j, k)] - sy1 * xp[qAY(g, i, j - 1, k)]) / (dt * dy)
                 + (sz0 * xp[qAZ(g, i, j, k)] - sz1 * xp[qAZ(g, i, j, k - 1)]) / (dt * dz);
        } else {
            b[r] = 0.0;
        }
        const double dz2 = dz * dz, dy2 = dy * dy, dx2 = dx * dx;
        PUT(qAX(g, i - 1, j, k - 1), sx1 * vz / (2.0 * dz * dx) - sz1 * vx / (2.0 * dz2));
        PUT(qAX(g, i, j, k - 1), -sx0 * vz / (2.0 * dz * dx) - sz1 * vx / (2.0 * dz2));
        PUT(qAX(g, i - 1, j - 1, k), sx1 * vy / (2.0 * dy * dx) - sy1 * vx / (2.0 * dy2));
        PUT(qAX(g, i, j - 1, k), -sx0 * vy / (2.0 * dy * dx) - sy1 * vx / (2.0 * dy2));
        {
            double w = (sy0 + sy1) * vx / (2.0 * dy2) + (sz0 + sz1) * vx / (2.0 * dz2);
            if (tr) w = w - sx1 / (dx * dt);
            PUT(qAX(g, i - 1, j, k), w);
            w = (sy0 + sy1) * vx / (2.0 * dy2) + (sz0 + sz1) * vx / (2.0 * dz2);
            if (tr) w = w + sx0 / (dx * dt);
            PUT(qAX(g, i, j, k), w);
        }
        PUT(qAX(g, i - 1, j + 1, k), -sx1 * vy / (2.0 * dy * dx) - sy0 * vx / (2.0 * dy2));
        PUT(qAX(g, i, j + 1, k), sx0 * vy / (2.0 * dy * dx) - sy0 * vx / (2.0 * dy2));
        PUT(qAX(g, i - 1, j, k + 1), -sx1 * vz / (2.0 * dz * dx) - sz0 * vx / (2.0 * dz2));
        PUT(qAX(g, i, j, k + 1), sx0 * vz / (2.0 * dz * dx) - sz0 * vx / (2.0 * dz2));
        PUT(qAY(g, i, j - 1, k - 1), sy1 * vz / (2.0 * dz * dy) - sz1 * vy / (2.0 * dz2));
        PUT(qAY(g, i, j, k - 1), -sy0 * vz / (2.0 * dz * dy) - sz1 * vy / (2.0 * dz2));
        PUT(qAY(g, i - 1, j - 1, k), -sx1 * vy / (2.0 * dx2) + sy1 * vx / (2.0 * dx * dy));
        {
            double w = (sx0 + sx1) * vy / (2.0 * dx2) + (sz0 + sz1) * vy / (2.0 * dz2);
            if (tr) w = w - sy1 / (dy * dt);
            PUT(qAY(g, i, j - 1, k), w);
        }
        PUT(qAY(g, i + 1, j - 1, k), -sx0 * vy / (2.0 * dx2) - sy1 * vx / (2.0 * dx * dy));
        PUT(qAY(g, i - 1, j, k), -sx1 * vy / (2.0 * dx2) - sy0 * vx / (2.0 * dx * dy));
        {
            double w = (sx0 + sx1) * vy / (2.0 * dx2) + (sz0 + sz1) * vy / (2.0 * dz2);
            if (tr) w = w + sy0 / (dy * dt);
            PUT(qAY(g, i, j, k), w);
        }
        PUT(qAY(g, i + 1, j, k), -sx0 * vy / (2.0 * dx2) + sy0 * vx / (2.0 * dx * dy));
        PUT(qAY(g, i, j - 1, k + 1), -sy1 * vz / (2.0 * dz * dy) - sz0 * vy / (2.0 * dz2));
        PUT(qAY(g, i, j, k + 1), sy0 * vz / (2.0 * dz * dy) - sz0 * vy / (2.0 * dz2));
        PUT(qAZ(g, i, j - 1, k - 1), -sy1 * vz / (2.0 * dy2) + sz1 * vy / (2.0 * dy * dz));
        PUT(qAZ(g, i - 1, j, k - 1), -sx1 * vz / (2.0 * dx2) + sz1 * vx / (2.0 * dx * dz));
        {
            double w = (sx0 + sx1) * vz / (2.0 * dx2) + (sy0 + sy1) * vz / (2.0 * dy2);
            if (tr) w = w - sz1 / (dz * dt);
            PUT(qAZ(g, i, j, k - 1), w);
        }
        PUT(qAZ(g, i + 1, j, k - 1), -sx0 * vz / (2.0 * dx2) - sz1 * vx / (2.0 * dx * dz));
        PUT(qAZ(g, i, j + 1, k - 1), -sy0 * vz / (2.0 * dy2) - sz1 * vy / (2.0 * dy * dz));
        PUT(qAZ(g, i, j - 1, k), -sy1 * vz / (2.0 * dy2) - sz0 * vy / (2.0 * dy * dz));
        PUT(qAZ(g, i - 1, j, k), -sx1 * vz / (2.0 * dx2) - sz0 * vx / (2.0 * dx * dz));
        {
            double w = (sx0 + sx1) * vz / (2.0 * dx2) + (sy0 + sy1) * vz / (2.0 * dy2);
            if (tr) w = w + sz0 / (dz * dt);
            PUT(qAZ(g, i, j, k), w);
        }
        PUT(qAZ(g, i + 1, j, k), -sx0 * vz / (2.0 * dx2) + sz0 * vx / (2.0 * dx * dz));
        PUT(qAZ(g, i, j + 1, k), -sy0 * vz / (2.0 * dy2) + sz0 * vy / (2.0 * dy * dz));
        PUT(qV(g, i, j, k - 1), -fmax(c.sgz(i, j, k - 1), FLOOR) / dz2);
        PUT(qV(g, i, j - 1, k), -fmax(c.sgy(i, j - 1, k), FLOOR) / dy2);
        PUT(qV(g, i - 1, j, k), -fmax(c.sgx(i - 1, j, k), FLOOR) / dx2);
        PUT(qV(g, i, j, k), (fmax(c.sgx(i, j, k), FLOOR) + fmax(c.sgx(i - 1, j, k), FLOOR)) / dx2
                          + (fmax(c.sgy(i, j, k), FLOOR) + fmax(c.sgy(i, j - 1, k), FLOOR)) / dy2
                          + (fmax(c.sgz(i, j, k), FLOOR) + fmax(c.sgz(i, j, k - 1), FLOOR)) / dz2);
        PUT(qV(g, i + 1, j, k), -fmax(c.sgx(i, j, k), FLOOR) / dx2);
        PUT(qV(g, i, j + 1, k), -fmax(c.sgy(i, j, k), FLOOR) / dy2);
        PUT(qV(g, i, j, k + 1), -fmax(c.sgz(i, j, k), FLOOR) / dz2);
    }
}
#undef PUT

// K7: right-hand side of the steady (tr = 0) or transient (tr = 1) system.
// xp is the previous solution (read only when tr = 1).  When `x_dirichlet` is
// not null the Dirichlet rows of that vector are set to their fixed values, so
// an iterative solve started from it keeps them exact.  With `sg` (edge sigma of every A row)
// and `sdt` (the same divided by dt), both formed by qk_rhs_coef with the same expressions, the
// transient rows read them instead of forming them again (bit-identical values).
__global__ void qk_build_rhs(QGrid g, const uint8_t* __restrict__ ids, const QMatTable<double>* __restrict__ tab,
                             Excite e, double dt, int tr, const double* __restrict__ xp, double* __restrict__ b,
                             double* __restrict__ x_dirichlet, const double* __restrict__ sg,
                             const double* __restrict__ sdt) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n) return;
    ExactCoef c{g, ids, tab};
    const double dx = g.dx, dy = g.dy, dz = g.dz;
    double val;
    bool fixed;
    if (sg && r < g.oV) {
        // A rows from the stored sigma / dt
        long long q = r;
        int i, j, k;
        if (r < g.oY) {
            i = (int)(q % g.xs) + 1; j = (int)((q / g.xs) % g.Ny) + 1; k = (int)(q / ((long long)g.xs * g.Ny)) + 1;
            fixed = qFixX(g, i, j, k);
            if (fixed) val = lift_ax(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
        } else if (r < g.oZ) {
            q = r - g.oY;
            i = (int)(q % g.Nx) + 1; j = (int)((q / g.Nx) % g.ys) + 1; k = (int)(q / ((long long)g.Nx * g.ys)) + 1;
            fixed = qFixY(g, i, j, k);
            if (fixed) val = lift_ay(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
        } else {
            q = r - g.oZ;
            i = (int)(q % g.Nx) + 1; j = (int)((q / g.Nx) % g.Ny) + 1; k = (int)(q / ((long long)g.Nx * g.Ny)) + 1;
            fixed = qFixZ(g, i, j, k);
            if (fixed) val = lift_az(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
        }
        if (!fixed) val = tr ? sdt[r] * xp[r] : 0.0;
    } else if (sg) {
        // V rows: the divergence of sigma A_prev / dt from the stored edge sigma
        long long q = r - g.oV;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.Ny) + 1, k = (int)(q / ((long long)g.Nx * g.Ny)) + 1;
        fixed = qFixV(g, i, j, k);
        if (fixed) {
            val = lift_v(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
        } else if (tr) {
            const long long ax = qAX(g, i, j, k), axm = qAX(g, i - 1, j, k);
            const long long ay = qAY(g, i, j, k), aym = qAY(g, i, j - 1, k);
            const long long az = qAZ(g, i, j, k), azm = qAZ(g, i, j, k - 1);
            val = (sg[ax] * xp[ax] - sg[axm] * xp[axm]) / (dt * dx)
                + (sg[ay] * xp[ay] - sg[aym] * xp[aym]) / (dt * dy)
                + (sg[az] * xp[az] - sg[azm] * xp[azm]) / (dt * dz);
        } else {
            val = 0.0;
        }
    } else if (r < g.oY) {
        long long q = r;
        int i = (int)(q % g.xs) + 1, j = (int)((q / g.xs) % g.Ny) + 1, k = (int)(q / ((long long)g.xs * g.Ny)) + 1;
        fixed = qFixX(g, i, j, k);
        val = fixed ? lift_ax(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz)
                    : (tr ? (c.sgx(i, j, k) / dt) * xp[r] : 0.0);
    } else if (r < g.oZ) {
        long long q = r - g.oY;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.ys) + 1, k = (int)(q / ((long long)g.Nx * g.ys)) + 1;
        fixed = qFixY(g, i, j, k);
        val = fixed ? lift_ay(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz)
                    : (tr ? (c.sgy(i, j, k) / dt) * xp[r] : 0.0);
    } else if (r < g.oV) {
        long long q = r - g.oZ;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.Ny) + 1, k = (int)(q / ((long long)g.Nx * g.Ny)) + 1;
        fixed = qFixZ(g, i, j, k);
        val = fixed ? lift_az(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz)
                    : (tr ? (c.sgz(i, j, k) / dt) * xp[r] : 0.0);
    } else {
        long long q = r - g.oV;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.Ny) + 1, k = (int)(q / ((long long)g.Nx * g.Ny)) + 1;
        fixed = qFixV(g, i, j, k);
        if (fixed) {
            val = lift_v(e, (i - 1) * dx, (j - 1) * dy, (k - 1) * dz);
        } else if (tr) {
            val = (c.sgx(i, j, k) * xp[qAX(g, i, j, k)] - c.sgx(i - 1, j, k) * xp[qAX(g, i - 1, j, k)]) / (dt * dx)
                + (c.sgy(i, j, k) * xp[qAY(g, i, j, k)] - c.sgy(i, j - 1, k) * xp[qAY(g, i, j - 1, k)]) / (dt * dy)
                + (c.sgz(i, j, k) * xp[qAZ(g, i, j, k)] - c.sgz(i, j, k - 1) * xp[qAZ(g, i, j, k - 1)]) / (dt * dz);
        } else {
            val = 0.0;
        }
    }
    b[r] = val;
    if (x_dirichlet && fixed) x_dirichlet[r] = val;
}

// a / c for a constant c with yc = RN(1/c): the quotient rounded once more through the exact
// remainder (Markstein's FMA correction, IBM J. Res. Dev. 34(1), 1990): q = RN(a yc),
// r = a - q c (exact with an FMA), result RN(q + r yc), which is the correctly rounded a / c
// (checked bit for bit against the oracle's division in the tests)
struct QDivC {
    double c, yc;          // the divisor and RN(1 / c), both formed on the host
};
__device__ __forceinline__ double qms_div_const(double a, QDivC d) {
    const double q = a * d.yc;
    const double r = fma(-q, d.c, a);
    return fma(r, d.yc, q);
}

// The same right-hand side with the stored edge sigma, one thread per node (its up to four rows):
// the same expressions as qk_build_rhs's stored-sigma path, without per-row index divisions.
// dv*: dt dx, dt dy, dt dz and their correctly rounded reciprocals.  xp and x_dirichlet may be
// the same vector: the Dirichlet rows written here are never read through xp (a V row that is
// not a Dirichlet row reads the A rows of its own and the lower neighbour nodes, none of which
// is a Dirichlet row).
__global__ void qk_build_rhs_nodes(QGrid g, Excite e, double dt, int tr, const double* __restrict__ xp,
                                   double* __restrict__ b, double* __restrict__ x_dirichlet,
                                   const double* __restrict__ sg, const double* __restrict__ sdt, QDivC dvx,
                                   QDivC dvy, QDivC dvz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    // FP64 issue bounds this kernel (GB300's FP64 rate is a small fraction of its FP32 one): the
    // the Dirichlet values (boundary rows) out of line, dt h from the host
    auto row = [&](long long r, int comp, bool fixed) {
        double val;
        if (fixed) {
            val = lift_comp(e, comp, i, j, k, g.dx, g.dy, g.dz);
            if (x_dirichlet) x_dirichlet[r] = val;
        } else {
            val = tr ? sdt[r] * xp[r] : 0.0;
        }
        b[r] = val;
    };
    if (i <= g.xs) row(qAX(g, i, j, k), 0, qFixX(g, i, j, k));
    if (j <= g.ys) row(qAY(g, i, j, k), 1, qFixY(g, i, j, k));
    if (k <= g.zs) row(qAZ(g, i, j, k), 2, qFixZ(g, i, j, k));
    {
        const long long r = qV(g, i, j, k);
        const bool fixed = qFixV(g, i, j, k);
        double val;
        if (fixed) {
            val = lift_comp(e, 3, i, j, k, g.dx, g.dy, g.dz);
        } else if (tr) {
            const long long ax = qAX(g, i, j, k), axm = qAX(g, i - 1, j, k);
            const long long ay = qAY(g, i, j, k), aym = qAY(g, i, j - 1, k);
            const long long az = qAZ(g, i, j, k), azm = qAZ(g, i, j, k - 1);
            val = qms_div_const(sg[ax] * xp[ax] - sg[axm] * xp[axm], dvx)
                + qms_div_const(sg[ay] * xp[ay] - sg[aym] * xp[aym], dvy)
                + qms_div_const(sg[az] * xp[az] - sg[azm] * xp[azm], dvz);
        } else {
            val = 0.0;
        }
        b[r] = val;
        if (x_dirichlet && fixed) x_dirichlet[r] = val;
    }
}

// Edge sigma of every A row (the expression of F:1465-1476 etc., as ExactCoef forms it) and the
// same divided by dt: the per-geometry part of the transient right-hand side.
__global__ void qk_rhs_coef(QGrid g, const uint8_t* __restrict__ ids, const QMatTable<double>* __restrict__ tab,
                            double dt, double* __restrict__ sg, double* __restrict__ sdt) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.oV) return;
    ExactCoef c{g, ids, tab};
    double s;
    if (r < g.oY) {
        long long q = r;
        int i = (int)(q % g.xs) + 1, j = (int)((q / g.xs) % g.Ny) + 1, k = (int)(q / ((long long)g.xs * g.Ny)) + 1;
        s = c.sgx(i, j, k);
    } else if (r < g.oZ) {
        long long q = r - g.oY;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.ys) + 1, k = (int)(q / ((long long)g.Nx * g.ys)) + 1;
        s = c.sgy(i, j, k);
    } else {
        long long q = r - g.oZ;
        int i = (int)(q % g.Nx) + 1, j = (int)((q / g.Nx) % g.Ny) + 1, k = (int)(q / ((long long)g.Nx * g.Ny)) + 1;
        s = c.sgz(i, j, k);
    }
    sg[r] = s;
    sdt[r] = s / dt;
}

// K8: H at cell centres from the A blocks of x (F:1346-1376); cubes are xs*ys*zs, F-order.
// H at cell (i, j, k) from the A blocks of x (F:1346-1376)
__device__ __forceinline__ void qms_hcell(const QGrid& g, const ExactCoef& c, const double* __restrict__ x, int i, int j,
                                          int k, double& hx, double& hy, double& hz) {
    const double dx = g.dx, dy = g.dy, dz = g.dz;
#define XAX(a, b_, d) x[qAX(g, a, b_, d)]
#define XAY(a, b_, d) x[qAY(g, a, b_, d)]
#define XAZ(a, b_, d) x[qAZ(g, a, b_, d)]
    hx = 0.5 * (((XAZ(i, j + 1, k) - XAZ(i, j, k)) / dy - (XAY(i, j, k + 1) - XAY(i, j, k)) / dz) / c.mux(i, j, k) +
                ((XAZ(i + 1, j + 1, k) - XAZ(i + 1, j, k)) / dy - (XAY(i + 1, j, k + 1) - XAY(i + 1, j, k)) / dz) / c.mux(i + 1, j, k));
    hy = 0.5 * (((XAX(i, j, k + 1) - XAX(i, j, k)) / dz - (XAZ(i + 1, j, k) - XAZ(i, j, k)) / dx) / c.muy(i, j, k) +
                ((XAX(i, j + 1, k + 1) - XAX(i, j + 1, k)) / dz - (XAZ(i + 1, j + 1, k) - XAZ(i, j + 1, k)) / dx) / c.muy(i, j + 1, k));
    hz = 0.5 * (((XAY(i + 1, j, k) - XAY(i, j, k)) / dx - (XAX(i, j + 1, k) - XAX(i, j, k)) / dy) / c.muz(i, j, k) +
                ((XAY(i + 1, j, k + 1) - XAY(i, j, k + 1)) / dx - (XAX(i, j + 1, k + 1) - XAX(i, j, k + 1)) / dy) / c.muz(i, j, k + 1));
#undef XAX
#undef XAY
#undef XAZ
}

__global__ void qk_hfield(QGrid g, const uint8_t* __restrict__ ids, const QMatTable<double>* __restrict__ tab,
                          const double* __restrict__ x, double* __restrict__ Hx, double* __restrict__ Hy,
                          double* __restrict__ Hz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > g.xs || j > g.ys || k > g.zs) return;
    ExactCoef c{g, ids, tab};
    const long long cq = qCELL(g, i, j, k);
    qms_hcell(g, c, x, i, j, k, Hx[cq], Hy[cq], Hz[cq]);
}

// H on the cells of one slice only (the same values as qk_hfield + qk_slice), in qk_slice's layout
__global__ void qk_hslice(QGrid g, const uint8_t* __restrict__ ids, const QMatTable<double>* __restrict__ tab,
                          const double* __restrict__ x, int axis, int index, double* __restrict__ out) {
    int n1 = axis == 0 ? g.ys : g.xs;
    int n2 = axis == 2 ? g.ys : g.zs;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n1 * n2) return;
    int a = (int)(t % n1) + 1, b = (int)(t / n1) + 1;
    int i, j, k;
    if (axis == 0) { i = index; j = a; k = b; }
    else if (axis == 1) { i = a; j = index; k = b; }
    else { i = a; j = b; k = index; }
    ExactCoef c{g, ids, tab};
    const long long m = (long long)n1 * n2;
    qms_hcell(g, c, x, i, j, k, out[t], out[m + t], out[2 * m + t]);
}
__global__ void qk_slice(QGrid g, int axis, int index, const double* __restrict__ Hx, const double* __restrict__ Hy,
                         const double* __restrict__ Hz, double* __restrict__ out) {
    int n1 = axis == 0 ? g.ys : g.xs;
    int n2 = axis == 2 ? g.ys : g.zs;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n1 * n2) return;
    int a = (int)(t % n1) + 1, b = (int)(t / n1) + 1;
    int i, j, k;
    if (axis == 0) { i = index; j = a; k = b; }
    else if (axis == 1) { i = a; j = index; k = b; }
    else { i = a; j = b; k = index; }
    long long cq = qCELL(g, i, j, k);
    long long m = (long long)n1 * n2;
    out[t] = Hx[cq];
    out[m + t] = Hy[cq];
    out[2 * m + t] = Hz[cq];
}

// K9: float64 geometry IDs -> uint8 slots through a LUT (F:234-254).  IDs above
// the table maximum or negative set QMS_ST_BAD_MATERIAL and map to vacuum.
__global__ void qk_ids_from_geom(long long ncell, const double* __restrict__ geom, const uint8_t* __restrict__ lut,
                                 int maxid, uint8_t* __restrict__ ids, unsigned* __restrict__ status) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) return;
    double gv = geom[t];
    // int() truncation toward zero, F:243
    long long id = (gv >= -2147483648.0 && gv < 2147483648.0) ? (long long)gv : -1;
    if (id < 0 || id > maxid) {
        ids[t] = 0;
        atomicOr(status, (unsigned)QMS_ST_BAD_MATERIAL);
        return;
    }
    ids[t] = lut[id];
}

// ---------------------------------------------------------------------------
// host launchers (called from qms_capi.cu)
// ---------------------------------------------------------------------------
static Excite to_excite(const QmsExcite& q) {
    Excite e;
    for (int d = 0; d < 3; d++) { e.B[d] = q.B[d]; e.v[d] = q.v[d]; }
    for (int d = 0; d < 9; d++) e.G[d] = q.G[d];
    return e;
}

long long qms_launch_assemble(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const QmsExcite& ex,
                              double dt, int tr, const double* xp, long long* ia, int32_t* ja, double* a, double* b,
                              cudaStream_t st) {
    CsrLayout L = qms_csr_layout(g);
    int bs = 128;
    long long nb = (g.n + bs - 1) / bs;
    qk_assemble_csr<<<(unsigned)nb, bs, 0, st>>>(g, ids, tab, to_excite(ex), dt, tr, xp, L, ia, ja, a, b);
    return L.nnz;
}

void qms_launch_rhs(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const QmsExcite& ex, double dt,
                    int tr, const double* xp, double* b, double* x_dirichlet, cudaStream_t st, const double* sg,
                    const double* sdt) {
    if (sg) {
        qk_build_rhs_nodes<<<qms_node_grid(g), qms_node_block(), 0, st>>>(
            g, to_excite(ex), dt, tr, xp, b, x_dirichlet, sg, sdt, QDivC{dt * g.dx, 1.0 / (dt * g.dx)},
            QDivC{dt * g.dy, 1.0 / (dt * g.dy)}, QDivC{dt * g.dz, 1.0 / (dt * g.dz)});
        return;
    }
    int bs = 256;
    long long nb = (g.n + bs - 1) / bs;
    qk_build_rhs<<<(unsigned)nb, bs, 0, st>>>(g, ids, tab, to_excite(ex), dt, tr, xp, b, x_dirichlet, sg, sdt);
}

void qms_launch_rhs_coef(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, double dt, double* sg,
                         double* sdt, cudaStream_t st) {
    int bs = 256;
    long long nb = (g.oV + bs - 1) / bs;
    qk_rhs_coef<<<(unsigned)nb, bs, 0, st>>>(g, ids, tab, dt, sg, sdt);
}

void qms_launch_hfield(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const double* x, double* Hx,
                       double* Hy, double* Hz, cudaStream_t st) {
    dim3 bs(32, 4, 2);
    dim3 gs((g.xs + 31) / 32, (g.ys + 3) / 4, (g.zs + 1) / 2);
    qk_hfield<<<gs, bs, 0, st>>>(g, ids, tab, x, Hx, Hy, Hz);
}

void qms_launch_hslice(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const double* x, int axis,
                       int index, double* out, cudaStream_t st) {
    long long m = (long long)(axis == 0 ? g.ys : g.xs) * (axis == 2 ? g.ys : g.zs);
    qk_hslice<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(g, ids, tab, x, axis, index, out);
}

void qms_launch_slice(const QGrid& g, int axis, int index, const double* Hx, const double* Hy, const double* Hz,
                      double* out, cudaStream_t st) {
    long long m = (long long)(axis == 0 ? g.ys : g.xs) * (axis == 2 ? g.ys : g.zs);
    qk_slice<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(g, axis, index, Hx, Hy, Hz, out);
}

void qms_launch_ids(long long ncell, const double* geom, const uint8_t* lut, int maxid, uint8_t* ids, unsigned* status,
                    cudaStream_t st) {
    qk_ids_from_geom<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(ncell, geom, lut, maxid, ids, status);
}

long long qms_csr_nnz(const QGrid& g) { return qms_csr_layout(g).nnz; }
