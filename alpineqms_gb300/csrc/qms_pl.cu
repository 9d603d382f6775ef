// qms_pl.cu -- the inner solver's operator on the padded node layout (qms_tma.cuh), its
// FP32 diagonal, and the maps between that layout and the reference's unknown order.
//
// qk_op_pl: one CTA of 32 x 8 threads owns a column of nodes and marches 16 k-planes.  Per
// plane, one thread issues two cp.async.bulk.tensor copies: the four unknown blocks of
// plane k+2 (+-1 halo, zero-filled outside the grid) into a four-slot ring, and the six node
// coefficients of plane k+1 into a three-slot ring, each completing on its own mbarrier.
// All threads wait (bounded) for the planes they need and evaluate their node's (up to)
// four rows from shared memory (qms_op_rows.cuh).  The only per-thread global traffic is
// the output row (and the optional dot vector).
#include "qms_internal.h"
#include "qms_df.cuh"
#include "qms_op_rows.cuh"
#include "qms_pl.h"
#include "qms_tile.cuh"

#include <cudaTypedefs.h>
#include <atomic>
#include <mutex>

// ---------------------------------------------------------------------------
// Self-test of the bounded tile wait (mbar_wait_n, the wait every staged kernel uses): one CTA
// waits on an mbarrier that nothing arrives at and no copy targets, gives up after `spins`
// polls, flags QMS_ST_TIMEOUT and returns.  The context stays usable.
// ---------------------------------------------------------------------------
__global__ void qk_wait_selftest(int spins, unsigned* err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    mbar_wait_n(&bar, 0, err, spins);    // the barrier's first phase never completes
}

void qms_launch_wait_selftest(int spins, unsigned* err, cudaStream_t st) {
    qk_wait_selftest<<<1, 32, 0, st>>>(spins, err);
}

// ---------------------------------------------------------------------------
// tensor maps
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

bool qms_make_pl_map(CUtensorMap* map, const void* base, const QGrid& g, int elem_bytes, int arrays, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return false;
    const QPL L = qms_pl(g);
    const cuuint64_t dims[4] = {(cuuint64_t)L.P, (cuuint64_t)g.Ny, (cuuint64_t)g.Nz, (cuuint64_t)arrays};
    const cuuint64_t strides[3] = {(cuuint64_t)L.P * elem_bytes, (cuuint64_t)L.P * g.Ny * elem_bytes,
                                   (cuuint64_t)L.comp * elem_bytes};
    const cuuint32_t box[4] = {PLX, (cuuint32_t)box_rows, 1, (cuuint32_t)arrays};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(map, elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                           const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

bool qms_make_pl16_map(CUtensorMap* map, const void* base, const QGrid& g, int arrays) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return false;
    const long long P16 = qms_pl16_pitch(g);
    const cuuint64_t dims[4] = {(cuuint64_t)P16, (cuuint64_t)g.Ny, (cuuint64_t)g.Nz, (cuuint64_t)arrays};
    const cuuint64_t strides[3] = {(cuuint64_t)P16 * 2, (cuuint64_t)P16 * g.Ny * 2, (cuuint64_t)P16 * g.Ny * g.Nz * 2};
    const cuuint32_t box[4] = {PLX16, (cuuint32_t)PLCY, 1, (cuuint32_t)arrays};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// the bf16 copy of the FP32 node coefficients (padding stays zero: the caller clears it)
__global__ void qk_coef_bf16(QGrid g, const float* __restrict__ nc, __nv_bfloat16* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const QPL L = qms_pl(g);
    const long long src = qms_pl_node(g, L, i, j, k);
    const long long P16 = qms_pl16_pitch(g), comp16 = P16 * g.Ny * g.Nz;
    const long long dst = ((long long)(k - 1) * g.Ny + (j - 1)) * P16 + i;
#pragma unroll
    for (int q = 0; q < 6; q++) out[q * comp16 + dst] = __float2bfloat16_rn(nc[q * L.comp + src]);
}

void qms_launch_coef_bf16(const QGrid& g, const float* nc, __nv_bfloat16* out, cudaStream_t st) {
    const long long P16 = qms_pl16_pitch(g);
    cudaMemsetAsync(out, 0, 6 * P16 * g.Ny * g.Nz * sizeof(__nv_bfloat16), st);
    qk_coef_bf16<<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, nc, out);
}

// ---------------------------------------------------------------------------
// operator on the padded layout
// ---------------------------------------------------------------------------
namespace {

template <typename T>
__device__ __forceinline__ T pl_div(T a, T d) {
    if constexpr (sizeof(T) == 4) return __fdividef(a, d);
    else return a / d;
}

// MODE: QOPH_APPLY (y = M x), QOPH_SCALED (y = D^-1 M x), QOPH_VCOUPLE (V rows only:
// y = w - D^-1 M (x_A, 0)) or QOPH_RESID (T = qdf: y = (float) (w - D^-1 M x), the refinement
// residual in double-float arithmetic, with w the residual of the anchor and x the change of
// the solution since then).  Partials (optional, FP64 across warps): APPLY / SCALED [0] += y . w
// (w may be null), [1] += y . y; RESID |r_A|^2, |r_V|^2; none with VCOUPLE.
template <typename T, int VM, int MODE, typename YT = T, typename WT = T>
__global__ void __launch_bounds__(OTX * OTY, sizeof(T) == 4 ? QMS_STENCIL_MINB : 2)
qk_op_pl(QGrid g, QStepPar<T> P, const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap cmap,
         YT* __restrict__ y, const WT* __restrict__ w, double* __restrict__ partials, unsigned* __restrict__ err,
         WT* __restrict__ yfull = nullptr) {
    // VCOUPLE reads only what the V rows' A couplings need: the three A blocks of x (xmap over
    // them) and the three conductivities (cmap over them)
    constexpr bool VC = MODE == QOPH_VCOUPLE;
    constexpr int C0 = VC ? 3 : 0;
    using TL = PLTiles<T, VC ? 3 : 4, VC ? 3 : 6>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* xsm = reinterpret_cast<T*>(smem_raw);                  // [4 slots][4][PLXY][PLX]
    T* csm = xsm + 4 * TL::XSLOT;                             // [3 slots][6][PLCY][PLX]
    __shared__ __align__(8) uint64_t xbar[4], cbar[3];
    const int tid = threadIdx.x + OTX * threadIdx.y;
    const int i0 = blockIdx.x * OTX + 1, j0 = blockIdx.y * OTY + 1, k0 = blockIdx.z * OKB + 1;
    const int li = threadIdx.x + 1, lj = threadIdx.y + 1;
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    const bool inij = i <= g.Nx && j <= g.Ny;
    const int kend = min(k0 + OKB - 1, g.Nz);
    const QPL L = qms_pl(g);
    // tile origin in tensor coordinates: column i0 - 1 (a multiple of 32), row j0 - 2 (0-based)
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
    // parity of the use of a ring slot by plane kk (planes k0-1, k0, ... fill the slots in turn)
    auto xpar = [&](int kk) { return (unsigned)(((kk - (k0 - 1)) >> 2) & 1); };
    auto cpar = [&](int kk) { return (unsigned)(((kk - (k0 - 1)) / 3) & 1); };
    if (tid == 0) {
        for (int q = 0; q < 4; q++) mbar_init(&xbar[q], 1);
        for (int q = 0; q < 3; q++) mbar_init(&cbar[q], 1);
        fence_mbar_init();
        issue_x(k0 - 1);
        issue_x(k0);
        issue_x(k0 + 1);
        issue_c(k0 - 1);
        issue_c(k0);
    }
    __syncthreads();
    bool ok = mbar_wait(&xbar[(k0 - 1) & 3], xpar(k0 - 1), err) && mbar_wait(&xbar[k0 & 3], xpar(k0), err) &&
              mbar_wait(&cbar[(k0 - 1) % 3], cpar(k0 - 1), err);
    // (i, j) parts of the Dirichlet predicates; rows at plane k0 (padded layout)
    const bool fxA = i <= 2 || i >= g.Nx - 1, fyA = j <= 2 || j >= g.Ny - 1;
    const bool fijX = fyA || i == 1 || i == g.xs, fijY = fxA || j == 1 || j == g.ys, fijZ = fxA || fyA;
    long long rX = qms_pl_node(g, L, i, j, k0);
    const long long plane = (long long)g.Ny * L.P;
    // per-thread sums in FP32 (the dot vectors of the inner solver are FP32 or FP64 already;
    // FP64 arithmetic per row would make the kernel FP64-throughput bound), FP64 across warps
    using RT = float;
    RT red0 = 0, red1 = 0;
    auto emit = [&](long long row, T acc, T diag, bool is_a, T) {
        if constexpr (MODE == QOPH_RESID) {
            const T out = w[row] - acc / diag;
            y[row] = out.h;
            if (yfull) yfull[row] = out;          // the residual in full, for the next solve's anchor
            if (partials) {
                const float o = out.h;
                if (is_a) red0 += o * o;
                else red1 += o * o;
            }
        } else if constexpr (MODE == QOPH_VCOUPLE) {   // the A rows are not wanted (dead code)
            if (!is_a) y[row] = w[row] - pl_div(acc, diag);
        } else {
            const T out = MODE == QOPH_APPLY ? acc : pl_div(acc, diag);
            y[row] = out;
            if (partials) {
                if (w) red0 += (RT)(out * w[row]);
                red1 += (RT)(out * out);
            }
        }
    };
    for (int k = k0; k <= kend; k++) {
        // all threads are done with plane k-1's slots; a copy that never arrived (flagged in
        // *err) ends the sweep for the whole CTA at once
        if (!__syncthreads_and(ok)) break;
        if (tid == 0) {
            fence_proxy_async();
            if (k + 2 <= kend + 1) issue_x(k + 2);   // into the slot of plane k-2
            if (k < kend) issue_c(k + 1);            // into the slot of plane k-2
        }
        ok = mbar_wait(&xbar[(k + 1) & 3], xpar(k + 1), err) && mbar_wait(&cbar[k % 3], cpar(k), err);
        const T* xm = xsm + ((k - 1) & 3) * TL::XSLOT;
        const T* x0 = xsm + (k & 3) * TL::XSLOT;
        const T* xp = xsm + ((k + 1) & 3) * TL::XSLOT;
        const T* cprv = csm + ((k - 1) % 3) * TL::CSLOT;
        const T* ccur = csm + (k % 3) * TL::CSLOT;
        if (inij) {
            auto xsf = [&](int comp, int dk, int dj, int di) -> T {
                if (MODE == QOPH_VCOUPLE && comp == 3) return T(0);
                const T* b = dk < 0 ? xm : (dk > 0 ? xp : x0);
                return b[(comp * PLXY + lj + dj) * PLX + li + di];
            };
            auto cff = [&](int q, int dk, int dj, int di) -> T {
                if (VC && q < C0) return T(0);     // read by the A rows only, which VCOUPLE drops
                return (dk < 0 ? cprv : ccur)[((q - C0) * PLCY + lj + dj) * PLX + li + di];
            };
            const bool kfA = k <= 2 || k >= g.Nz - 1, kfZ = k == 1 || k == g.zs;
            qms_op_node<T, VM>(g, P, i, j, k, fijX, fijY, fijZ, kfA, kfZ, rX, L.comp + rX, 2 * L.comp + rX,
                                3 * L.comp + rX, xsf, cff, emit);
        }
        rX += plane;
    }
    if (partials) {
        __shared__ double sh[32];
        const long long bid = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
        const long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
        double s0 = qBlockSum(red0, sh);
        if (qLinTid() == 0) partials[bid] = s0;
        double s1 = qBlockSum(red1, sh);
        if (qLinTid() == 0) partials[nb + bid] = s1;
    }
}

// dx = x - x0 (FP64 subtraction, reference order) as double-float in the padded layout, with
// the partials |x_A|^2, |x_V|^2 at [2 nb + block] and [3 nb + block] (gridDim.x == nb)
__global__ void __launch_bounds__(256) qk_delta_split(QGrid g, const double* __restrict__ x,
                                                      const double* __restrict__ x0, qdf* __restrict__ dx,
                                                      double* __restrict__ partials) {
    const QPL L = qms_pl(g);
    float xa = 0.f, xv = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.Nn; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.Nx) + 1, j = (int)((t / g.Nx) % g.Ny) + 1, k = (int)(t / ((long long)g.Nx * g.Ny)) + 1;
        const long long nd = qms_pl_node(g, L, i, j, k);
        auto one = [&](long long ref, long long pl, float& acc) {
            const double v = x[ref];
            dx[pl] = qdf_split(v - x0[ref]);
            const float f = qdf_split(v).h;
            acc += f * f;
        };
        if (i <= g.xs) one(qAX(g, i, j, k), nd, xa);
        if (j <= g.ys) one(qAY(g, i, j, k), L.comp + nd, xa);
        if (k <= g.zs) one(qAZ(g, i, j, k), 2 * L.comp + nd, xa);
        one(qV(g, i, j, k), 3 * L.comp + nd, xv);
    }
    __shared__ double sh[32];
    const double sa = qBlockSum(xa, sh);
    if (threadIdx.x == 0) partials[2 * (long long)gridDim.x + blockIdx.x] = sa;
    const double sv = qBlockSum(xv, sh);
    if (threadIdx.x == 0) partials[3 * (long long)gridDim.x + blockIdx.x] = sv;
}

// 1 / diag M (transient form), formed in FP64 like the rows' own diagonal, as double-float
__global__ void qk_dinv_df(QGrid g, QCoef<double> c, QStepPar<double> P, qdf* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const QPL L = qms_pl(g);
    const long long t = qms_pl_node(g, L, i, j, k);
    if (i <= g.xs) {
        double d = 1.0;
        if (!qFixX(g, i, j, k))
            d = (c.imuz(i, j, k) + c.imuz(i, j - 1, k)) * P.idy2 + (c.imuy(i, j, k) + c.imuy(i, j, k - 1)) * P.idz2 +
                (c.imux(i, j, k) + c.imux(i - 1, j, k)) * P.idx2 + c.sgx(i, j, k) * P.idt;
        out[t] = qdf_split(1.0 / d);
    }
    if (j <= g.ys) {
        double d = 1.0;
        if (!qFixY(g, i, j, k))
            d = (c.imuz(i, j, k) + c.imuz(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j, k - 1)) * P.idz2 +
                (c.imuy(i, j, k) + c.imuy(i, j - 1, k)) * P.idy2 + c.sgy(i, j, k) * P.idt;
        out[L.comp + t] = qdf_split(1.0 / d);
    }
    if (k <= g.zs) {
        double d = 1.0;
        if (!qFixZ(g, i, j, k))
            d = (c.imuy(i, j, k) + c.imuy(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j - 1, k)) * P.idy2 +
                (c.imuz(i, j, k) + c.imuz(i, j, k - 1)) * P.idz2 + c.sgz(i, j, k) * P.idt;
        out[2 * L.comp + t] = qdf_split(1.0 / d);
    }
    double d = 1.0;
    if (!qFixV(g, i, j, k)) {
        const double f = P.sigfloor;
        d = (fmax(c.sgx(i, j, k), f) + fmax(c.sgx(i - 1, j, k), f)) * P.idx2 +
            (fmax(c.sgy(i, j, k), f) + fmax(c.sgy(i, j - 1, k), f)) * P.idy2 +
            (fmax(c.sgz(i, j, k), f) + fmax(c.sgz(i, j, k - 1), f)) * P.idz2;
    }
    out[3 * L.comp + t] = qdf_split(1.0 / d);
}

// The polynomial extrapolation of the state from the last solutions (x the newest, xo1 the one
// before, ...), the start of the next solve: order 1 x = 2 x - xo1, order 2 x = 3 (x - xo1) + xo2,
// order 3 x = 4 (x + xo2) - 6 xo1 - xo3; in fused multiply-adds (1, 2, 3 FP64 operations)
__device__ __forceinline__ double qms_extrap(int order, double x, double x1, double x2, double x3) {
    if (order == 1) return fma(2.0, x, -x1);
    if (order == 2) return fma(3.0, x - x1, x2);
    return fma(-6.0, x1, fma(4.0, x + x2, -x3));
}

// The extrapolated start on the rows that are not Dirichlet rows (those keep the values just
// written)
__global__ void qk_extrapolate(QGrid g, double* __restrict__ x, const double* __restrict__ xold,
                               const double* __restrict__ xold2, const double* __restrict__ xold3, int order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    auto one = [&](long long r) {
        x[r] = qms_extrap(order, x[r], xold[r], order >= 2 ? xold2[r] : 0.0, order >= 3 ? xold3[r] : 0.0);
    };
    if (i <= g.xs && !qFixX(g, i, j, k)) one(qAX(g, i, j, k));
    if (j <= g.ys && !qFixY(g, i, j, k)) one(qAY(g, i, j, k));
    if (k <= g.zs && !qFixZ(g, i, j, k)) one(qAZ(g, i, j, k));
    if (!qFixV(g, i, j, k)) one(qV(g, i, j, k));
}

// The start of a transient step chained to the previous one, in one pass over the unknowns:
//   r0 = rfin + D^-1 (b - b_prev)      the anchor: the residual of x_n, the previous solution,
//                                      against the new right-hand side
//   w  = r0_prev - rfin = D^-1 M (x_n - x_{n-1})    (into wnew; when the previous step's own
//                                      anchor state was x_{n-1})
// x extrapolated to order xo (qk_extrapolate's formulas), and with rfloat the residual of that
// x by linearity from the anchor and the differences w of the last steps (w1 = the stored w of
// the step before, w2 the one before that):
//   xo 1: x = x_n + d_n                     r = r0 - w
//   xo 2: x = x_n + 2 d_n - d_{n-1}         r = r0 - (2 w - w1)
//   xo 3: x = x_n + 3 d_n - 3 d_{n-1} + d_{n-2}    r = r0 - (3 (w - w1) + w2)
// (d_n = x_n - x_{n-1}; valid when the Dirichlet values are the same in all these states), into
// rfloat (FP32), rfin (in full) and the partials |r_A|^2, |r_V|^2, |x_A|^2, |x_V|^2 of the
// launch's blocks.
// b - b_prev comes either from the two FP64 right-hand sides (b, bprev), or, with hx (a copy of
// x_n) and the edge sigma sg, sdt = sg / dt, from the linear map that forms the transient
// right-hand side, applied to d_n = hx - xo1 in double-float (the Dirichlet values unchanged):
//   A rows  sdt d_n,    V rows  sum over the axes (sg_e d_e - sg_e' d_e') / (dt h)
// with e, e' the node's two incident edges along the axis.  That skips the FP64 right-hand side
// (FP64 issue is scarce on GB300); x0 then receives x_n here.
// A block is 64 nodes x 4 components (thread c = threadIdx.x / 64): the V rows take the
// products sg_e d_e of their own node's edges and of the edge before along x from the A threads
// through shared memory.  Node indices are 32-bit (2^32 nodes would need terabytes of state).
struct QStartRhs {
    const double* hx;               // x_n (null: b - b_prev from b and bprev)
    const double* sg;
    const double* sdt;
    qdf idt[3];                     // 1 / (dt dx), 1 / (dt dy), 1 / (dt dz)
    double* x0;                     // receives x_n
};
// dp (optional): the pointers of the history buffers that rotate from step to step, read from
// device memory instead of the arguments (a step captured in a CUDA graph replays with the
// pointers of the step it runs)
//
// LS (the first pass of the least-squares start, qms_launch_step_start): r0 and w as above, x and
// the residual left alone; instead each block sums, for the ls directions of the difference basis
//   u1 = w,  u2 = w - w1,  u3 = w - 2 w1 + w2,  u4 = w - 3 w1 + 3 w2 - w3
// (the residual images of d_n and of its backward differences: nearly independent, unlike the
// w themselves), the Gram matrix u_i . u_j, the products u_i . r_b with the residual r_b of the
// polynomial start of order min(ls, 3) (r_b = r0 - u1 - u2 - u3), and r_b . r_b, into lsp
// (QMS_LS_SUMS x nb, quantity-major).  The basis and r_b in float (from both words of each
// double-float value), products summed per thread in float and across the block in double: the
// solve only needs the coefficients to a few digits, because the apply pass forms the residual
// of the start it writes exactly (by linearity).  The launch is one resident wave of blocks.
template <bool LS>
__global__ void __launch_bounds__(256, 4) qk_step_start(
    QGrid g, qdf* __restrict__ rfin, const double* b_a, const double* bprev_a, const qdf* __restrict__ dinv,
    qdf* __restrict__ r0, double* __restrict__ x, const double* xo1_a, const double* xo2_a, const double* xo3_a,
    const int xo, qdf* wnew_a, const qdf* w1_a, const qdf* w2_a, float* __restrict__ rfloat,
    double* __restrict__ partials, const QStartRhs R, const QStepPtrs* __restrict__ dp, const qdf* w3_a,
    double* __restrict__ lsp) {
    __shared__ qdf prod[3][64];
    const QPL L = qms_pl(g);
    const int c = threadIdx.x >> 6, lane = threadIdx.x & 63;
    const unsigned Nx = (unsigned)g.Nx, Nxy = (unsigned)g.Nx * (unsigned)g.Ny, Nn = (unsigned)g.Nn;
    const double* __restrict__ b = dp ? dp->b : b_a;
    const double* __restrict__ bprev = dp ? dp->bprev : bprev_a;
    const double* __restrict__ xo1 = dp ? dp->xo1 : xo1_a;
    const double* __restrict__ xo2 = dp ? dp->xo2 : xo2_a;
    const double* __restrict__ xo3 = dp ? dp->xo3 : xo3_a;
    qdf* __restrict__ wnew = dp ? dp->wnew : wnew_a;
    const qdf* __restrict__ w1 = dp ? dp->w1 : w1_a;
    const qdf* __restrict__ w2 = dp ? dp->w2 : w2_a;
    const double* __restrict__ hx = dp ? dp->hx : R.hx;
    const double* __restrict__ sg = R.sg;
    const qdf* __restrict__ w3 = dp ? dp->w3 : w3_a;
    float racc = 0.f, xacc = 0.f;
    float ls_acc[QMS_LS_SUMS];
    if constexpr (LS) {
#pragma unroll
        for (int q = 0; q < QMS_LS_SUMS; q++) ls_acc[q] = 0.f;
    }
    for (unsigned base = blockIdx.x * 64u; base < Nn; base += gridDim.x * 64u) {
        const unsigned t = base + lane;
        const bool valid = t < Nn;
        const unsigned tt = valid ? t : 0u;
        const unsigned kk = tt / Nxy, rem = tt - kk * Nxy, jj = rem / Nx;
        const int i = (int)(rem - jj * Nx) + 1, j = (int)jj + 1, k = (int)kk + 1;
        bool has;
        long long ref;
        bool fix;
        if (c == 0) { has = valid && i <= g.xs; ref = has ? qAX(g, i, j, k) : 0; fix = qFixX(g, i, j, k); }
        else if (c == 1) { has = valid && j <= g.ys; ref = has ? qAY(g, i, j, k) : 0; fix = qFixY(g, i, j, k); }
        else if (c == 2) { has = valid && k <= g.zs; ref = has ? qAZ(g, i, j, k) : 0; fix = qFixZ(g, i, j, k); }
        else { has = valid; ref = has ? qV(g, i, j, k) : 0; fix = qFixV(g, i, j, k); }
        const long long pl = c * L.comp + qms_pl_node(g, L, i, j, k);
        const bool ex = has && xo > 0 && !fix;
        double xs = 0.0, x1 = 0.0;
        qdf db;
        if (has) {
            xs = x[ref];
            if (ex || (hx && !fix)) x1 = xo1[ref];
        }
        if (hx) {
            // the right-hand side's change from d_n; the A threads leave sg_e d_e for the V rows
            if (c < 3) {
                qdf p, q;
                if (has && !fix) {
                    const qdf d = qdf_split(hx[ref] - x1);
                    p = qdf_split(sg[ref]) * d;
                    q = qdf_split(R.sdt[ref]) * d;
                }
                prod[c][lane] = p;
                db = q;
            }
            __syncthreads();
            if (c == 3 && has && !fix) {
                // edge products of the V row's incident edges: its own node's from shared memory,
                // the ones before along y and z (and along x at the first lane) formed here
                auto edge = [&](long long e) { return qdf_split(sg[e]) * qdf_split(hx[e] - xo1[e]); };
                const qdf pxm = lane > 0 ? prod[0][lane - 1] : edge(qAX(g, i - 1, j, k));
                db = (prod[0][lane] - pxm) * R.idt[0] + (prod[1][lane] - edge(qAY(g, i, j - 1, k))) * R.idt[1] +
                     (prod[2][lane] - edge(qAZ(g, i, j, k - 1))) * R.idt[2];
            }
            __syncthreads();
        } else if (has) {
            db = qdf_split(b[ref] - bprev[ref]);
        }
        if (!has) continue;
        const qdf rf = rfin[pl];
        const qdf a = rf + db * dinv[pl];
        qdf w;
        if (wnew) {
            w = r0[pl] - rf;
            wnew[pl] = w;
        }
        r0[pl] = a;
        if (R.x0) R.x0[ref] = xs;
        if constexpr (LS) {
            // xo = ls >= 1 directions; wnew is formed (w).  The differences in float from both
            // words (consecutive w agree to a few per cent, so each word's difference is nearly
            // exact): the sums only steer the coefficients
            const qdf v1 = xo >= 2 ? w1[pl] : qdf(), v2 = xo >= 3 ? w2[pl] : qdf(), v3 = xo >= 4 ? w3[pl] : qdf();
            const float d1 = (w.h - v1.h) + (w.l - v1.l);        // w - w1
            const float d2 = (v1.h - v2.h) + (v1.l - v2.l);      // w1 - w2
            const float d3 = (v2.h - v3.h) + (v2.l - v3.l);      // w2 - w3
            const float u2 = d1, u3 = d1 - d2, u4 = (d1 - d2) - (d2 - d3);
            float rb = (a.h - w.h) + (a.l - w.l);
            if (xo >= 2) rb -= u2;
            if (xo >= 3) rb -= u3;
            const float u[4] = {w.h + w.l, xo >= 2 ? u2 : 0.f, xo >= 3 ? u3 : 0.f, xo >= 4 ? u4 : 0.f};
            int q = 0;
#pragma unroll
            for (int i0 = 0; i0 < 4; i0++)
#pragma unroll
                for (int j0 = i0; j0 < 4; j0++) ls_acc[q++] += u[i0] * u[j0];
#pragma unroll
            for (int i0 = 0; i0 < 4; i0++) ls_acc[10 + i0] += u[i0] * rb;
            ls_acc[14] += rb * rb;
            continue;
        }
        if (ex) {
            xs = qms_extrap(xo, xs, x1, xo >= 2 ? xo2[ref] : 0.0, xo >= 3 ? xo3[ref] : 0.0);
            x[ref] = xs;
        }
        if (rfloat) {
            qdf d = w;
            if (xo == 2) d = (w + w) - w1[pl];
            else if (xo == 3) d = qdf(3.f) * (w - w1[pl]) + w2[pl];
            const qdf r = a - d;
            rfloat[pl] = r.h;
            rfin[pl] = r;
            racc += r.h * r.h;
            const float f = qdf_split(xs).h;
            xacc += f * f;
        }
    }
    __shared__ double sh[32];
    const long long nb = gridDim.x;
    if constexpr (LS) {
#pragma unroll
        for (int q = 0; q < QMS_LS_SUMS; q++) {
            const double t = qBlockSum(ls_acc[q], sh);
            if (threadIdx.x == 0) lsp[q * nb + blockIdx.x] = t;
        }
        return;
    }
    if (!rfloat) return;
    double s = qBlockSum(c < 3 ? racc : 0.f, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    s = qBlockSum(c < 3 ? 0.f : racc, sh);
    if (threadIdx.x == 0) partials[nb + blockIdx.x] = s;
    s = qBlockSum(c < 3 ? xacc : 0.f, sh);
    if (threadIdx.x == 0) partials[2 * nb + blockIdx.x] = s;
    s = qBlockSum(c < 3 ? 0.f : xacc, sh);
    if (threadIdx.x == 0) partials[3 * nb + blockIdx.x] = s;
}

// The coefficients of the least-squares start from the partial sums of its first pass (one
// block): the sums over the blocks in a fixed order, then the normal equations G c = h of the
// ls directions of the difference basis, scaled to a unit diagonal and solved by Cholesky; a
// direction whose pivot falls below 1e-5 (numerically dependent at the float accuracy of the
// sums) gets no coefficient.  The start is the polynomial one (base coefficients 1 on
// u1..u_min(ls,3)) plus c; out[0..3] = its coefficients g_j on d_1..d_4 (g = T^T (base + c) for the
// map u = T w), out[4] = |r_b|^2, out[5] = the predicted |r|^2 of the start, out[6] = the
// directions used.  Non-finite sums leave the polynomial start.
__global__ void __launch_bounds__(256) qk_ls_solve(const double* __restrict__ lsp, long long nb, int ls,
                                                  double* __restrict__ out) {
    __shared__ double sh[32];
    __shared__ double tot[QMS_LS_SUMS];
    for (int q = 0; q < QMS_LS_SUMS; q++) {
        double t = 0.0;
        for (long long b = threadIdx.x; b < nb; b += blockDim.x) t += lsp[q * nb + b];
        t = qBlockSum(t, sh);
        if (threadIdx.x == 0) tot[q] = t;
    }
    if (threadIdx.x != 0) return;
    double G[4][4], h[4], sc[4], A[4][4], L[4][4], z[4], c[4];
    int q = 0;
    for (int i = 0; i < 4; i++)
        for (int j = i; j < 4; j++) { G[i][j] = tot[q]; G[j][i] = tot[q]; q++; }
    for (int i = 0; i < 4; i++) h[i] = tot[10 + i];
    const double rb2 = tot[14];
    bool on[4];
    for (int i = 0; i < 4; i++) {
        on[i] = i < ls && G[i][i] > 0.0 && isfinite(G[i][i]) && isfinite(h[i]);
        sc[i] = on[i] ? sqrt(G[i][i]) : 1.0;
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) A[i][j] = on[i] && on[j] ? G[i][j] / (sc[i] * sc[j]) : (i == j ? 1.0 : 0.0);
    int used = 0;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) L[i][j] = 0.0;
    for (int k = 0; k < 4; k++) {
        if (!on[k]) { L[k][k] = 1.0; z[k] = 0.0; continue; }
        double d = A[k][k];
        for (int m = 0; m < k; m++) d -= L[k][m] * L[k][m];
        if (!(d > 1e-5)) {                       // dependent on the directions before it
            on[k] = false;
            L[k][k] = 1.0;
            z[k] = 0.0;
            continue;
        }
        L[k][k] = sqrt(d);
        for (int i = k + 1; i < 4; i++) {
            if (!on[i]) continue;
            double t = A[i][k];
            for (int m = 0; m < k; m++) t -= L[i][m] * L[k][m];
            L[i][k] = t / L[k][k];
        }
        double t = h[k] / sc[k];
        for (int m = 0; m < k; m++) t -= L[k][m] * z[m];
        z[k] = t / L[k][k];
        used++;
    }
    for (int k = 3; k >= 0; k--) {
        double t = z[k];
        for (int m = k + 1; m < 4; m++) t -= L[m][k] * c[m];
        c[k] = on[k] ? t / L[k][k] : 0.0;
    }
    bool ok = true;
    for (int k = 0; k < 4; k++) { c[k] = on[k] ? c[k] / sc[k] : 0.0; ok = ok && isfinite(c[k]); }
    double pred = rb2;
    if (ok) {
        for (int i = 0; i < 4; i++) {
            pred -= 2.0 * c[i] * h[i];
            for (int j = 0; j < 4; j++) pred += c[i] * G[i][j] * c[j];
        }
    }
    if (!ok) {
        for (int k = 0; k < 4; k++) c[k] = 0.0;
        pred = rb2;
        used = 0;
    }
    const int p = ls < 3 ? ls : 3;              // the polynomial base
    double u[4];
    for (int k = 0; k < 4; k++) u[k] = (k < p ? 1.0 : 0.0) + c[k];
    out[0] = u[0] + u[1] + u[2] + u[3];
    out[1] = -u[1] - 2.0 * u[2] - 3.0 * u[3];
    out[2] = u[2] + 3.0 * u[3];
    out[3] = -u[3];
    out[4] = rb2;
    out[5] = pred;
    out[6] = (double)used;
}

// The second pass of the least-squares start: with the coefficients g (qk_ls_solve)
//   x = x_n + sum_j g_j d_j   (the rows that are not Dirichlet rows)
//   r = r0 - sum_j g_j w_j    (w_1 = w, the one this step formed; in double-float)
// into x, rfin, rfloat (FP32) and the partials |r_A|^2, |r_V|^2, |x_A|^2, |x_V|^2 of the launch's
// blocks, the layout and block shape of qk_step_start.
__global__ void __launch_bounds__(256) qk_start_apply(
    QGrid g, double* __restrict__ x, const double* xo1_a, const double* xo2_a, const double* xo3_a,
    const double* xo4_a, const int ls, const qdf* __restrict__ r0, const qdf* wnew_a, const qdf* w1_a,
    const qdf* w2_a, const qdf* w3_a, const double* __restrict__ coef, qdf* __restrict__ rfin,
    float* __restrict__ rfloat, double* __restrict__ partials, const QStepPtrs* __restrict__ dp) {
    const QPL L = qms_pl(g);
    const int c = threadIdx.x >> 6, lane = threadIdx.x & 63;
    const unsigned Nx = (unsigned)g.Nx, Nxy = (unsigned)g.Nx * (unsigned)g.Ny, Nn = (unsigned)g.Nn;
    const double* __restrict__ xo1 = dp ? dp->xo1 : xo1_a;
    const double* __restrict__ xo2 = dp ? dp->xo2 : xo2_a;
    const double* __restrict__ xo3 = dp ? dp->xo3 : xo3_a;
    const double* __restrict__ xo4 = dp ? dp->xo4 : xo4_a;
    const qdf* __restrict__ w0 = dp ? dp->wnew : wnew_a;
    const qdf* __restrict__ w1 = dp ? dp->w1 : w1_a;
    const qdf* __restrict__ w2 = dp ? dp->w2 : w2_a;
    const qdf* __restrict__ w3 = dp ? dp->w3 : w3_a;
    const double g1 = coef[0], g2 = coef[1], g3 = coef[2], g4 = coef[3];
    const qdf q1 = qdf_split(g1), q2 = qdf_split(g2), q3 = qdf_split(g3), q4 = qdf_split(g4);
    // x_n + sum_j g_j d_j as one combination of the states (FP64 issue is scarce on GB300)
    const double c0 = 1.0 + g1, c1 = g2 - g1, c2 = g3 - g2, c3 = g4 - g3, c4 = -g4;
    float racc = 0.f, xacc = 0.f;
    for (unsigned base = blockIdx.x * 64u; base < Nn; base += gridDim.x * 64u) {
        const unsigned t = base + lane;
        if (t >= Nn) continue;
        const unsigned kk = t / Nxy, rem = t - kk * Nxy, jj = rem / Nx;
        const int i = (int)(rem - jj * Nx) + 1, j = (int)jj + 1, k = (int)kk + 1;
        bool has, fix;
        long long ref;
        if (c == 0) { has = i <= g.xs; ref = has ? qAX(g, i, j, k) : 0; fix = qFixX(g, i, j, k); }
        else if (c == 1) { has = j <= g.ys; ref = has ? qAY(g, i, j, k) : 0; fix = qFixY(g, i, j, k); }
        else if (c == 2) { has = k <= g.zs; ref = has ? qAZ(g, i, j, k) : 0; fix = qFixZ(g, i, j, k); }
        else { has = true; ref = qV(g, i, j, k); fix = qFixV(g, i, j, k); }
        if (!has) continue;
        const long long pl = c * L.comp + qms_pl_node(g, L, i, j, k);
        qdf s = q1 * w0[pl];
        if (ls >= 2) s = s + q2 * w1[pl];
        if (ls >= 3) s = s + q3 * w2[pl];
        if (ls >= 4) s = s + q4 * w3[pl];
        const qdf r = r0[pl] - s;
        double xs = x[ref];
        if (!fix) {
            double t = c1 * xo1[ref];
            if (ls >= 2) t = fma(c2, xo2[ref], t);
            if (ls >= 3) t = fma(c3, xo3[ref], t);
            if (ls >= 4) t = fma(c4, xo4[ref], t);
            xs = fma(c0, xs, t);
            x[ref] = xs;
        }
        rfloat[pl] = r.h;
        rfin[pl] = r;
        racc += r.h * r.h;
        const float f = qdf_split(xs).h;
        xacc += f * f;
    }
    __shared__ double sh[32];
    const long long nb = gridDim.x;
    double s = qBlockSum(c < 3 ? racc : 0.f, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    s = qBlockSum(c < 3 ? 0.f : racc, sh);
    if (threadIdx.x == 0) partials[nb + blockIdx.x] = s;
    s = qBlockSum(c < 3 ? xacc : 0.f, sh);
    if (threadIdx.x == 0) partials[2 * nb + blockIdx.x] = s;
    s = qBlockSum(c < 3 ? 0.f : xacc, sh);
    if (threadIdx.x == 0) partials[3 * nb + blockIdx.x] = s;
}

// The residual is the anchor itself (x is the anchor state): r = r0 into rfloat (FP32) and rfull,
// with the partials |r_A|^2, |r_V|^2, |x_A|^2, |x_V|^2 of gridDim.x (= nb) blocks
__global__ void __launch_bounds__(256) qk_anchor_resid(QGrid g, const qdf* __restrict__ r0, const double* __restrict__ x,
                                                       float* __restrict__ rfloat, qdf* __restrict__ rfull,
                                                       double* __restrict__ partials) {
    const QPL L = qms_pl(g);
    float ra = 0.f, rv = 0.f, xa = 0.f, xv = 0.f;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.Nn; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.Nx) + 1, j = (int)((t / g.Nx) % g.Ny) + 1, k = (int)(t / ((long long)g.Nx * g.Ny)) + 1;
        const long long nd = qms_pl_node(g, L, i, j, k);
        auto one = [&](long long ref, long long pl, float& racc, float& xacc) {
            const qdf r = r0[pl];
            rfloat[pl] = r.h;
            rfull[pl] = r;
            racc += r.h * r.h;
            const float f = qdf_split(x[ref]).h;
            xacc += f * f;
        };
        if (i <= g.xs) one(qAX(g, i, j, k), nd, ra, xa);
        if (j <= g.ys) one(qAY(g, i, j, k), L.comp + nd, ra, xa);
        if (k <= g.zs) one(qAZ(g, i, j, k), 2 * L.comp + nd, ra, xa);
        one(qV(g, i, j, k), 3 * L.comp + nd, rv, xv);
    }
    __shared__ double sh[32];
    const long long nb = gridDim.x;
    double s = qBlockSum(ra, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    s = qBlockSum(rv, sh);
    if (threadIdx.x == 0) partials[nb + blockIdx.x] = s;
    s = qBlockSum(xa, sh);
    if (threadIdx.x == 0) partials[2 * nb + blockIdx.x] = s;
    s = qBlockSum(xv, sh);
    if (threadIdx.x == 0) partials[3 * nb + blockIdx.x] = s;
}

// double -> double-float, reference unknown order -> padded layout; its high words also to hi
// when given
__global__ void qk_split_ref_pl(QGrid g, const double* __restrict__ src, qdf* __restrict__ dst,
                                float* __restrict__ hi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const QPL L = qms_pl(g);
    const long long t = qms_pl_node(g, L, i, j, k);
    auto one = [&](long long ref, long long pl) {
        const qdf v = qdf_split(src[ref]);
        dst[pl] = v;
        if (hi) hi[pl] = v.h;
    };
    if (i <= g.xs) one(qAX(g, i, j, k), t);
    if (j <= g.ys) one(qAY(g, i, j, k), L.comp + t);
    if (k <= g.zs) one(qAZ(g, i, j, k), 2 * L.comp + t);
    one(qV(g, i, j, k), 3 * L.comp + t);
}

// elementwise double -> double-float (the node coefficients)
__global__ void qk_split_flat(long long n, const double* __restrict__ src, qdf* __restrict__ dst) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = qdf_split(src[t]);
}

// out = r * scale[0] (padded layout, FP32)
__global__ void qk_pl_scale(long long n, const float* __restrict__ r, const double* __restrict__ scale,
                            float* __restrict__ out) {
    const float s = (float)scale[0];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = r[t] * s;
}

// FP32 diagonal of the operator in the padded layout (Dirichlet rows 1)
__global__ void qk_diag_pl(QGrid g, QCoef<float> c, QStepPar<float> P, float* __restrict__ dg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const QPL L = qms_pl(g);
    const long long t = qms_pl_node(g, L, i, j, k);
    if (i <= g.xs) {
        float d = 1.f;
        if (!qFixX(g, i, j, k))
            d = (c.imuz(i, j, k) + c.imuz(i, j - 1, k)) * P.idy2 + (c.imuy(i, j, k) + c.imuy(i, j, k - 1)) * P.idz2 +
                (c.imux(i, j, k) + c.imux(i - 1, j, k)) * P.idx2 + c.sgx(i, j, k) * P.idt;
        dg[t] = d;
    }
    if (j <= g.ys) {
        float d = 1.f;
        if (!qFixY(g, i, j, k))
            d = (c.imuz(i, j, k) + c.imuz(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j, k - 1)) * P.idz2 +
                (c.imuy(i, j, k) + c.imuy(i, j - 1, k)) * P.idy2 + c.sgy(i, j, k) * P.idt;
        dg[L.comp + t] = d;
    }
    if (k <= g.zs) {
        float d = 1.f;
        if (!qFixZ(g, i, j, k))
            d = (c.imuy(i, j, k) + c.imuy(i - 1, j, k)) * P.idx2 + (c.imux(i, j, k) + c.imux(i, j - 1, k)) * P.idy2 +
                (c.imuz(i, j, k) + c.imuz(i, j, k - 1)) * P.idz2 + c.sgz(i, j, k) * P.idt;
        dg[2 * L.comp + t] = d;
    }
    float d = 1.f;
    if (!qFixV(g, i, j, k)) {
        const float f = P.sigfloor;
        d = (fmaxf(c.sgx(i, j, k), f) + fmaxf(c.sgx(i - 1, j, k), f)) * P.idx2 +
            (fmaxf(c.sgy(i, j, k), f) + fmaxf(c.sgy(i, j - 1, k), f)) * P.idy2 +
            (fmaxf(c.sgz(i, j, k), f) + fmaxf(c.sgz(i, j, k - 1), f)) * P.idz2;
    }
    dg[3 * L.comp + t] = d;
}

// out[PL] = (T)(r64[ref] * scale[0])
template <typename T>
__global__ void qk_pl_from_ref(QGrid g, const double* __restrict__ r64, const double* __restrict__ scale,
                               T* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const QPL L = qms_pl(g);
    const long long t = qms_pl_node(g, L, i, j, k);
    const double s = scale ? scale[0] : 1.0;
    if (i <= g.xs) out[t] = (T)(r64[qAX(g, i, j, k)] * s);
    if (j <= g.ys) out[L.comp + t] = (T)(r64[qAY(g, i, j, k)] * s);
    if (k <= g.zs) out[2 * L.comp + t] = (T)(r64[qAZ(g, i, j, k)] * s);
    out[3 * L.comp + t] = (T)(r64[qV(g, i, j, k)] * s);
}

// x[ref] += scale[0] * e[PL]
template <typename T>
__global__ void qk_ref_add_pl(QGrid g, const T* __restrict__ e, const double* __restrict__ scale,
                              double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.Nx || j > g.Ny) return;
    const QPL L = qms_pl(g);
    const long long t = qms_pl_node(g, L, i, j, k);
    const double s = scale[0];
    if (i <= g.xs) x[qAX(g, i, j, k)] += s * (double)e[t];
    if (j <= g.ys) x[qAY(g, i, j, k)] += s * (double)e[L.comp + t];
    if (k <= g.zs) x[qAZ(g, i, j, k)] += s * (double)e[2 * L.comp + t];
    x[qV(g, i, j, k)] += s * (double)e[3 * L.comp + t];
}

}  // namespace

dim3 qms_node_grid(const QGrid& g) {
    return dim3((g.Nx + QMS_NODE_BX - 1) / QMS_NODE_BX, (g.Ny + QMS_NODE_BY - 1) / QMS_NODE_BY, g.Nz);
}
dim3 qms_node_block() { return dim3(QMS_NODE_BX, QMS_NODE_BY, 1); }

// The velocity components a step uses pick the instantiation: no advection term, one axis, or
// the general form (FP64 inner vectors: none or general).
__host__ __forceinline__ bool qms_nonzero(float v) { return v != 0.f; }
__host__ __forceinline__ bool qms_nonzero(double v) { return v != 0.0; }
__host__ __forceinline__ bool qms_nonzero(const qdf& v) { return v.h != 0.f || v.l != 0.f; }
template <typename T>
static int qms_vel_mask(const QStepPar<T>& P, bool adv, bool axes) {
    if (!adv) return 0;
    const int m = (qms_nonzero(P.vx) ? 1 : 0) | (qms_nonzero(P.vy) ? 2 : 0) | (qms_nonzero(P.vz) ? 4 : 0);
    return axes && (m == 1 || m == 2 || m == 4) ? m : 7;
}

// STMT with the constant VM set to the mask's instantiation
#define QMS_WITH_VM(vm, STMT)                                 \
    switch (vm) {                                             \
        case 0: { constexpr int VM = 0; STMT; } break;        \
        case 1: { constexpr int VM = 1; STMT; } break;        \
        case 2: { constexpr int VM = 2; STMT; } break;        \
        case 4: { constexpr int VM = 4; STMT; } break;        \
        default: { constexpr int VM = 7; STMT; } break;       \
    }

template <typename T, int VM>
static void op_pl_attrs(int shm) {
    cudaFuncSetAttribute(qk_op_pl<T, VM, QOPH_APPLY>, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
    cudaFuncSetAttribute(qk_op_pl<T, VM, QOPH_SCALED>, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
    cudaFuncSetAttribute(qk_op_pl<T, VM, QOPH_VCOUPLE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)PLTiles<T, 3, 3>::SMEM);
}

template <typename T>
static void op_pl_prepare() {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    const int shm = (int)PLTiles<T>::SMEM;
    op_pl_attrs<T, 0>(shm);
    op_pl_attrs<T, 7>(shm);
    if constexpr (sizeof(T) == 4) {
        op_pl_attrs<T, 1>(shm);
        op_pl_attrs<T, 2>(shm);
        op_pl_attrs<T, 4>(shm);
        const int shd = (int)PLTiles<qdf>::SMEM;
        cudaFuncSetAttribute(qk_op_pl<qdf, 0, QOPH_RESID, float, qdf>, cudaFuncAttributeMaxDynamicSharedMemorySize, shd);
        cudaFuncSetAttribute(qk_op_pl<qdf, 1, QOPH_RESID, float, qdf>, cudaFuncAttributeMaxDynamicSharedMemorySize, shd);
        cudaFuncSetAttribute(qk_op_pl<qdf, 2, QOPH_RESID, float, qdf>, cudaFuncAttributeMaxDynamicSharedMemorySize, shd);
        cudaFuncSetAttribute(qk_op_pl<qdf, 4, QOPH_RESID, float, qdf>, cudaFuncAttributeMaxDynamicSharedMemorySize, shd);
        cudaFuncSetAttribute(qk_op_pl<qdf, 7, QOPH_RESID, float, qdf>, cudaFuncAttributeMaxDynamicSharedMemorySize, shd);
    }
    done.fetch_or(bit, std::memory_order_acq_rel);
}

long long qms_op_pl_num_blocks(const QGrid& g) {
    return (long long)((g.Nx + OTX - 1) / OTX) * ((g.Ny + OTY - 1) / OTY) * ((g.Nz + OKB - 1) / OKB);
}

template <typename T, int VM>
static void op_pl_launch(dim3 gs, dim3 bs, size_t shm, cudaStream_t st, int mode, const QGrid& g,
                         const QStepPar<T>& P, const CUtensorMap& xmap, const CUtensorMap& cmap, T* y, const T* w,
                         double* partials, unsigned* err) {
    if constexpr (sizeof(T) == 8 && VM != 0 && VM != 7) {
        return;                                   // FP64 inner vectors: no or general advection only
    } else {
        if (mode == QOPH_APPLY)
            qk_op_pl<T, VM, QOPH_APPLY><<<gs, bs, shm, st>>>(g, P, xmap, cmap, y, w, partials, err);
        else if (mode == QOPH_VCOUPLE)
            qk_op_pl<T, VM, QOPH_VCOUPLE><<<gs, bs, PLTiles<T, 3, 3>::SMEM, st>>>(g, P, xmap, cmap, y, w, partials,
                                                                                    err);
        else
            qk_op_pl<T, VM, QOPH_SCALED><<<gs, bs, shm, st>>>(g, P, xmap, cmap, y, w, partials, err);
    }
}

template <typename T>
void qms_launch_op_pl(const QGrid& g, const QStepPar<T>& P, const CUtensorMap& xmap, const CUtensorMap& cmap, bool adv,
                      int mode, T* y, const T* w, double* partials, unsigned* err, cudaStream_t st) {
    op_pl_prepare<T>();
    const dim3 bs(OTX, OTY, 1), gs((g.Nx + OTX - 1) / OTX, (g.Ny + OTY - 1) / OTY, (g.Nz + OKB - 1) / OKB);
    const size_t shm = PLTiles<T>::SMEM;
    const int vm = qms_vel_mask(P, adv, sizeof(T) == 4);
    QMS_WITH_VM(vm, (op_pl_launch<T, VM>(gs, bs, shm, st, mode, g, P, xmap, cmap, y, w, partials, err)));
}
template void qms_launch_op_pl<float>(const QGrid&, const QStepPar<float>&, const CUtensorMap&, const CUtensorMap&,
                                      bool, int, float*, const float*, double*, unsigned*, cudaStream_t);
template void qms_launch_op_pl<double>(const QGrid&, const QStepPar<double>&, const CUtensorMap&, const CUtensorMap&,
                                       bool, int, double*, const double*, double*, unsigned*, cudaStream_t);

void qms_launch_resid_df(const QGrid& g, const QStepPar<qdf>& P, const CUtensorMap& xmap, const CUtensorMap& cmap,
                         bool adv, float* r, const qdf* b, double* partials, unsigned* err, cudaStream_t st,
                         qdf* rfull) {
    op_pl_prepare<float>();
    const dim3 bs(OTX, OTY, 1), gs((g.Nx + OTX - 1) / OTX, (g.Ny + OTY - 1) / OTY, (g.Nz + OKB - 1) / OKB);
    const size_t shm = PLTiles<qdf>::SMEM;
    const int vm = qms_vel_mask(P, adv, true);
    QMS_WITH_VM(vm, (qk_op_pl<qdf, VM, QOPH_RESID, float, qdf><<<gs, bs, shm, st>>>(g, P, xmap, cmap, r, b, partials, err,
                                                                                   rfull)));
}

void qms_launch_delta_split(const QGrid& g, const double* x, const double* x0, qdf* dx, double* partials,
                            long long nb, cudaStream_t st) {
    qk_delta_split<<<(unsigned)nb, 256, 0, st>>>(g, x, x0, dx, partials);
}

void qms_launch_split_ref_pl(const QGrid& g, const double* src, qdf* dst, float* hi, cudaStream_t st) {
    qk_split_ref_pl<<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, src, dst, hi);
}

void qms_launch_split_flat(long long n, const double* src, qdf* dst, cudaStream_t st) {
    qk_split_flat<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 16), 256, 0, st>>>(n, src, dst);
}

void qms_launch_anchor_resid(const QGrid& g, const qdf* r0, const double* x, float* rfloat, qdf* rfull,
                             double* partials, long long nb, cudaStream_t st) {
    qk_anchor_resid<<<(unsigned)nb, 256, 0, st>>>(g, r0, x, rfloat, rfull, partials);
}

void qms_launch_extrapolate(const QGrid& g, double* x, const double* xold, const double* xold2, const double* xold3,
                            int order, cudaStream_t st) {
    qk_extrapolate<<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, x, xold, xold2, xold3, order);
}

// blocks of the least-squares start's first pass that are resident at once on the device
static long long qms_step_start_ls_blocks() {
    static std::atomic<long long> cached{0};
    long long c = cached.load();
    if (c > 0) return c;
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, qk_step_start<true>, 256, 0);
    c = (long long)std::max(1, sms) * std::max(1, per);
    cached.store(c);
    return c;
}

void qms_launch_step_start(const QGrid& g, qdf* rfin, const double* b, const double* bprev, const qdf* dinv, qdf* r0,
                           const QStepStart& h, float* rfloat, double* partials, long long nb, cudaStream_t st,
                           const QStepPtrs* dptrs) {
    QStartRhs R{};
    if (h.hx) {
        R.hx = h.hx;
        R.sg = h.sg;
        R.sdt = h.sdt;
        R.idt[0] = qdf(1.0 / (h.dt * g.dx));
        R.idt[1] = qdf(1.0 / (h.dt * g.dy));
        R.idt[2] = qdf(1.0 / (h.dt * g.dz));
        R.x0 = h.x0;
    }
    if (h.ls > 0) {
        // the first pass: one resident wave of blocks (fewer block sums to form and to add up)
        const long long nb1 = std::min(nb, qms_step_start_ls_blocks());
        qk_step_start<true><<<(unsigned)nb1, 256, 0, st>>>(g, rfin, b, bprev, dinv, r0, h.x, h.xo1, h.xo2, h.xo3, h.ls,
                                                            h.wnew, h.w1, h.w2, nullptr, partials, R, dptrs, h.w3,
                                                            h.lsp);
        qk_ls_solve<<<1, 256, 0, st>>>(h.lsp, nb1, h.ls, h.lsg);
        qk_start_apply<<<(unsigned)nb, 256, 0, st>>>(g, h.x, h.xo1, h.xo2, h.xo3, h.xo4, h.ls, r0, h.wnew, h.w1, h.w2,
                                                     h.w3, h.lsg, rfin, rfloat, partials, dptrs);
        return;
    }
    qk_step_start<false><<<(unsigned)nb, 256, 0, st>>>(g, rfin, b, bprev, dinv, r0, h.x, h.xo1, h.xo2, h.xo3, h.xo,
                                                        h.wnew, h.w1, h.w2, rfloat, partials, R, dptrs, nullptr,
                                                        nullptr);
}

void qms_launch_dinv_df(const QGrid& g, const QCoef<double>& c, const QStepPar<double>& P, qdf* out, cudaStream_t st) {
    qk_dinv_df<<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, c, P, out);
}


void qms_launch_pl_scale(long long n, const float* r, const double* scale, float* out, cudaStream_t st) {
    qk_pl_scale<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 16), 256, 0, st>>>(n, r, scale, out);
}

void qms_launch_diag_pl(const QGrid& g, const QCoef<float>& c, const QStepPar<float>& P, float* dg, cudaStream_t st) {
    cudaMemsetAsync(dg, 0, qms_pl(g).n * sizeof(float), st);
    qk_diag_pl<<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, c, P, dg);
}

template <typename T>
void qms_launch_pl_from_ref(const QGrid& g, const double* r64, const double* scale, T* out, cudaStream_t st) {
    qk_pl_from_ref<T><<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, r64, scale, out);
}
template void qms_launch_pl_from_ref<float>(const QGrid&, const double*, const double*, float*, cudaStream_t);
template void qms_launch_pl_from_ref<double>(const QGrid&, const double*, const double*, double*, cudaStream_t);

template <typename T>
void qms_launch_ref_add_pl(const QGrid& g, const T* e, const double* scale, double* x, cudaStream_t st) {
    qk_ref_add_pl<T><<<qms_node_grid(g), qms_node_block(), 0, st>>>(g, e, scale, x);
}
template void qms_launch_ref_add_pl<float>(const QGrid&, const float*, const double*, double*, cudaStream_t);
template void qms_launch_ref_add_pl<double>(const QGrid&, const double*, const double*, double*, cudaStream_t);
