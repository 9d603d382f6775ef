// qms_pl.h -- launchers of the padded-layout kernels (qms_pl.cu).
#pragma once
#include "qms_internal.h"
#include "qms_tma.cuh"
#include "qms_df.cuh"

#include <cuda_bf16.h>

// one thread per node: blocks of QMS_NODE_BX (along x) x QMS_NODE_BY (along y) nodes of a plane
#define QMS_NODE_BX 32
#define QMS_NODE_BY 16
dim3 qms_node_grid(const QGrid& g);
dim3 qms_node_block();
long long qms_op_pl_num_blocks(const QGrid& g);

// y = M x (mode QOPH_APPLY) or D^-1 M x (QOPH_SCALED) on padded vectors; x and the node
// coefficients come through their tensor maps (qms_make_pl_map, 10 and 9 rows per box).
// QOPH_VCOUPLE takes the maps of x's three A blocks and of the three conductivities.
template <typename T>
void qms_launch_op_pl(const QGrid& g, const QStepPar<T>& P, const CUtensorMap& xmap, const CUtensorMap& cmap, bool adv,
                      int mode, T* y, const T* w, double* partials, unsigned* err, cudaStream_t st);

// refinement residual in double-float from an anchor: r = (float) (r0 - D^-1 M dx) on padded
// vectors, with r0 the anchor's scaled residual and dx (xmap) the change of x since the anchor,
// both double-float, and the node coefficients (cmap) as double-float; partials |r_A|^2, |r_V|^2
// rfull (optional): the residual itself, double-float
void qms_launch_resid_df(const QGrid& g, const QStepPar<qdf>& P, const CUtensorMap& xmap, const CUtensorMap& cmap,
                         bool adv, float* r, const qdf* r0, double* partials, unsigned* err, cudaStream_t st,
                         qdf* rfull = nullptr);
// the residual when x is the anchor state: rfloat = (float) r0, rfull = r0, the four partials of nb blocks
void qms_launch_anchor_resid(const QGrid& g, const qdf* r0, const double* x, float* rfloat, qdf* rfull,
                             double* partials, long long nb, cudaStream_t st);
// x = the extrapolation of order 1..3 from x, xold, xold2, xold3 on the non-Dirichlet rows
// (reference order)
void qms_launch_extrapolate(const QGrid& g, double* x, const double* xold, const double* xold2, const double* xold3,
                            int order, cudaStream_t st);
// the state history that the chained step start reads (qk_step_start)
struct QStepStart {
    double* x;                      // x_n, extrapolated in place when xo > 0
    const double* xo1;              // x_{n-1}, x_{n-2}, x_{n-3}
    const double* xo2;
    const double* xo3;
    int xo;                         // extrapolation order (0: x unchanged)
    qdf* wnew;                      // where w = D^-1 M (x_n - x_{n-1}) goes (null: not formed)
    const qdf* w1;                  // the stored w of the step before, and the one before that
    const qdf* w2;                  // (no two of x, xo*, wnew, w1, w2 alias)
    // b - b_prev from x_n - x_{n-1} instead of two right-hand sides (hx: a copy of x_n; null:
    // from b and bprev): the transient right-hand side's edge sigma and sigma / dt, dt, and x0,
    // which receives x_n
    const double* hx;
    const double* sg;
    const double* sdt;
    double dt;
    double* x0;
    // Least-squares start (ls > 0 directions, at most 4; xo = ls): x = x_n + sum_j g_j d_j with
    // the coefficients g that minimise the scaled residual over the span of the last ls state
    // differences d_j = x_{n-j+1} - x_{n-j}, whose residual images are w, w1, w2, w3; x_{n-4} in
    // xo4.  lsp: 15 x nb partial sums, lsg: 8 doubles (the coefficients, then diagnostics).
    const double* xo4;
    const qdf* w3;
    int ls;
    double* lsp;
    double* lsg;
};
// the history pointers that rotate from step to step, for a step start that reads them from
// device memory (dptrs) instead of its arguments (with hx: the pointers are those of h)
struct QStepPtrs {
    const double* xo1;
    const double* xo2;
    const double* xo3;
    qdf* wnew;
    const qdf* w1;
    const qdf* w2;
    const double* hx;
    const double* b;
    const double* bprev;
    const double* xo4;
    const qdf* w3;
};
// partial sums per block of the least-squares start (Gram matrix of 4 directions, their products
// with the base residual, and the base residual's square)
#define QMS_LS_SUMS 15
// nb: the blocks of the launch and the partials per quantity
void qms_launch_step_start(const QGrid& g, qdf* rfin, const double* b, const double* bprev, const qdf* dinv, qdf* r0,
                           const QStepStart& h, float* rfloat, double* partials, long long nb, cudaStream_t st,
                           const QStepPtrs* dptrs = nullptr);
// 1 / diag M as double-float (padded layout)
void qms_launch_dinv_df(const QGrid& g, const QCoef<double>& c, const QStepPar<double>& P, qdf* out, cudaStream_t st);
// dx = x - x0 as double-float (padded layout) and the partials |x_A|^2, |x_V|^2 of nb blocks
void qms_launch_delta_split(const QGrid& g, const double* x, const double* x0, qdf* dx, double* partials,
                            long long nb, cudaStream_t st);
// ref -> padded double-float (and its high words to hi when given)
void qms_launch_split_ref_pl(const QGrid& g, const double* src, qdf* dst, float* hi, cudaStream_t st);
void qms_launch_split_flat(long long n, const double* src, qdf* dst, cudaStream_t st);
void qms_launch_pl_scale(long long n, const float* r, const double* scale, float* out, cudaStream_t st);

// one CTA waiting (at most `spins` polls) on an mbarrier that never completes: sets QMS_ST_TIMEOUT
void qms_launch_wait_selftest(int spins, unsigned* err, cudaStream_t st);

// the bf16 copy (qms_pl16_pitch rows) of the FP32 node coefficients, for the multigrid's level 0
void qms_launch_coef_bf16(const QGrid& g, const float* nc, __nv_bfloat16* out, cudaStream_t st);

void qms_launch_diag_pl(const QGrid& g, const QCoef<float>& c, const QStepPar<float>& P, float* dg, cudaStream_t st);

// out[PL] = r64[ref] * scale[0] (scale may be null: 1)
template <typename T>
void qms_launch_pl_from_ref(const QGrid& g, const double* r64, const double* scale, T* out, cudaStream_t st);
// x[ref] += scale[0] * e[PL]
template <typename T>
void qms_launch_ref_add_pl(const QGrid& g, const T* e, const double* scale, double* x, cudaStream_t st);
