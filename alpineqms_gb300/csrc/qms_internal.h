// qms_internal.h -- launchers shared between the translation units of libqms_gb300.
#pragma once
#include "qms_common.cuh"

struct QmsExcite { double B[3]; double G[9]; double v[3]; };

// QOPH_VCOUPLE (padded-layout stencil only): y_V = w_V - D_V^-1 (M_VA x_A) on the V rows, the
// A-to-V coupling of the operator applied to x's A blocks (x's V block is not read)
enum QOpModeH { QOPH_APPLY = 0, QOPH_SCALED = 1, QOPH_RESID = 2, QOPH_VCOUPLE = 3 };

// qms_exact.cu
long long qms_launch_assemble(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const QmsExcite& ex,
                              double dt, int tr, const double* xp, long long* ia, int32_t* ja, double* a, double* b,
                              cudaStream_t st);
void qms_launch_rhs(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const QmsExcite& ex, double dt,
                    int tr, const double* xp, double* b, double* x_dirichlet, cudaStream_t st,
                    const double* sg = nullptr, const double* sdt = nullptr);
// edge sigma of every A row and sigma / dt (for qms_launch_rhs)
void qms_launch_rhs_coef(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, double dt, double* sg,
                         double* sdt, cudaStream_t st);
void qms_launch_hfield(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const double* x, double* Hx,
                       double* Hy, double* Hz, cudaStream_t st);
// H on the cells of one slice straight from x (qk_slice's layout)
void qms_launch_hslice(const QGrid& g, const uint8_t* ids, const QMatTable<double>* tab, const double* x, int axis,
                       int index, double* out, cudaStream_t st);
void qms_launch_slice(const QGrid& g, int axis, int index, const double* Hx, const double* Hy, const double* Hz,
                      double* out, cudaStream_t st);
void qms_launch_ids(long long ncell, const double* geom, const uint8_t* lut, int maxid, uint8_t* ids, unsigned* status,
                    cudaStream_t st);
long long qms_csr_nnz(const QGrid& g);

// qms_operator.cu
long long qms_op_num_blocks(const QGrid& g);
template <typename T>
void qms_launch_operator(const QGrid& g, const QCoef<T>& c, const QStepPar<T>& P, bool adv, int mode, const T* x,
                         const T* b, T* y, const T* w, double* partials, cudaStream_t st);
void qms_launch_diag(const QGrid& g, const QCoef<float>& c, const QStepPar<float>& P, float* dg, cudaStream_t st);
template <typename T>
void qms_launch_node_coef(const QGrid& g, const QCoef<T>& c, T* nc, cudaStream_t st);
void qms_launch_csr_spmv(long long n, const long long* ia, const int32_t* ja, const double* a, const double* x,
                         double* y, cudaStream_t st);

// host-side material table (slot 0 = vacuum); rows: mu_r xyz, sigma xyz
template <typename T>
void qms_fill_table(QMatTable<T>& t, const double* rows6, int nmat);
