// qms_solver.h -- the solver object behind a qms_handle.
#pragma once
#include "qms.h"
#include "qms_internal.h"
#include "qms_mg.h"
#include "qms_tma.cuh"
#include "qms_df.cuh"
#include "qms_pl.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>

#define QMS_NVEC 9   // r, rh, p, v, s, t, e, y, z  (+ MG level-0 temporary)

size_t qms_device_bytes_impl(const qms_desc& d);

// transient steps chained to an anchor before an exact FP64 one is taken again
#define QMS_CHAIN_MAX 32

struct QmsSolver {
    qms_desc desc{};
    QGrid g{};
    int dev = -1;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    bool fp64_inner = false;
    bool trace = false;         // QMS_TRACE set: one stderr line per refinement iteration
    size_t tsize = 4;
    long long vec_blocks = 0, nbop = 0;

    uint8_t* ids = nullptr;
    QMatTable<double> htab64{};
    QMatTable<float> htab32{};
    QMatTable<double>* dtab64 = nullptr;
    QMatTable<float>* dtab32 = nullptr;
    double* x = nullptr;        // current solution [Ax|Ay|Az|V]
    double* b = nullptr;        // RHS of the last solve
    double* r64 = nullptr;      // scaled FP64 residual
    double* xbest = nullptr;    // best iterate of the current solve
    double* H = nullptr;        // Hx|Hy|Hz cubes
    double* slicebuf = nullptr;
    double* part = nullptr;     // block partial sums
    double* S = nullptr;        // device scalars
    double* hS = nullptr;       // pinned host mirror
    unsigned* status = nullptr;
    float* nc32 = nullptr;      // node coefficients (6 x Nn), FP32 and FP64
    double* nc64 = nullptr;
    float* dg_steady = nullptr; // Jacobi diagonals
    float* dg_tr = nullptr;
    void* vec[QMS_NVEC] = {};   // inner Krylov vectors (FP32 or FP64)
    float* mgtmp = nullptr;     // level-0 Jacobi temporary of the multigrid
    float* mgtmp2 = nullptr;    // V right-hand side of the block-triangular preconditioner
    // Mixed precision: the first residual of a solve (the anchor) is exact FP64; the later ones
    // are r = r0 - D^-1 M (x - x0) in double-float on the FP32 pipe, from the anchor's residual r0
    // and the change of x since the anchor state x0 (node coefficients split into float pairs,
    // padded layout).  Every residual also lands in rpl (FP32, padded) for the inner solver.
    bool df_resid = false;
    bool anchor_ready = false;
    double* x0 = nullptr;
    // Chained anchor: a transient solve with the operator of the previous one starts from that
    // solve's final residual, r0 = r_fin + D^-1 (b - b_prev), instead of an FP64 residual (an
    // exact one after QMS_CHAIN_MAX chained steps, and whenever the operator or the state changed
    // otherwise).  Each chained step adds the double-float rounding of one residual (~1e-16 of
    // |x|) to the anchor; the drift test runs a full chain against the FP64 residual.
    double* bprev = nullptr;    // right-hand side of the previous solve
    qdf* rfin = nullptr;        // the last double-float residual, in full
    qdf* dinvdf = nullptr;      // 1 / diag M of the transient operator
    bool rfin_ok = false;       // rfin is the final residual of the state in x, for chain_v
    bool last_resid_df = false;
    int chain_len = 0;
    double chain_v[3] = {0, 0, 0};
    double chain_B[3] = {0, 0, 0}, chain_G[9] = {};
    bool anchor_is_residual = false;  // x is still the anchor state (same Dirichlet values)
    double* hist_x = nullptr;   // the last converged transient solution
    double* xold = nullptr;     // the one before it
    double* xold2 = nullptr;    // ... and the one before that (quadratic extrapolation)
    double* xold3 = nullptr;    // ... and the one before that (cubic)
    double* xold4 = nullptr;    // ... and the one before that (least-squares start over 4 differences)
    int hist_len = 0;           // consecutive converged transient solves with the same operator (<= 5)
    // Residual of the extrapolated start by linearity (qk_step_start): w_n = D^-1 M (x_n - x_{n-1})
    // is the difference of a chained solve's anchor and final residual; wh[0] holds the last
    // step's, wh[1] the one before (cubic), ..., w_len of them valid; one more buffer takes the next
    qdf* wh[4] = {nullptr, nullptr, nullptr, nullptr};
    int w_len = 0;
    int nwh = 0;                // w buffers allocated
    double* lsp = nullptr;      // least-squares start: QMS_LS_SUMS x nbop partial sums
    double* lsg = nullptr;      // ... and its coefficients and diagnostics (8 doubles)
    bool last_chained = false;  // the last solve's anchor state was the solution before it
    int field_run = 0;          // consecutive solves (this one included) with the same B, G
    bool start_resid_ready = false;   // the step start formed the first residual
    // b holds the last solve's right-hand side (false: that solve took b - b_prev from x_n -
    // x_(n-1); ensure_b forms it from x0, that solve's start state, and last_ex / last_tr)
    bool b_fresh = false;
    QmsExcite last_ex{};
    bool last_tr = false;
    void ensure_b();
    double* rsg = nullptr;      // edge sigma of every A row, and / dt (transient right-hand side)
    double* rsdt = nullptr;
    qdf* xdf = nullptr;         // x - x0
    qdf* r0df = nullptr;
    qdf* ncdf = nullptr;
    float* rpl = nullptr;
    CUtensorMap xdfmap{}, cdfmap{};
    template <typename T> void resid_to_inner(T* out);   // out = r / |r| in the inner precision
    QmsMG<float> mgf[2];        // hierarchies of the steady [0] and transient [1] operators (mixed)
    QmsMG<double> mgd[2];       // the same in FP64 (plain FP64 solver)
    bool use_mg = false;
    QmsRegions regions;         // conductor-region coarse space of the V block (with MG)
    // z = preconditioner(r): multigrid on (bscale .* r) or the Jacobi / identity fallback
    // With P (transient rows of the unmasked system, desc.mg_coupling = 1) the multigrid is
    // lower block-triangular in (A, V): z_A = MG_A(r_A), z_V = MG_V(r_V - D_V^-1 M_VA z_A).
    template <typename T> void precond(const T* r, const float* bscale, T* z, bool mask_v, bool transient,
                                       bool jacobi_pcg, const QStepPar<T>* P = nullptr, bool adv = false);

    qms_stats stats{};
    std::string err;

    // instrumentation (qms_profile_enable)
    bool prof = false;
    long long nlaunch = 0;
    // kind: 0 op32, 1 op64, 2 V-cycle, 3 FP64 residual, 4 level-0 A-block Jacobi sweep
    struct OpEv { cudaEvent_t a, b; int kind; double bytes; };
    OpEv* prof_begin(int kind, double bytes);
    void prof_end(OpEv* ev);
    bool prof_accum(const OpEv& e);              // false when the events cannot be timed
    // a deque: prof_begin hands out pointers into it that stay valid while later events are
    // added (profile events nest: the A-block sweeps inside a V-cycle's own event)
    std::deque<OpEv> evpool;
    size_t evused = 0;
    bool capturing = false;                      // event records go into a graph being captured
    bool graph_prof_broken = false;
    qms_profile profacc{};
    // the multigrid's timing hook (the A-block sweeps), forwarding to prof_begin / prof_end
    struct MgHook : MgProf {
        QmsSolver* s = nullptr;
        void* begin(int kind, double bytes) override { return s->prof_begin(kind, bytes); }
        void end(void* token) override { s->prof_end((OpEv*)token); }
    } mghook;
    int profile_enable(bool on);
    int profile_collect(qms_profile* out);
    template <typename T>
    void op(bool adv, int mode, const QStepPar<T>& P, const T* x, const T* b, T* y, const T* w, double* partials);
    // the inner solver's operator on padded vectors (TMA-staged)
    template <typename T>
    void op_pl(bool adv, int mode, const QStepPar<T>& P, const T* x, T* y, const T* w, double* partials);
    long long npl = 0;                              // padded inner-vector length
    std::unordered_map<const void*, CUtensorMap> tmaps;   // tensor maps of the padded vectors
    CUtensorMap cmap32{}, cmap64{};                 // ... and of the node coefficients
    std::unordered_map<const void*, CUtensorMap> tmapsA, tmapsV;   // ... of their A blocks / V block
    CUtensorMap cmapV32{}, cmapV64{};               // ... of the three conductivities
    // bf16 copy of the FP32 node coefficients (the multigrid's level-0 tiles) and its maps
    __nv_bfloat16* nc16 = nullptr;
    CUtensorMap cmap16{}, cmapV16{};
    const CUtensorMap& tmap(const void* p) const;
    const CUtensorMap& tmapq(const void* p, int qs) const;

    ~QmsSolver();
    void release();
    int init(const qms_desc& d);
    int set_materials(const uint8_t* host_slots, const double* rows6, int nmat);
    int solve(bool transient, const double v[3], const double B[3], const double G[9]);
    // exact: the FP64 residual even where the double-float one would do (the public entry point)
    int residual(bool adv, bool transient, const double v[3], bool exact = false);
    int fields(int which, int axis, int index, double* host_out);
    // Asynchronous field output: H (cubes or slice) formed on the solver stream into the device
    // buffer of `slot`, copied to host_out on a copy stream that overlaps the solver's next work;
    // fields_sync(slot) waits for that copy (callable from another host thread).
    static constexpr int kFieldSlots = 4;
    cudaStream_t cst = nullptr;
    cudaEvent_t fev_ready[kFieldSlots] = {}, fev_done[kFieldSlots] = {};
    double* fbuf[kFieldSlots] = {};
    size_t fbuf_n[kFieldSlots] = {};
    int fields_async(int which, int axis, int index, double* host_out, int slot);
    int fields_sync(int slot);
    int finalize(int op, int nsum, long long nb);
    int read_scalars();

    QCoef<float> coef32() const;
    QCoef<double> coef64() const;
    template <typename T> QCoef<T> coef() const;

    template <typename T> int inner_bicgstab(bool adv, bool transient, const double v[3], int& iters);
    template <typename T> int inner_pcg(bool transient, int& iters);
    template <typename T> int inner_gmres(bool adv, bool transient, const double v[3], int& iters, int fixed_k);
    int residual_launch(bool adv, bool transient, const double v[3], bool exact = false);
    int ir_iteration_graph(bool adv, bool transient, const double v[3], int k);
    // captured refinement iterations, one per FGMRES count k (and step parameters); the
    // profile event records of a capture belong to its entry
    struct IrGraph {
        cudaGraphExec_t exec = nullptr;
        int k = 0;
        bool tr = false, adv = false, prof = false;
        bool resid_df = false;      // the captured residual is the double-float one (rfin)
        double v[3] = {0, 0, 0};
        long long launches = 0;
        std::deque<OpEv> ev;
        size_t evn = 0;
        unsigned long long used = 0;
    };
    std::vector<IrGraph> graphs;
    // Whole chained transient steps as one CUDA graph each: the status reset, the step start (its
    // rotating history pointers copied from pinned host memory by a node of the graph), the start
    // residual, and a conditional WHILE node whose body is one refinement cycle (FGMRES with k
    // steps, the FP64 update, the double-float residual) ended by a kernel that sets the
    // condition from the residual (at most kStepGraphCycles cycles; the host loop continues a
    // solve that needs more).  One host synchronisation per step.
    static constexpr int kStepGraphCycles = 3;
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        int k = 0, xo = 0, ls = 0;
        bool wcalc = false, dbx = false;
        double v[3] = {0, 0, 0};
        long long pro = 0, body = 0;     // kernel launches of the prologue and of one cycle
        unsigned long long used = 0;
    };
    std::vector<StepGraph> sgraphs;
    QStepPtrs* hptrs = nullptr;          // pinned host copy of the step start's rotating pointers
    QStepPtrs* dptrs = nullptr;          // ... and the device copy the graph's step start reads
    int step_graph(bool adv, const double v[3], const QStepStart& hs, bool wcalc, int k, int& cycles);
    unsigned long long graph_clock = 0;
    void drop_graphs();
    bool graph_resid_ready = false;
    int gm_k_est = 0;           // FGMRES iterations replayed per refinement iteration (0: not yet known)
    int gm_k_seen = 0;          // largest count seen while running with host checks
    int gm_ls_floor = 0;        // lowest count for solves after a least-squares start, and its age
    int gm_ls_floor_age = 0;
    bool gm_k_fine = false;     // gm_k_est has overshot downwards once: tune it in single steps
    int gm_k_floor = 0;         // smallest count not yet known to need a third replay
    int gm_k_floor_age = 0;     // solves since gm_k_floor was set or lowered
    // log of the per-iteration residual reduction of FGMRES, smoothed over solves: [0] the first
    // cycle of a solve, [1] the later ones (which start from a residual rich in slow modes)
    double gm_lrate[2] = {0, 0};
    void* gmV[65] = {};         // FGMRES basis (m + 1) and preconditioned directions (m), m <= 64
    void* gmZ[64] = {};
    double* gm_H = nullptr;     // Hessenberg matrix (m+1) x m, row-major with stride m
    double* gm_scal = nullptr;  // beta, |g_{j+1}|, 1/h, rotations, g, y
    int last_gm_k = 0;
    int last_inner = 0;         // 0 PCG, 1 BiCGSTAB, 2 FGMRES
};

template <> inline QCoef<float> QmsSolver::coef<float>() const { return coef32(); }
template <> inline QCoef<double> QmsSolver::coef<double>() const { return coef64(); }
