/*
 * qms.h -- C-ABI of libqms_gb300.so, the GB300 implementation of the
 * AlpineQMS QMS_3D per-step hot path (Yee-grid A-V assembly and solve).
 *
 * The reference has no library boundary: 3D/master.py:84 runs the Fortran
 * executable (`./QMS_3D inputs.txt`) and the program calls MKL PARDISO on a
 * CSR matrix it assembles itself.  The entry points below replace, one for
 * one, the pieces of that program (3D/QMS_3D.f90, cited as F:line):
 *
 *   qms_create / qms_destroy        allocation of fields, CSR and PARDISO
 *                                   handles (F:286-357, F:398-405) and the
 *                                   final release (F:2315-2318)
 *   qms_set_materials               material table -> Yee coefficients
 *                                   (F:193-279); geometry as uint8 slots
 *   qms_set_geometry_f64            geom.bin float64 IDs + table lookup
 *                                   (F:229-254), converted on the GPU
 *   qms_steady                      steady-state assembly + phase-13 solve
 *                                   (F:430-1317)
 *   qms_step                        one backward-Euler step: assembly +
 *                                   phase-23/33 solve (F:1451-2208)
 *   qms_get_fields                  unpack + H at cell centres + slice
 *                                   (F:1319-1394, F:2210-2290)
 *   qms_get_state / qms_set_state   the x_vec solution [Ax|Ay|Az|V] (F:1316)
 *   qms_assemble_csr                the CSR matrix and RHS handed to PARDISO
 *                                   (F:448-1312 steady, F:1457-2191
 *                                   transient), bit-exact; verification path
 *   qms_apply                       y = M x with the matrix-free operator
 *   qms_residual_norm               ||D^-1 (b - M x)|| of the current state
 *
 * Conventions: every function returns 0 on success and a negative QMS_ERR_*
 * code otherwise (no exceptions cross the ABI); qms_last_error() gives the
 * message.  Host pointers are borrowed for the duration of the call.  Device
 * pointers (d_*) must be allocations on the handle's device.  A handle is
 * used by one host thread at a time.  Velocities are the frame velocity
 * solve_v{x,y,z} of the step (F:431-433, F:1447-1449); B and G are the
 * background field and its 3x3 gradient (row-major gxx gxy gxz gyx ... gzz)
 * in effect for that solve.
 */
#ifndef QMS_GB300_H
#define QMS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QMS_ABI_VERSION 1

enum {
    QMS_OK = 0,
    QMS_ERR_ARG = -1,        /* invalid argument / size */
    QMS_ERR_CUDA = -2,       /* CUDA runtime error */
    QMS_ERR_NOMEM = -3,      /* device allocation failed */
    QMS_ERR_STATE = -4,      /* call out of order */
    QMS_ERR_CONVERGE = -5    /* solver did not reach the tolerance (state kept) */
};

enum { QMS_PREC_MIXED = 0, QMS_PREC_FP64 = 1 };
enum { QMS_FIELD_CUBES = 0, QMS_FIELD_SLICE = 1 };
enum { QMS_PRECOND_JACOBI = 0, QMS_PRECOND_MG = 1 };
enum { QMS_KRYLOV_GMRES = 0, QMS_KRYLOV_BICGSTAB = 1 };

/* status bits reported in qms_stats.status */
enum {
    QMS_STATUS_BAD_MATERIAL = 1,
    QMS_STATUS_NAN = 2,
    QMS_STATUS_NO_CONVERGENCE = 4,
    QMS_STATUS_BREAKDOWN = 8,
    QMS_STATUS_TIMEOUT = 16      /* a bounded device-side wait for a tile copy gave up */
};

typedef struct {
    int xs, ys, zs;          /* cells per axis (F:123) */
    double dx, dy, dz;       /* cell size, m (F:124) */
    double dt;               /* time step, s (F:125) */
    int precision;           /* QMS_PREC_MIXED: FP32 inner Krylov in FP64 refinement;
                                QMS_PREC_FP64: the same solver entirely in FP64 */
    double tol;              /* stop when ||D^-1 (b - M x)|| <= tol * ||x|| */
    int max_outer;           /* refinement iterations */
    int max_inner;           /* Krylov iterations per refinement iteration */
    double inner_rtol;       /* relative reduction asked of each inner solve */
    int check_every;         /* inner iterations between host convergence checks */
    int device;              /* CUDA device ordinal */
    int precond;             /* QMS_PRECOND_MG (default) or QMS_PRECOND_JACOBI */
    int mg_sweeps;           /* Jacobi sweeps before and after each coarse correction */
    double mg_omega;         /* Jacobi weight */
    double mg_vshift;        /* relative diagonal shift of the preconditioner's V block (0 by default:
                                the coarsest V solve is a pseudo-inverse that drops the floating
                                potential of isolated conductors) */
    int krylov;              /* nonsymmetric inner solver: QMS_KRYLOV_GMRES (default) or _BICGSTAB */
    int gmres_m;             /* FGMRES basis size per refinement iteration (<= 64) */
    int use_graphs;          /* replay each refinement iteration of a step as one CUDA graph, with the
                                FGMRES iteration count learned from the first solve (1 = on) */
    double mg_region_cut;    /* conductor-region coarse space of the potential block: eigenvalues of
                                its region-stiffness-scaled Galerkin matrix at or below this are
                                dropped (0 = automatic: 1e-9 with FP64 inner vectors, 1e-6 with FP32;
                                negative = no region space) */
    double mg_alpha;         /* scale of every coarse-grid correction of the V-cycle (over-correction
                                of the piecewise-constant aggregation prolongation; <= 0 means 1) */
    int mg_coupling;         /* transient steps: 1 (default) lower block-triangular preconditioner in
                                (A, V) -- a cycle on the A blocks, then one on the V block for the
                                residual the A correction leaves in the V rows; 0 block-diagonal */
    int mg_coarse_sweeps;    /* Jacobi sweeps before and after the coarse correction on levels >= 1
                                (0: mg_sweeps) */
    int mg_v_sweeps;         /* sweeps on each side, on every level, of the block-triangular
                                preconditioner's V-block cycle (0: as the A blocks) */
    int mg_tail_points;      /* the coarse levels with at most this many points per block run their
                                sub-cycle as one launch, one CTA per block (0: 4096; < 0: off) */
    int extrapolate;         /* a transient step that follows steps with the same operator starts
                                from an extrapolation of the last solutions instead of x_n, of
                                this order at most (lower while fewer solutions are known):
                                3 (default) cubic, 4 x_n - 6 x_(n-1) + 4 x_(n-2) - x_(n-3);
                                2 quadratic, 3 x_n - 3 x_(n-1) + x_(n-2); 1 linear,
                                2 x_n - x_(n-1); 0 none */
    double mg_v_coarse_cut;  /* near-null modes of the potential block's multigrid: a coarse point whose
                                Galerkin diagonal is at or below this times the summed level-0
                                diagonals it aggregates leaves the hierarchy, and the coarsest solve
                                drops eigenvalues of its operator scaled by those sums at or below
                                it (0 = automatic: 1e-9 with FP64 inner vectors, 1e-5 with FP32) */
    int gm_first_extend;     /* replayed refinement iterations: the first FGMRES cycle of a solve may run
                                up to this many steps beyond the learned count when the start residual
                                and the observed first-cycle rate say that one cycle then reaches the
                                tolerance (instead of two cycles); 0 = never (the default: on the
                                moving plate it kept longer single cycles, 30.6 vs 28.0 ms per step) */
    double tol_v;            /* > 0: a solve also stops only when ||r_V|| <= tol_v * ||x_V|| (the potential block's
                                scaled residual against its own size); 0 = off (the default) */
    int start_ls;            /* chained transient steps (mixed precision): the start is x_n plus the combination
                                of the last start_ls (<= 4) state differences that minimises the
                                scaled residual (found on the device from the stored residual
                                images of those differences, one extra pass); 0 = the polynomial
                                extrapolation alone.  Default 4 */
} qms_desc;

typedef struct {
    int outer_iterations;
    int inner_iterations;
    double initial_residual; /* relative scaled residual before the solve */
    double final_residual;   /* after */
    unsigned status;         /* QMS_STATUS_* bits */
    int step_graph;          /* 1 when the step ran as one CUDA graph (start, residual and its refinement
                                cycles behind a device-side convergence test), 0 otherwise */
    int start_ls;            /* directions of the least-squares start of this step (0: none) */
    double start_coef[4];    /* its start x_n + sum_j start_coef[j] (x_(n-j) - x_(n-j-1)), j = 0..3 */
    double start_base;       /* |r|^2 of the polynomial start it improved on, and the |r|^2 the */
    double start_pred;       /* least-squares solve predicted (unscaled sums of squares) */
} qms_stats;

typedef struct qms_handle qms_handle;

/* Fills `d` with the defaults for a grid (mixed precision, tol 2e-13). */
void qms_default_desc(qms_desc* d, int xs, int ys, int zs, double dx, double dy, double dz, double dt);
/* Device bytes a handle with this descriptor allocates (admission control). */
size_t qms_device_bytes(const qms_desc* d);
int64_t qms_n_dims(int xs, int ys, int zs);
int64_t qms_csr_nnz(int xs, int ys, int zs);

int qms_create(const qms_desc* d, qms_handle** out);
void qms_destroy(qms_handle* h);
const char* qms_last_error(const qms_handle* h);   /* h may be NULL: last create error */

/* slots: xs*ys*zs uint8 in Fortran order, 0 = vacuum, r = row r of `rows`;
 * rows: nmat x 6 doubles (mu_r x,y,z, sigma x,y,z), nmat <= 255 */
int qms_set_materials(qms_handle* h, const uint8_t* slots, const double* rows, int nmat);
/* geom: xs*ys*zs float64 material IDs (geom.bin); table: nmat x 7 doubles
 * (ID, mu_r x,y,z, sigma x,y,z) as read from inputs.txt (F:157-161).  IDs absent
 * from the table are vacuum; IDs above the table maximum or negative are
 * rejected (QMS_ERR_ARG). */
int qms_set_geometry_f64(qms_handle* h, const double* geom, const double* table, int nmat);

int qms_steady(qms_handle* h, const double v[3], const double B[3], const double G[9]);
int qms_step(qms_handle* h, const double v[3], const double B[3], const double G[9]);
int qms_get_stats(const qms_handle* h, qms_stats* out);
/* Failure-detection self-test (no counterpart in the reference, whose PARDISO error code is
 * never checked, F:2196-2202): one CTA on the handle's stream waits on a shared-memory
 * mbarrier that nothing completes, with the bounded wait every TMA-staged kernel uses for its
 * tile copies (here at most `spins` polls, 1..2^20).  The wait gives up, the kernel returns
 * and sets QMS_STATUS_TIMEOUT, which is reported in *status_out (may be NULL) and in
 * qms_get_stats; the handle stays usable for the next call. */
int qms_wait_selftest(qms_handle* h, int spins, unsigned* status_out);

/* which = QMS_FIELD_CUBES: out = Hx|Hy|Hz cubes (3*xs*ys*zs doubles, F-order);
 * which = QMS_FIELD_SLICE: out = the three slices (axis 0/1/2 = x/y/z, 1-based
 * index), each in the record layout of F:1380-1394. */
int qms_get_fields(qms_handle* h, int which, int axis, int index, double* out);
/* The same fields without waiting (the per-step dumps of F:2274-2300, overlapped with the next
 * step): H is formed on the handle's stream into the device buffer of `slot` (0..3) and copied
 * to `out` on a separate copy stream, so the handle's next calls (qms_step ...) run while the
 * copy is in flight.  `out` should be pinned host memory (qms_pinned_alloc) for the copy to be
 * asynchronous, and must stay untouched until qms_fields_sync(h, slot) has returned.  A slot's
 * next use waits for its previous copy. */
int qms_get_fields_async(qms_handle* h, int which, int axis, int index, double* out, int slot);
/* Waits until the copy issued on `slot` has landed.  Unlike the other calls on a handle, it may
 * be made from another host thread while the owning thread keeps stepping. */
int qms_fields_sync(qms_handle* h, int slot);
/* Page-locked host memory for qms_get_fields_async (NULL on failure) and its release. */
void* qms_pinned_alloc(size_t bytes);
void qms_pinned_free(void* p);
int qms_get_state(qms_handle* h, double* x_out);          /* n_dims doubles */
int qms_get_rhs(qms_handle* h, double* b_out);            /* n_dims doubles: the right-hand side of the last
                                                             solve (RHS of F:1457-2191, Dirichlet values
                                                             in their rows), bit-exact; a chained transient
                                                             step with an unchanged field does not form it,
                                                             and this call then forms it from that step's
                                                             start state */
int qms_set_state(qms_handle* h, const double* x_in);

/* Verification path: CSR of the steady (transient = 0) or transient system and
 * its RHS, bit-identical to the reference's (F:448-1312 / F:1457-2191).
 * d_ia: n_dims+1 int64 (1-based), d_ja: nnz int32 (1-based), d_a: nnz doubles,
 * d_b: n_dims doubles, d_xprev: previous solution (transient only).  The int64
 * row pointer replaces the reference's int32 one (which overflows above
 * ~2^31 non-zeros). */
int qms_assemble_csr(qms_handle* h, int transient, const double v[3], const double B[3], const double G[9],
                     const double* d_xprev, int64_t* d_ia, int32_t* d_ja, double* d_a, double* d_b);
/* y = M x with the matrix-free operator in FP64 (fp32 = 0) or FP32 (fp32 = 1);
 * d_x, d_y: n_dims elements of that type. */
int qms_apply(qms_handle* h, int transient, const double v[3], int fp32, const void* d_x, void* d_y);
/* CSR SpMV on the verification-path arrays (FP64). */
int qms_csr_spmv(qms_handle* h, const int64_t* d_ia, const int32_t* d_ja, const double* d_a, const double* d_x,
                 double* d_y);
/* ||D^-1 (b - M x)||_2 / ||x||_2 for the current state and the RHS of the last solve. */
int qms_residual_norm(qms_handle* h, int transient, const double v[3], double* rel_out);

/* Instrumentation for benchmarks: when enabled, every operator launch is
 * bracketed by CUDA events on the handle's stream, and every kernel launch of
 * the handle is counted.  Enabling resets the counters. */
typedef struct {
    int64_t launches;        /* all kernel launches since the reset */
    int64_t op32_launches;   /* FP32 inner operator applications */
    double op32_ms;          /* their summed device time */
    double op32_bytes;       /* their summed algorithmic bytes (x, y, dot vector, material slots) */
    int64_t op64_launches;   /* FP64 inner operator applications (QMS_PREC_FP64) */
    double op64_ms;
    double op64_bytes;
    int64_t mg_cycles;       /* multigrid V-cycles */
    double mg_ms;            /* their summed device time */
    int64_t resid_launches;  /* FP64 refinement residuals r = D^-1 (b - M x) */
    double resid_ms;
    double resid_bytes;
    int64_t mg0a_launches;   /* level-0 Jacobi sweeps on the three A blocks (the largest kernel of a step) */
    double mg0a_ms;
    double mg0a_bytes;       /* their algorithmic bytes: x and b read, x written (3 p n_A), one byte per cell */
} qms_profile;
int qms_profile_enable(qms_handle* h, int on);
int qms_get_profile(qms_handle* h, qms_profile* out);
/* The cudaStream_t all work of the handle runs on (to record events around calls). */
void* qms_get_stream(qms_handle* h);

/* Residual check for callers that cannot allocate device memory.  This entry
 * point has no counterpart in the reference (whose solve is a direct PARDISO
 * call with no residual output).  It is meant for code that may not call
 * cudaMalloc -- for example an allocator-free real-time loop, or a process
 * whose device memory is owned by another runtime's pool -- and therefore
 * cannot create a qms_handle.  It computes, on `stream`,
 *   d_r    = D^-1 (b - M x)                      (n_dims doubles, D = diag M)
 *   d_sums = |r_A|^2, |r_V|^2, |x_A|^2, |x_V|^2  (4 doubles)
 * for the steady (transient = 0) or transient operator with frame velocity v,
 * from caller-owned device buffers: d_slots (xs*ys*zs uint8 material slots,
 * Fortran order), d_x and d_b (n_dims doubles).  rows: host array of nmat x 6
 * doubles (mu_r x,y,z, sigma x,y,z).  It allocates nothing: its scratch is a
 * fixed static device array sized for at most 32768 operator tiles (grids up
 * to about 512 x 512 x 256 cells, or any grid with
 * ceil((xs+1)/32) * ceil((ys+1)/8) * ceil((zs+1)/16) <= 32768; see
 * qms_residual_noalloc_fits); larger grids are rejected with QMS_ERR_ARG
 * before any launch.  The first call on a device looks up the scratch address
 * on that device.  The call synchronises `stream` before it returns, so it
 * must not be made while `stream` (or a stream it waits on) is being captured
 * into a CUDA graph.  All calls on one device share the scratch: they are
 * serialised on the host, and calls that overlap on the GPU (from other
 * processes) race.  It returns QMS_ERR_CUDA without launching anything when
 * the calling thread has an uncollected CUDA error. */
int qms_residual_noalloc(int xs, int ys, int zs, double dx, double dy, double dz, double dt, int transient,
                         const double v[3], const uint8_t* d_slots, const double* rows, int nmat,
                         const double* d_x, const double* d_b, double* d_r, double* d_sums, void* stream);
/* 1 when qms_residual_noalloc's fixed scratch holds a grid of xs x ys x zs cells, 0 otherwise
 * (host arithmetic only; no CUDA call). */
int qms_residual_noalloc_fits(int xs, int ys, int zs);

/* ------------------------------------------------------------------------
 * Serving: whole solves (the content of one inputs.txt + geom.bin pair, as
 * the reference program reads them, 3D/master.py:16-77) submitted to a
 * server object that admits them in arrival order while an HBM budget and a
 * slot limit allow, charging each its qms_device_bytes footprint.  Every
 * admitted solve is resident on its own handle, CUDA stream and worker thread,
 * so a request that arrives while others run starts as soon as memory and a
 * slot free up.  All reductions are fixed-order block sums: a request's
 * results are bit-identical alone and in any mix.  The server object is
 * internally synchronised; its calls may come from any thread.
 * ------------------------------------------------------------------------ */
typedef struct qms_server qms_server;

typedef struct {
    double budget_bytes;     /* HBM admission budget (bytes) */
    int max_resident;        /* concurrently resident solves */
    int device;
} qms_srv_desc;

enum { QMS_KEEP_NONE = 0, QMS_KEEP_SLICES = 1 };
enum { QMS_EXC_NONE = 0, QMS_EXC_COS = 1, QMS_EXC_SIN = 2 };

typedef struct {
    int xs, ys, zs;
    double dx, dy, dz, dt;
    int nt;                  /* transient steps after the steady state (inputs.txt line 4) */
    int tt;                  /* slice record every tt steps (line 5) */
    int slice_axis;          /* 0 = x, 1 = y, 2 = z (line 6) */
    int slice_index;         /* 1-based */
    int keep;                /* QMS_KEEP_NONE or QMS_KEEP_SLICES */
    int precision;           /* QMS_PREC_* */
    double B[3];             /* background field (line 8) */
    double G[9];             /* its gradient, row-major (lines 9-11) */
    double traj[3][3];       /* per axis: v0, acceleration, n_acc of trajectory type 1 (line 12);
                                amplitude, f, phase of type 2 */
    int exc_kind;            /* QMS_EXC_*: B and G scaled by cos/sin(2 pi f t + phase) */
    double exc_f, exc_phase;
    const double* geom;      /* xs*ys*zs float64 material IDs, Fortran order (copied at submit) */
    const double* table;     /* nmat x 7: ID, mu_r xyz, sigma xyz (copied at submit) */
    int nmat;
    /* Trajectory type per axis: 0 or 1 = the reference's type 1 (F:136-150); 2 = harmonic,
     * v(n) = amplitude sin(2 pi f n dt + phase); 3 = a velocity table of traj_len[d] values,
     * v(n) = traj_table[d][min(n, len - 1)] (copied at submit).  Types 2 and 3 extend the
     * reference, which stops on any type but 1 (F:135-151); the first-step pad applies to
     * type-1 axes only. */
    int traj_kind[3];
    const double* traj_table[3];
    int traj_len[3];
} qms_request;

enum { QMS_SRV_QUEUED = 0, QMS_SRV_RUNNING = 1, QMS_SRV_DONE = 2, QMS_SRV_FAILED = 3, QMS_SRV_REJECTED = 4 };

typedef struct {
    int state;               /* QMS_SRV_* */
    int rc;                  /* the failing call's return code (QMS_ERR_*) or 0 */
    long long n_dims;
    int steps_done;          /* transient steps completed */
    double arrival_s, admitted_s, finished_s;   /* seconds since the server was created */
    double steady_s;         /* steady-state solve */
    double step_mean_s, step_max_s;
    long long n_slice_values; /* values held by qms_srv_slices */
} qms_srv_result;

typedef struct {
    long long submitted, completed, failed, rejected;
    double step_p50_ms, step_p99_ms;             /* per transient step */
    double request_p50_s, request_p99_s;         /* arrival to finish */
    double queue_wait_p50_s, queue_wait_p99_s;   /* arrival to admission */
    double dof_timesteps;                        /* n_dims x steps over completed requests */
    double wall_s;                               /* first arrival to last finish */
    double peak_bytes;
    int peak_resident;
} qms_srv_stats;

int qms_srv_create(const qms_srv_desc* d, qms_server** out);
/* Queue a request (inputs are copied; the call returns at once).  A request whose
 * footprint exceeds the whole budget is recorded as QMS_SRV_REJECTED. */
int qms_srv_submit(qms_server* s, const qms_request* r, long long* id);
int qms_srv_poll(qms_server* s, long long id, qms_srv_result* out);      /* non-blocking */
int qms_srv_wait(qms_server* s, long long id, qms_srv_result* out);      /* until done, failed or rejected */
/* The slice records of a finished request (steady state, then every tt steps),
 * each the three components (Hx, Hy, Hz) of the slice back to back.  Copies at
 * most `cap` values; returns the number copied or a negative error. */
long long qms_srv_slices(qms_server* s, long long id, double* out, long long cap);
/* The error message of a failed or rejected request ("" otherwise; a fixed message for an
 * unknown id).  A request's message is written once, when it ends, and requests are never
 * removed from the server, so the pointer stays valid until qms_srv_destroy. */
const char* qms_srv_error(qms_server* s, long long id);
int qms_srv_stats_get(qms_server* s, qms_srv_stats* out);
/* Waits for every queued and running request, then frees the server. */
void qms_srv_destroy(qms_server* s);
/* The frame velocities a request's solve uses (host only, no device work): out[0..2] for the
 * steady state, out[3n..3n+2] for step n = 1..nsteps ((nsteps + 1) x 3 values). */
int qms_srv_velocities(const qms_request* r, int nsteps, double* out);

#ifdef __cplusplus
}
#endif
#endif
