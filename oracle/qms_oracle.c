/*
 * qms_oracle.c -- CPU restatement of the AlpineQMS QMS_3D per-step algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU library is
 * checked against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it.  The product path (alpineqms_gb300/) never links or
 * calls it.
 *
 * It restates, in source order and with the reference's literal precisions,
 * the parts of 3D/QMS_3D.f90 that make up the per-step hot path:
 *   sizes                     F:172-181
 *   material -> Yee coeffs    F:234-269  (face mu = harmonic mean, edge sigma = 4-cell mean,
 *                                         only indices 2..size, quirk kept)
 *   Dirichlet masks           F:361-396  (two-layer shell, as index predicates)
 *   steady CSR + RHS          F:448-1296 (row order, column order, formulas)
 *   CSR self-checks           F:1298-1312
 *   transient CSR + RHS       F:1457-2191
 *   unpack + H at centres     F:1320-1376, F:2211-2267
 *   trajectory_1 + pad        F:1428-1449, F:2331-2350
 *
 * Precision rules kept from the Fortran source (gfortran/ifx semantics of the
 * literals): "1/3.0" is a single-precision quotient (0.3333333432674408),
 * "1.0e-12" and "1E-8" are single-precision constants; every other literal
 * (0.5, 1.0, 2.0, 4.0) is exact.  Compile with -ffp-contract=off so no FMA
 * contraction changes the rounding of the source-order expressions.
 *
 * Indices are 1-based inside the formulas (as in the reference) and the CSR
 * arrays ia/ja are 1-based int32, exactly what the reference hands PARDISO
 * (F:1316, F:2196, F:2201).  The row pointer is closed form (1, 17 or 37
 * entries per row), so rows are filled in parallel with OpenMP after a serial
 * row-pointer pass; the values do not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MU0 1.25663706E-6 /* F:22, double literal (_dp) */

static const double THIRD = (double)(1.0f / 3.0f); /* F:465 "1/3.0" single precision */
static const double SIG_FLOOR = (double)1.0e-12f;  /* F:1237 "1.0e-12" single precision */
static const double PAD_EPS = (double)1E-8f;       /* F:1432 "1E-8" single precision */

typedef struct {
    int xs, ys, zs;        /* cells */
    int Nx, Ny, Nz;        /* nodes = cells + 1 (F:172-174) */
    int64_t Nn;            /* Nx*Ny*Nz (n_dims_1vec, F:176) */
    int64_t oY, oZ, oV;    /* global row offsets of the Ay, Az, V blocks (0-based count of rows before) */
    int64_t n;             /* n_dims (F:175) */
    double dx, dy, dz;
} grid_t;

static void grid_init(grid_t *g, int xs, int ys, int zs, double dx, double dy, double dz) {
    g->xs = xs; g->ys = ys; g->zs = zs;
    g->Nx = xs + 1; g->Ny = ys + 1; g->Nz = zs + 1;
    g->Nn = (int64_t)g->Nx * g->Ny * g->Nz;
    g->oY = g->Nn - (int64_t)g->Ny * g->Nz;
    g->oZ = 2 * g->Nn - (int64_t)g->Ny * g->Nz - (int64_t)g->Nx * g->Nz;
    g->oV = 3 * g->Nn - (int64_t)g->Ny * g->Nz - (int64_t)g->Nx * g->Nz - (int64_t)g->Nx * g->Ny;
    g->n = 4 * g->Nn - (int64_t)g->Ny * g->Nz - (int64_t)g->Nx * g->Nz - (int64_t)g->Nx * g->Ny;
    g->dx = dx; g->dy = dy; g->dz = dz;
}

/* 1-based global column numbers, F:455-457, F:628-631, F:802-805, F:976-979 */
#define CAX(i, j, k) ((int64_t)(i) + (int64_t)((j) - 1) * g->xs + (int64_t)((k) - 1) * g->xs * g->Ny)
#define CAY(i, j, k) (g->oY + (int64_t)(i) + (int64_t)((j) - 1) * g->Nx + (int64_t)((k) - 1) * g->Nx * g->ys)
#define CAZ(i, j, k) (g->oZ + (int64_t)(i) + (int64_t)((j) - 1) * g->Nx + (int64_t)((k) - 1) * g->Nx * g->Ny)
#define CV(i, j, k)  (g->oV + (int64_t)(i) + (int64_t)((j) - 1) * g->Nx + (int64_t)((k) - 1) * g->Nx * g->Ny)
/* node-sized coefficient arrays (Mu_x.., Sigma_x..), F-order, 1-based */
#define ND(i, j, k) ((int64_t)((i) - 1) + (int64_t)((j) - 1) * g->Nx + (int64_t)((k) - 1) * g->Nx * g->Ny)
/* cell arrays, F-order, 1-based */
#define CL(i, j, k) ((int64_t)((i) - 1) + (int64_t)((j) - 1) * g->xs + (int64_t)((k) - 1) * g->xs * g->ys)

/* Dirichlet predicates, F:361-396 */
static int fixed_x(const grid_t *g, int i, int j, int k) {
    return j <= 2 || j >= g->Ny - 1 || k <= 2 || k >= g->Nz - 1 || i == 1 || i == g->xs;
}
static int fixed_y(const grid_t *g, int i, int j, int k) {
    return i <= 2 || i >= g->Nx - 1 || k <= 2 || k >= g->Nz - 1 || j == 1 || j == g->ys;
}
static int fixed_z(const grid_t *g, int i, int j, int k) {
    return i <= 2 || i >= g->Nx - 1 || j <= 2 || j >= g->Ny - 1 || k == 1 || k == g->zs;
}
static int fixed_v(const grid_t *g, int i, int j, int k) {
    return i <= 2 || i >= g->Nx - 1 || j <= 2 || j >= g->Ny - 1 || k <= 2 || k >= g->Nz - 1;
}

/* ------------------------------------------------------------------------ */
/* sizes (F:172-181)                                                        */
/* ------------------------------------------------------------------------ */
void qmso_sizes(int xs, int ys, int zs, int64_t *n_dims, int64_t *nnz, int64_t *exact_nn) {
    grid_t G, *g = &G;
    grid_init(g, xs, ys, zs, 1, 1, 1);
    *n_dims = g->n;
    int64_t cnt = 0;
    for (int k = 1; k <= g->Nz; k++) for (int j = 1; j <= g->Ny; j++) for (int i = 1; i <= g->xs; i++)
        cnt += fixed_x(g, i, j, k) ? 1 : 17;
    for (int k = 1; k <= g->Nz; k++) for (int j = 1; j <= g->ys; j++) for (int i = 1; i <= g->Nx; i++)
        cnt += fixed_y(g, i, j, k) ? 1 : 17;
    for (int k = 1; k <= g->zs; k++) for (int j = 1; j <= g->Ny; j++) for (int i = 1; i <= g->Nx; i++)
        cnt += fixed_z(g, i, j, k) ? 1 : 17;
    for (int k = 1; k <= g->Nz; k++) for (int j = 1; j <= g->Ny; j++) for (int i = 1; i <= g->Nx; i++)
        cnt += fixed_v(g, i, j, k) ? 1 : 37;
    *nnz = cnt;
    /* F:179-181 (evaluated in 64-bit here; the reference's int32 overflows at >= 298^3) */
    int64_t nb = (2 * (int64_t)g->Nx + 2 * (int64_t)g->Ny - 4) * g->Nz;
    int64_t ni = ((int64_t)(g->Nx - 2) * (g->Ny - 2)) * g->Nz;
    *exact_nn = nb * 1 + ni * (15 * 3 + 37);
}

/* ------------------------------------------------------------------------ */
/* materials -> Yee coefficients (F:193-269)                                */
/*   geom: xs*ys*zs float64 material IDs, F-order (geom.bin, F:229-232)      */
/*   props: nmat rows of 7 doubles: id, mur_x, mur_y, mur_z, sig_x, sig_y, sig_z */
/*   out: mu_x..sig_z, each Nx*Ny*Nz, F-order                               */
/* returns 0, or -1 if an ID in geom is negative or above the largest table ID */
/* (the reference indexes temp_mat_id out of bounds there, F:243)            */
/* ------------------------------------------------------------------------ */
int qmso_materials(int xs, int ys, int zs, const double *geom, int nmat, const double *props,
                   double *mu_x, double *mu_y, double *mu_z,
                   double *sig_x, double *sig_y, double *sig_z) {
    grid_t G, *g = &G;
    grid_init(g, xs, ys, zs, 1, 1, 1);
    int maxid = 0;
    for (int r = 0; r < nmat; r++) { int id = (int)props[r * 7]; if (id > maxid) maxid = id; }
    int *tmi = (int *)calloc((size_t)maxid + 1, sizeof(int)); /* F:234-238 */
    for (int r = 0; r < nmat; r++) tmi[(int)props[r * 7]] = r + 1;
    int64_t nc = (int64_t)xs * ys * zs;
    double *mcx = malloc(nc * 8), *mcy = malloc(nc * 8), *mcz = malloc(nc * 8);
    double *scx = malloc(nc * 8), *scy = malloc(nc * 8), *scz = malloc(nc * 8);
    int bad = 0;
    for (int64_t c = 0; c < nc; c++) {
        mcx[c] = MU0; mcy[c] = MU0; mcz[c] = MU0;     /* F:211-213 */
        scx[c] = 0.0; scy[c] = 0.0; scz[c] = 0.0;     /* F:219-221 */
        int id = (int)geom[c];                        /* F:243 int() truncates */
        if (id < 0 || id > maxid) { bad = 1; continue; }
        int m = tmi[id];
        if (m != 0) {                                 /* F:244-251 */
            const double *p = props + (int64_t)(m - 1) * 7;
            mcx[c] = p[1] * MU0; mcy[c] = p[2] * MU0; mcz[c] = p[3] * MU0;
            scx[c] = p[4]; scy[c] = p[5]; scz[c] = p[6];
        }
    }
    for (int64_t q = 0; q < g->Nn; q++) {             /* F:215-225 */
        mu_x[q] = MU0; mu_y[q] = MU0; mu_z[q] = MU0;
        sig_x[q] = 0.0; sig_y[q] = 0.0; sig_z[q] = 0.0;
    }
    for (int k = 2; k <= zs; k++)                     /* F:258-269 */
        for (int j = 2; j <= ys; j++)
            for (int i = 2; i <= xs; i++) {
                double a, b;
                a = mcx[CL(i, j, k)]; b = mcx[CL(i - 1, j, k)];
                mu_x[ND(i, j, k)] = 2.0 * a * b / (a + b);
                a = mcy[CL(i, j, k)]; b = mcy[CL(i, j - 1, k)];
                mu_y[ND(i, j, k)] = 2.0 * a * b / (a + b);
                a = mcz[CL(i, j, k)]; b = mcz[CL(i, j, k - 1)];
                mu_z[ND(i, j, k)] = 2.0 * a * b / (a + b);
                sig_x[ND(i, j, k)] = (scx[CL(i, j, k)] + scx[CL(i, j, k - 1)] + scx[CL(i, j - 1, k)] + scx[CL(i, j - 1, k - 1)]) / 4.0;
                sig_y[ND(i, j, k)] = (scy[CL(i, j, k)] + scy[CL(i - 1, j, k)] + scy[CL(i, j, k - 1)] + scy[CL(i - 1, j, k - 1)]) / 4.0;
                sig_z[ND(i, j, k)] = (scz[CL(i, j, k)] + scz[CL(i - 1, j, k)] + scz[CL(i, j - 1, k)] + scz[CL(i - 1, j - 1, k)]) / 4.0;
            }
    free(tmi); free(mcx); free(mcy); free(mcz); free(scx); free(scy); free(scz);
    return bad ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* trajectory_1 (F:2331-2350) and the first-step pad (F:1428-1449)          */
/* ------------------------------------------------------------------------ */
double qmso_trajectory(double v, double a, int t, int n, double dt) {
    double r = 0.0;
    if (n <= t) r = v + a * n * dt;
    if (n > t) r = v + a * t * dt;
    return r;
}

/* velocity used by transient step `counter` (1-based).  `prev_v` is the
 * velocity in effect before the step (solve_v* at that point), `acc_state`
 * carries temp_acc_* between steps (static storage, starts at 0). */
double qmso_step_velocity(double v0, double a, int t, int counter, double dt,
                          double prev_v, double *acc_state) {
    if (counter == 1) {
        if (a * dt < v0 * PAD_EPS) *acc_state = prev_v * PAD_EPS / dt;
    } else {
        *acc_state = 0.0;
    }
    return qmso_trajectory(v0, a + *acc_state, t, counter, dt);
}

/* ------------------------------------------------------------------------ */
/* CSR assembly: steady (F:448-1296) and transient (F:1457-2191)            */
/* ------------------------------------------------------------------------ */
typedef struct {
    const grid_t *g;
    const double *mux, *muy, *muz, *sgx, *sgy, *sgz;
} coef_t;

#define MUX(i, j, k) (c->mux[ND(i, j, k)])
#define MUY(i, j, k) (c->muy[ND(i, j, k)])
#define MUZ(i, j, k) (c->muz[ND(i, j, k)])
#define SGX(i, j, k) (c->sgx[ND(i, j, k)])
#define SGY(i, j, k) (c->sgy[ND(i, j, k)])
#define SGZ(i, j, k) (c->sgz[ND(i, j, k)])
#define PUT(col, val) do { ja[p] = (int32_t)(col); a[p] = (val); p++; } while (0)

/* Fills row `rr` (0-based row index into b, 1-based column numbers into ja)
 * starting at CSR position p.  tr = 1 for the transient form. */
static void row_ax(const coef_t *c, int i, int j, int k, int tr, double dt, const double *v,
                   const double *B, const double *Gm, const double *xp,
                   int64_t rr, int64_t p, int32_t *ja, double *a, double *b) {
    const grid_t *g = c->g;
    const double dx = g->dx, dy = g->dy, dz = g->dz, vx = v[0], vy = v[1], vz = v[2];
    (void)vx;
    if (fixed_x(g, i, j, k)) {                                       /* F:460-469, F:1465-1473 */
        double xq = (i - 1) * dx, yq = (j - 1) * dy, zq = (k - 1) * dz;
        b[rr] = 0.5 * B[1] * (zq) - 0.5 * B[2] * (yq) +
                THIRD * ((Gm[3] * xq + Gm[4] * yq + Gm[5] * zq) * zq - (Gm[6] * xq + Gm[7] * yq + Gm[8] * zq) * yq);
        PUT(rr + 1, 1.0);
        return;
    }
    if (tr) b[rr] = (SGX(i, j, k) / dt) * xp[CAX(i, j, k) - 1];     /* F:1475 */
    const double s = SGX(i, j, k);
    PUT(CAX(i, j, k - 1), -1.0 / MUY(i, j, k - 1) / (dz * dz) + (s * vz) / (2.0 * dz));     /* F:476-481 */
    PUT(CAX(i, j - 1, k), -1.0 / MUZ(i, j - 1, k) / (dy * dy) + (s * vy) / (2.0 * dy));     /* F:483-488 */
    PUT(CAX(i - 1, j, k), -1.0 / MUX(i - 1, j, k) / (dx * dx));                            /* F:490-495 */
    {
        double w = (1.0 / MUZ(i, j, k) + 1.0 / MUZ(i, j - 1, k)) / (dy * dy)
                 + (1.0 / MUY(i, j, k) + 1.0 / MUY(i, j, k - 1)) / (dz * dz)
                 + (1.0 / MUX(i, j, k) + 1.0 / MUX(i - 1, j, k)) / (dx * dx);            /* F:497-504 */
        if (tr) w = w + s / dt;                                                            /* F:1500-1504 */
        PUT(CAX(i, j, k), w);
    }
    PUT(CAX(i + 1, j, k), -1.0 / MUX(i, j, k) / (dx * dx));                                /* F:506-511 */
    PUT(CAX(i, j + 1, k), -1.0 / MUZ(i, j, k) / (dy * dy) - (s * vy) / (2.0 * dy));         /* F:513-518 */
    PUT(CAX(i, j, k + 1), -1.0 / MUY(i, j, k) / (dz * dz) - (s * vz) / (2.0 * dz));         /* F:520-525 */
    PUT(CAY(i, j - 1, k), 1.0 / MUZ(i, j - 1, k) / (dx * dy) - (s * vy) / (2.0 * dx));      /* F:531-536 */
    PUT(CAY(i + 1, j - 1, k), -1.0 / MUZ(i, j - 1, k) / (dx * dy) + (s * vy) / (2.0 * dx)); /* F:538-543 */
    PUT(CAY(i, j, k), -1.0 / MUZ(i, j, k) / (dx * dy) - (s * vy) / (2.0 * dx));             /* F:545-550 */
    PUT(CAY(i + 1, j, k), 1.0 / MUZ(i, j, k) / (dx * dy) + (s * vy) / (2.0 * dx));          /* F:552-557 */
    PUT(CAZ(i, j, k - 1), 1.0 / MUY(i, j, k - 1) / (dx * dz) - (s * vz) / (2.0 * dx));      /* F:563-568 */
    PUT(CAZ(i + 1, j, k - 1), -1.0 / MUY(i, j, k - 1) / (dx * dz) + (s * vz) / (2.0 * dx)); /* F:570-575 */
    PUT(CAZ(i, j, k), -1.0 / MUY(i, j, k) / (dx * dz) - (s * vz) / (2.0 * dx));             /* F:577-582 */
    PUT(CAZ(i + 1, j, k), 1.0 / MUY(i, j, k) / (dx * dz) + (s * vz) / (2.0 * dx));          /* F:584-589 */
    PUT(CV(i, j, k), -SGX(i, j, k) / dx);                                                  /* F:595-600 */
    PUT(CV(i + 1, j, k), SGX(i, j, k) / dx);                                               /* F:602-607 */
}

static void row_ay(const coef_t *c, int i, int j, int k, int tr, double dt, const double *v,
                   const double *B, const double *Gm, const double *xp,
                   int64_t rr, int64_t p, int32_t *ja, double *a, double *b) {
    const grid_t *g = c->g;
    const double dx = g->dx, dy = g->dy, dz = g->dz, vx = v[0], vz = v[2];
    if (fixed_y(g, i, j, k)) {                                       /* F:634-644, F:1614-1622 */
        double xq = (i - 1) * dx, yq = (j - 1) * dy, zq = (k - 1) * dz;
        b[rr] = 0.5 * B[2] * (xq) - 0.5 * B[0] * (zq) +
                THIRD * ((Gm[6] * xq + Gm[7] * yq + Gm[8] * zq) * xq - (Gm[0] * xq + Gm[1] * yq + Gm[2] * zq) * zq);
        PUT(rr + 1, 1.0);
        return;
    }
    if (tr) b[rr] = (SGY(i, j, k) / dt) * xp[CAY(i, j, k) - 1];     /* F:1624 */
    const double s = SGY(i, j, k);
    PUT(CAX(i - 1, j, k), 1.0 / MUZ(i - 1, j, k) / (dx * dy) - (s * vx) / (2.0 * dy));      /* F:650-655 */
    PUT(CAX(i, j, k), -1.0 / MUZ(i, j, k) / (dx * dy) - (s * vx) / (2.0 * dy));             /* F:657-662 */
    PUT(CAX(i - 1, j + 1, k), -1.0 / MUZ(i - 1, j, k) / (dx * dy) + (s * vx) / (2.0 * dy)); /* F:664-669 */
    PUT(CAX(i, j + 1, k), 1.0 / MUZ(i, j, k) / (dx * dy) + (s * vx) / (2.0 * dy));          /* F:671-676 */
    PUT(CAY(i, j, k - 1), -1.0 / MUX(i, j, k - 1) / (dz * dz) + (s * vz) / (2.0 * dz));     /* F:682-687 */
    PUT(CAY(i, j - 1, k), -1.0 / MUY(i, j - 1, k) / (dy * dy));                            /* F:689-694 */
    PUT(CAY(i - 1, j, k), -1.0 / MUZ(i - 1, j, k) / (dx * dx) + (s * vx) / (2.0 * dx));     /* F:696-701 */
    {
        double w = (1.0 / MUZ(i, j, k) + 1.0 / MUZ(i - 1, j, k)) / (dx * dx)
                 + (1.0 / MUX(i, j, k) + 1.0 / MUX(i, j, k - 1)) / (dz * dz)
                 + (1.0 / MUY(i, j, k) + 1.0 / MUY(i, j - 1, k)) / (dy * dy);            /* F:703-710 */
        if (tr) w = w + s / dt;                                                            /* F:1677-1681 */
        PUT(CAY(i, j, k), w);
    }
    PUT(CAY(i + 1, j, k), -1.0 / MUZ(i, j, k) / (dx * dx) - (s * vx) / (2.0 * dx));         /* F:712-717 */
    PUT(CAY(i, j + 1, k), -1.0 / MUY(i, j, k) / (dy * dy));                                /* F:719-724 */
    PUT(CAY(i, j, k + 1), -1.0 / MUX(i, j, k) / (dz * dz) - (s * vz) / (2.0 * dz));         /* F:726-731 */
    PUT(CAZ(i, j, k - 1), 1.0 / MUX(i, j, k - 1) / (dy * dz) - (s * vz) / (2.0 * dy));      /* F:737-742 */
    PUT(CAZ(i, j + 1, k - 1), -1.0 / MUX(i, j, k - 1) / (dy * dz) + (s * vz) / (2.0 * dy)); /* F:744-749 */
    PUT(CAZ(i, j, k), -1.0 / MUX(i, j, k) / (dy * dz) - (s * vz) / (2.0 * dy));             /* F:751-756 */
    PUT(CAZ(i, j + 1, k), 1.0 / MUX(i, j, k) / (dy * dz) + (s * vz) / (2.0 * dy));          /* F:758-763 */
    PUT(CV(i, j, k), -SGY(i, j, k) / dy);                                                  /* F:769-774 */
    PUT(CV(i, j + 1, k), SGY(i, j, k) / dy);                                               /* F:776-781 */
}

static void row_az(const coef_t *c, int i, int j, int k, int tr, double dt, const double *v,
                   const double *B, const double *Gm, const double *xp,
                   int64_t rr, int64_t p, int32_t *ja, double *a, double *b) {
    const grid_t *g = c->g;
    const double dx = g->dx, dy = g->dy, dz = g->dz, vx = v[0], vy = v[1];
    if (fixed_z(g, i, j, k)) {                                       /* F:808-818, F:1762-1770 */
        double xq = (i - 1) * dx, yq = (j - 1) * dy, zq = (k - 1) * dz;
        b[rr] = 0.5 * B[0] * yq - 0.5 * B[1] * xq +
                THIRD * ((Gm[0] * xq + Gm[1] * yq + Gm[2] * zq) * yq - (Gm[3] * xq + Gm[4] * yq + Gm[5] * zq) * xq);
        PUT(rr + 1, 1.0);
        return;
    }
    if (tr) b[rr] = (SGZ(i, j, k) / dt) * xp[CAZ(i, j, k) - 1];     /* F:1772 */
    const double s = SGZ(i, j, k);
    PUT(CAX(i - 1, j, k), 1.0 / MUY(i - 1, j, k) / (dx * dz) - (s * vx) / (2.0 * dz));      /* F:824-829 */
    PUT(CAX(i, j, k), -1.0 / MUY(i, j, k) / (dx * dz) - (s * vx) / (2.0 * dz));             /* F:831-836 */
    PUT(CAX(i - 1, j, k + 1), -1.0 / MUY(i - 1, j, k) / (dx * dz) + (s * vx) / (2.0 * dz)); /* F:838-843 */
    PUT(CAX(i, j, k + 1), 1.0 / MUY(i, j, k) / (dx * dz) + (s * vx) / (2.0 * dz));          /* F:845-850 */
    PUT(CAY(i, j - 1, k), 1.0 / MUX(i, j - 1, k) / (dy * dz) - (s * vy) / (2.0 * dz));      /* F:856-861 */
    PUT(CAY(i, j, k), -1.0 / MUX(i, j, k) / (dy * dz) - (s * vy) / (2.0 * dz));             /* F:863-868 */
    PUT(CAY(i, j - 1, k + 1), -1.0 / MUX(i, j - 1, k) / (dy * dz) + (s * vy) / (2.0 * dz)); /* F:870-875 */
    PUT(CAY(i, j, k + 1), 1.0 / MUX(i, j, k) / (dy * dz) + (s * vy) / (2.0 * dz));          /* F:877-882 */
    PUT(CAZ(i, j, k - 1), -1.0 / MUZ(i, j, k - 1) / (dz * dz));                            /* F:888-893 */
    PUT(CAZ(i, j - 1, k), -1.0 / MUX(i, j - 1, k) / (dy * dy) + (s * vy) / (2.0 * dy));     /* F:895-900 */
    PUT(CAZ(i - 1, j, k), -1.0 / MUY(i - 1, j, k) / (dx * dx) + (s * vx) / (2.0 * dx));     /* F:902-907 */
    {
        double w = (1.0 / MUY(i, j, k) + 1.0 / MUY(i - 1, j, k)) / (dx * dx)
                 + (1.0 / MUX(i, j, k) + 1.0 / MUX(i, j - 1, k)) / (dy * dy)
                 + (1.0 / MUZ(i, j, k) + 1.0 / MUZ(i, j, k - 1)) / (dz * dz);            /* F:909-916 */
        if (tr) w = w + s / dt;                                                            /* F:1853-1857 */
        PUT(CAZ(i, j, k), w);
    }
    PUT(CAZ(i + 1, j, k), -1.0 / MUY(i, j, k) / (dx * dx) - (s * vx) / (2.0 * dx));         /* F:918-923 */
    PUT(CAZ(i, j + 1, k), -1.0 / MUX(i, j, k) / (dy * dy) - (s * vy) / (2.0 * dy));         /* F:925-930 */
    PUT(CAZ(i, j, k + 1), -1.0 / MUZ(i, j, k) / (dz * dz));                                /* F:932-937 */
    PUT(CV(i, j, k), -SGZ(i, j, k) / dz);                                                  /* F:943-948 */
    PUT(CV(i, j, k + 1), SGZ(i, j, k) / dz);                                               /* F:950-955 */
}

static void row_v(const coef_t *c, int i, int j, int k, int tr, double dt, const double *v,
                  const double *B, const double *Gm, const double *xp,
                  int64_t rr, int64_t p, int32_t *ja, double *a, double *b) {
    const grid_t *g = c->g;
    const double dx = g->dx, dy = g->dy, dz = g->dz, vx = v[0], vy = v[1], vz = v[2];
    if (fixed_v(g, i, j, k)) {                                       /* F:982-996, F:1910-1922 */
        double xq = (i - 1) * dx, yq = (j - 1) * dy, zq = (k - 1) * dz;
        double gx = Gm[0] * xq + Gm[1] * yq + Gm[2] * zq;
        double gy = Gm[3] * xq + Gm[4] * yq + Gm[5] * zq;
        double gz = Gm[6] * xq + Gm[7] * yq + Gm[8] * zq;
        b[rr] = -1.0 * (vy * B[2] - vz * B[1]) * xq
                - 1.0 * (vz * B[0] - vx * B[2]) * yq
                - 1.0 * (vx * B[1] - vy * B[0]) * zq
                - 0.5 * (vy * gz - vz * gy) * xq
                - 0.5 * (vz * gx - vx * gz) * yq
                - 0.5 * (vx * gy - vy * gx) * zq;
        PUT(rr + 1, 1.0);
        return;
    }
    if (tr) {                                                        /* F:1925-1928 */
        b[rr] = (SGX(i, j, k) * xp[CAX(i, j, k) - 1] - SGX(i - 1, j, k) * xp[CAX(i - 1, j, k) - 1]) / (dt * dx)
              + (SGY(i, j, k) * xp[CAY(i, j, k) - 1] - SGY(i, j - 1, k) * xp[CAY(i, j - 1, k) - 1]) / (dt * dy)
              + (SGZ(i, j, k) * xp[CAZ(i, j, k) - 1] - SGZ(i, j, k - 1) * xp[CAZ(i, j, k - 1) - 1]) / (dt * dz);
    }
    const double sx0 = SGX(i, j, k), sx1 = SGX(i - 1, j, k);          /* F:1003-1008 */
    const double sy0 = SGY(i, j, k), sy1 = SGY(i, j - 1, k);
    const double sz0 = SGZ(i, j, k), sz1 = SGZ(i, j, k - 1);
    const double dz2 = dz * dz, dy2 = dy * dy, dx2 = dx * dx;
    /* Ax entries, F:1014-1082 (transient additions F:1973-1985) */
    PUT(CAX(i - 1, j, k - 1), sx1 * vz / (2.0 * dz * dx) - sz1 * vx / (2.0 * dz2));
    PUT(CAX(i, j, k - 1), -sx0 * vz / (2.0 * dz * dx) - sz1 * vx / (2.0 * dz2));
    PUT(CAX(i - 1, j - 1, k), sx1 * vy / (2.0 * dy * dx) - sy1 * vx / (2.0 * dy2));
    PUT(CAX(i, j - 1, k), -sx0 * vy / (2.0 * dy * dx) - sy1 * vx / (2.0 * dy2));
    {
        double w = (sy0 + sy1) * vx / (2.0 * dy2) + (sz0 + sz1) * vx / (2.0 * dz2);
        if (tr) w = w - sx1 / (dx * dt);
        PUT(CAX(i - 1, j, k), w);
        w = (sy0 + sy1) * vx / (2.0 * dy2) + (sz0 + sz1) * vx / (2.0 * dz2);
        if (tr) w = w + sx0 / (dx * dt);
        PUT(CAX(i, j, k), w);
    }
    PUT(CAX(i - 1, j + 1, k), -sx1 * vy / (2.0 * dy * dx) - sy0 * vx / (2.0 * dy2));
    PUT(CAX(i, j + 1, k), sx0 * vy / (2.0 * dy * dx) - sy0 * vx / (2.0 * dy2));
    PUT(CAX(i - 1, j, k + 1), -sx1 * vz / (2.0 * dz * dx) - sz0 * vx / (2.0 * dz2));
    PUT(CAX(i, j, k + 1), sx0 * vz / (2.0 * dz * dx) - sz0 * vx / (2.0 * dz2));
    /* Ay entries, F:1088-1156 (transient F:2033-2035, F:2052-2054) */
    PUT(CAY(i, j - 1, k - 1), sy1 * vz / (2.0 * dz * dy) - sz1 * vy / (2.0 * dz2));
    PUT(CAY(i, j, k - 1), -sy0 * vz / (2.0 * dz * dy) - sz1 * vy / (2.0 * dz2));
    PUT(CAY(i - 1, j - 1, k), -sx1 * vy / (2.0 * dx2) + sy1 * vx / (2.0 * dx * dy));
    {
        double w = (sx0 + sx1) * vy / (2.0 * dx2) + (sz0 + sz1) * vy / (2.0 * dz2);
        if (tr) w = w - sy1 / (dy * dt);
        PUT(CAY(i, j - 1, k), w);
    }
    PUT(CAY(i + 1, j - 1, k), -sx0 * vy / (2.0 * dx2) - sy1 * vx / (2.0 * dx * dy));
    PUT(CAY(i - 1, j, k), -sx1 * vy / (2.0 * dx2) - sy0 * vx / (2.0 * dx * dy));
    {
        double w = (sx0 + sx1) * vy / (2.0 * dx2) + (sz0 + sz1) * vy / (2.0 * dz2);
        if (tr) w = w + sy0 / (dy * dt);
        PUT(CAY(i, j, k), w);
    }
    PUT(CAY(i + 1, j, k), -sx0 * vy / (2.0 * dx2) + sy0 * vx / (2.0 * dx * dy));
    PUT(CAY(i, j - 1, k + 1), -sy1 * vz / (2.0 * dz * dy) - sz0 * vy / (2.0 * dz2));
    PUT(CAY(i, j, k + 1), sy0 * vz / (2.0 * dz * dy) - sz0 * vy / (2.0 * dz2));
    /* Az entries, F:1162-1230 (transient F:2093-2095, F:2124-2126) */
    PUT(CAZ(i, j - 1, k - 1), -sy1 * vz / (2.0 * dy2) + sz1 * vy / (2.0 * dy * dz));
    PUT(CAZ(i - 1, j, k - 1), -sx1 * vz / (2.0 * dx2) + sz1 * vx / (2.0 * dx * dz));
    {
        double w = (sx0 + sx1) * vz / (2.0 * dx2) + (sy0 + sy1) * vz / (2.0 * dy2);
        if (tr) w = w - sz1 / (dz * dt);
        PUT(CAZ(i, j, k - 1), w);
    }
    PUT(CAZ(i + 1, j, k - 1), -sx0 * vz / (2.0 * dx2) - sz1 * vx / (2.0 * dx * dz));
    PUT(CAZ(i, j + 1, k - 1), -sy0 * vz / (2.0 * dy2) - sz1 * vy / (2.0 * dy * dz));
    PUT(CAZ(i, j - 1, k), -sy1 * vz / (2.0 * dy2) - sz0 * vy / (2.0 * dy * dz));
    PUT(CAZ(i - 1, j, k), -sx1 * vz / (2.0 * dx2) - sz0 * vx / (2.0 * dx * dz));
    {
        double w = (sx0 + sx1) * vz / (2.0 * dx2) + (sy0 + sy1) * vz / (2.0 * dy2);
        if (tr) w = w + sz0 / (dz * dt);
        PUT(CAZ(i, j, k), w);
    }
    PUT(CAZ(i + 1, j, k), -sx0 * vz / (2.0 * dx2) + sz0 * vx / (2.0 * dx * dz));
    PUT(CAZ(i, j + 1, k), -sy0 * vz / (2.0 * dy2) + sz0 * vy / (2.0 * dy * dz));
    /* V entries, F:1236-1285 (identical in the transient form, F:2147-2189) */
    PUT(CV(i, j, k - 1), -fmax(SGZ(i, j, k - 1), SIG_FLOOR) / dz2);
    PUT(CV(i, j - 1, k), -fmax(SGY(i, j - 1, k), SIG_FLOOR) / dy2);
    PUT(CV(i - 1, j, k), -fmax(SGX(i - 1, j, k), SIG_FLOOR) / dx2);
    PUT(CV(i, j, k), (fmax(SGX(i, j, k), SIG_FLOOR) + fmax(SGX(i - 1, j, k), SIG_FLOOR)) / dx2
                   + (fmax(SGY(i, j, k), SIG_FLOOR) + fmax(SGY(i, j - 1, k), SIG_FLOOR)) / dy2
                   + (fmax(SGZ(i, j, k), SIG_FLOOR) + fmax(SGZ(i, j, k - 1), SIG_FLOOR)) / dz2);
    PUT(CV(i + 1, j, k), -fmax(SGX(i, j, k), SIG_FLOOR) / dx2);
    PUT(CV(i, j + 1, k), -fmax(SGY(i, j, k), SIG_FLOOR) / dy2);
    PUT(CV(i, j, k + 1), -fmax(SGZ(i, j, k), SIG_FLOOR) / dz2);
}

/* The fmax() above differs from Fortran MAX only for NaN inputs, which the
 * material table cannot produce. */

/*
 * Assemble the full system.  tr = 0: steady form (F:448-1296, b is zero on
 * interior rows); tr = 1: transient form (F:1457-2191) whose RHS reads the
 * previous solution x_prev (n_dims, the reference's x_vec layout).
 * v = solve_v{x,y,z}; B = B_in; Gm = the 3x3 gradient row-major
 * (gxx gxy gxz gyx ... gzz).  ia has n+1 entries, ja/a have nnz entries.
 * Returns nnz, or -1 if nnz does not fit the int32 ja/ia of the reference,
 * or -2 if the sortedness / sign checks of F:1298-1312 fail.
 */
int64_t qmso_assemble(int xs, int ys, int zs, double dx, double dy, double dz,
                      const double *mu_x, const double *mu_y, const double *mu_z,
                      const double *sig_x, const double *sig_y, const double *sig_z,
                      int tr, double dt, const double *v, const double *B, const double *Gm,
                      const double *x_prev, int32_t *ia, int32_t *ja, double *a, double *b) {
    grid_t G, *g = &G;
    grid_init(g, xs, ys, zs, dx, dy, dz);
    coef_t C = {g, mu_x, mu_y, mu_z, sig_x, sig_y, sig_z}, *c = &C;
    /* serial row pointer pass (closed form row lengths) */
    int64_t p = 1, r = 0;
    for (int k = 1; k <= g->Nz; k++) for (int j = 1; j <= g->Ny; j++) for (int i = 1; i <= g->xs; i++, r++) {
        if (p > INT32_MAX) return -1;
        ia[r] = (int32_t)p; p += fixed_x(g, i, j, k) ? 1 : 17;
    }
    for (int k = 1; k <= g->Nz; k++) for (int j = 1; j <= g->ys; j++) for (int i = 1; i <= g->Nx; i++, r++) {
        if (p > INT32_MAX) return -1;
        ia[r] = (int32_t)p; p += fixed_y(g, i, j, k) ? 1 : 17;
    }
    for (int k = 1; k <= g->zs; k++) for (int j = 1; j <= g->Ny; j++) for (int i = 1; i <= g->Nx; i++, r++) {
        if (p > INT32_MAX) return -1;
        ia[r] = (int32_t)p; p += fixed_z(g, i, j, k) ? 1 : 17;
    }
    for (int k = 1; k <= g->Nz; k++) for (int j = 1; j <= g->Ny; j++) for (int i = 1; i <= g->Nx; i++, r++) {
        if (p > INT32_MAX) return -1;
        ia[r] = (int32_t)p; p += fixed_v(g, i, j, k) ? 1 : 37;
    }
    if (p > INT32_MAX) return -1;
    ia[g->n] = (int32_t)p;                                                   /* F:1296 */
    int64_t nnz = p - 1;
    for (int64_t q = 0; q < g->n; q++) b[q] = 0.0;                          /* F:354 */

    const int64_t nAx = (int64_t)g->xs * g->Ny * g->Nz, nAy = (int64_t)g->Nx * g->ys * g->Nz;
    const int64_t nAz = (int64_t)g->Nx * g->Ny * g->zs, nV = g->Nn;
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nAx; q++) {
        int i = (int)(q % g->xs) + 1, j = (int)((q / g->xs) % g->Ny) + 1, k = (int)(q / ((int64_t)g->xs * g->Ny)) + 1;
        row_ax(c, i, j, k, tr, dt, v, B, Gm, x_prev, q, ia[q] - 1, ja, a, b);
    }
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nAy; q++) {
        int i = (int)(q % g->Nx) + 1, j = (int)((q / g->Nx) % g->ys) + 1, k = (int)(q / ((int64_t)g->Nx * g->ys)) + 1;
        int64_t rr = g->oY + q;
        row_ay(c, i, j, k, tr, dt, v, B, Gm, x_prev, rr, ia[rr] - 1, ja, a, b);
    }
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nAz; q++) {
        int i = (int)(q % g->Nx) + 1, j = (int)((q / g->Nx) % g->Ny) + 1, k = (int)(q / ((int64_t)g->Nx * g->Ny)) + 1;
        int64_t rr = g->oZ + q;
        row_az(c, i, j, k, tr, dt, v, B, Gm, x_prev, rr, ia[rr] - 1, ja, a, b);
    }
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nV; q++) {
        int i = (int)(q % g->Nx) + 1, j = (int)((q / g->Nx) % g->Ny) + 1, k = (int)(q / ((int64_t)g->Nx * g->Ny)) + 1;
        int64_t rr = g->oV + q;
        row_v(c, i, j, k, tr, dt, v, B, Gm, x_prev, rr, ia[rr] - 1, ja, a, b);
    }
    /* F:1298-1312: strictly increasing columns in each row, no negative column */
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t q = 0; q < g->n; q++) {
        for (int64_t e = ia[q]; e <= (int64_t)ia[q + 1] - 2; e++)
            if (ja[e - 1] >= ja[e]) bad |= 1;
        for (int64_t e = ia[q]; e < ia[q + 1]; e++)
            if (ja[e - 1] < 0) bad |= 1;
    }
    return bad ? -2 : nnz;
}

/* ------------------------------------------------------------------------ */
/* H at cell centres from the solution vector (F:1320-1376, F:2211-2267)    */
/* x: n_dims solution (A blocks used, V dropped as in F:1319)               */
/* Hx, Hy, Hz: xs*ys*zs each, F-order                                       */
/* ------------------------------------------------------------------------ */
void qmso_hfield(int xs, int ys, int zs, double dx, double dy, double dz,
                 const double *mu_x, const double *mu_y, const double *mu_z,
                 const double *x, double *Hx, double *Hy, double *Hz) {
    grid_t G, *g = &G;
    grid_init(g, xs, ys, zs, dx, dy, dz);
#define XAX(i, j, k) x[CAX(i, j, k) - 1]
#define XAY(i, j, k) x[CAY(i, j, k) - 1]
#define XAZ(i, j, k) x[CAZ(i, j, k) - 1]
#define MX(i, j, k) mu_x[ND(i, j, k)]
#define MY(i, j, k) mu_y[ND(i, j, k)]
#define MZ(i, j, k) mu_z[ND(i, j, k)]
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= zs; k++)
        for (int j = 1; j <= ys; j++)
            for (int i = 1; i <= xs; i++) {
                int64_t cq = CL(i, j, k);
                Hx[cq] = 0.5 * (((XAZ(i, j + 1, k) - XAZ(i, j, k)) / dy - (XAY(i, j, k + 1) - XAY(i, j, k)) / dz) / MX(i, j, k) +
                                ((XAZ(i + 1, j + 1, k) - XAZ(i + 1, j, k)) / dy - (XAY(i + 1, j, k + 1) - XAY(i + 1, j, k)) / dz) / MX(i + 1, j, k));
                Hy[cq] = 0.5 * (((XAX(i, j, k + 1) - XAX(i, j, k)) / dz - (XAZ(i + 1, j, k) - XAZ(i, j, k)) / dx) / MY(i, j, k) +
                                ((XAX(i, j + 1, k + 1) - XAX(i, j + 1, k)) / dz - (XAZ(i + 1, j + 1, k) - XAZ(i, j + 1, k)) / dx) / MY(i, j + 1, k));
                Hz[cq] = 0.5 * (((XAY(i + 1, j, k) - XAY(i, j, k)) / dx - (XAX(i, j + 1, k) - XAX(i, j, k)) / dy) / MZ(i, j, k) +
                                ((XAY(i + 1, j, k + 1) - XAY(i, j, k + 1)) / dx - (XAX(i, j + 1, k + 1) - XAX(i, j, k + 1)) / dy) / MZ(i, j, k + 1));
            }
}

int qmso_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
