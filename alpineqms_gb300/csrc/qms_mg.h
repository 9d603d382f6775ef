// qms_mg.h -- block-diagonal aggregation multigrid (see qms_mg.cu).
#pragma once
#include "qms_internal.h"
#include "qms_tma.cuh"

#include <algorithm>
#include <string>
#include <vector>

#define MG_MAX_BLOCKS 4

struct MGBlockDesc {
    int n1, n2, n3;
    long long off;          // first point of this block in the level's flat arrays
};

// one level of the hierarchy: all blocks back to back (a packed descriptor table)
template <typename T>
struct MGLevelDev {
    int nb;
    MGBlockDesc blk[MG_MAX_BLOCKS];
    long long total;
    T* w1;                  // link to the +1 neighbour along axis 1 (0 when absent / inactive)
    T* w2;
    T* w3;
    T* dg;                  // diagonal
    T* dinv;                // 1/diagonal, 0 on inactive (Dirichlet) points
    T* x;                   // correction (levels > 0)
    T* b;                   // right-hand side (levels > 0)
    T* t;                   // Jacobi temporary
    T* mass;                // sum of the level-0 diagonals a point aggregates (levels > 0)
};

// Optional timing of selected multigrid launches (CUDA events bracketing them on the stream):
// begin() returns a token for end(), or null when profiling is off.
struct MgProf {
    virtual void* begin(int kind, double bytes) = 0;
    virtual void end(void* token) = 0;
    virtual ~MgProf() {}
};
enum { MGPROF_A_SWEEP = 4 };     // a level-0 Jacobi sweep on the three A blocks (mg0_tiled, KIND 1, QS 1)

template <typename T>
struct QmsMG {
    std::vector<MGLevelDev<T>> lv;
    std::vector<MGLevelDev<T>> views[3];   // [1]: the A blocks of every level, [2]: the V block
    double* dminv = nullptr;       // dense FP64 inverses of the coarsest blocks
    long long* dmoff = nullptr;
    int nu1 = 2, nu2 = 2;
    int nu_coarse = 0;             // sweeps on each side on levels >= 1 (0: nu1 / nu2)
    int nu_v = 0;                  // sweeps on each side, every level, of a V-block cycle (0: as above)
    long long tail_points = 4096;  // levels of at most this many points per block run as one launch (0: off)
    T omega = T(0.8);
    T alpha = T(1);
    int min_coarse = 5;
    int max_levels = 12;
    T* cur_x0 = nullptr;
    T* cur_t0 = nullptr;
    // level 0 on node tiles (the operator's staged coefficients) instead of stored links
    bool tiled0 = false;
    QGrid g0{};
    QCoef<T> c0{};
    QStepPar<T> P0{};
    T vshift0 = T(0);
    MgProf* prof = nullptr;
    // Near-null points and modes of the V block: a coarse point whose Galerkin diagonal is at or
    // below vcut times the summed level-0 diagonals it aggregates (a floating conductor that
    // collapsed into it; the value is then rounding noise) leaves the hierarchy, and the coarsest
    // V solve drops eigenvalues of its operator scaled by those sums at or below vcut.
    // 0 = automatic: 1e-9 for an FP64 hierarchy, 1e-5 for FP32 (its cancellation noise is ~1e-7).
    double vcut = 0.0;
    dim3 g0grid, g0block;
    std::string err;

    ~QmsMG();
    void release();
    static size_t bytes_for(const QGrid& g, int min_coarse, bool tiled);
    int build(const QGrid& g, const QCoef<T>& c, const QStepPar<T>& P, T vshift, cudaStream_t st);
    // z = MG(r) on the padded layout: b0 (scaled by the operator diagonal when `scaled`), x0 the
    // result, t0 a temporary; the tensor maps of x0, t0 and of the node coefficients
    // qs: 0 all blocks, 1 the A blocks only, 2 the V block only (x0map / t0map then cover those
    // blocks, cmap the node coefficients they read: all six, or the three conductivities)
    // b0map (qs 1 or 2, scaled): b0's tensor map over the cycle's blocks; the first two level-0
    // sweeps then run as one pass from b0's tiles
    int vcycle(const T* b0, bool scaled, T* x0, const CUtensorMap& x0map, T* t0, const CUtensorMap& t0map,
               const CUtensorMap& cmap, bool mask_v, unsigned* err, cudaStream_t st, int qs = 0,
               const CUtensorMap* b0map = nullptr);
    template <int QS>
    int vcycle_q(const T* b0, bool scaled, T* x0, const CUtensorMap& x0map, T* t0, const CUtensorMap& t0map,
                 const CUtensorMap& cmap, bool mask_v, unsigned* err, cudaStream_t st, const CUtensorMap* b0map);
    static int levels_for(const QGrid& g, int min_coarse);
};

// Coarse space of the V block spanned by one indicator vector per conductor region (a
// connected body of cells of one material with sigma > 1 S/m; a V node belongs to the
// region of its incident conductor cell with the largest sigma).  Potential offsets of
// bodies that touch others only through a few edges are near-null modes of the V
// operator that the geometric aggregation cannot represent; this space captures them.
// Applied additively to the multigrid V-cycle: z_V += W K^+ W^T (bscale .* r)_V, with K
// the Galerkin matrix W^T A_V W and K^+ its pseudo-inverse (the constant of every
// isolated conductor is a null mode and is dropped).
#define QMS_REGION_MAX 1024
struct QmsRegions {
    int K = 0;                    // regions carrying a coarse degree of freedom (0: disabled)
    int total_entries = 0;        // V rows in all regions
    int* ptr = nullptr;           // K+1 offsets into rows
    int* rows = nullptr;          // V rows (global unknown index) of each region, region by region
    int* rid = nullptr;           // region of each entry of rows
    double* Kp = nullptr;         // K x K pseudo-inverse, row-major
    double* s = nullptr;          // K region sums / coarse solution
    double* y = nullptr;
    std::string err;
    ~QmsRegions();
    void release();
    // slots: xs*ys*zs host material slots; rows6: per-slot mu_r xyz, sigma xyz (slot s at s-1)
    int build(const QGrid& g, const uint8_t* slots, const double* rows6, int nmat, double vshift, double cut,
              cudaStream_t st);
    // z_V += W K^+ W^T (bscale .* b)_V  (bscale may be null)
    template <typename T>
    void apply(const T* b, const float* bscale, T* z, cudaStream_t st, long long& launches);
};

