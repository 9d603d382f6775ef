// qms_noalloc.cu -- residual of the A-V system for callers that cannot allocate.
//
// Who needs it: code that runs where device allocation is unavailable or
// forbidden -- an allocator-free real-time loop, or a host process whose GPU
// memory is owned by another runtime (a framework memory pool) that does not
// let libraries call cudaMalloc.  Such a caller already owns its vectors and
// wants to check a solution without creating a qms_handle (whose creation
// allocates the solver workspace).  The call synchronises its stream before it
// returns, so it cannot be recorded into a CUDA graph: a caller must not make
// it while that stream is being captured.
//
// qms_residual_noalloc computes r = D^-1 (b - M x) and the block sums
// |r_A|^2, |r_V|^2, |x_A|^2, |x_V|^2 with the same FP64 matrix-free kernel as
// qms_residual_norm.  Its scratch (per-CTA partial sums and the per-slot
// material table) lives in file-scope __device__ arrays of fixed size instead
// of device allocations.
#include "qms.h"
#include "qms_internal.h"

#include <cmath>
#include <mutex>

// Scratch: at most QMS_NOALLOC_MAX_BLOCKS operator CTAs (tiles of 32 x 8 x 16
// nodes; 512 x 512 x 256 cells needs 18,785), four partial sums each, plus one
// material table.  Every GPU that loads the library holds these ~1.1 MB until
// the process exits.
#define QMS_NOALLOC_MAX_BLOCKS 32768
static __device__ __align__(256) double g_na_partials[4 * QMS_NOALLOC_MAX_BLOCKS];
static __device__ __align__(256) QMatTable<double> g_na_table;

namespace {

// One per device: the scratch arrays are per-device instances, so only calls on the same
// device share them and are serialised by its mutex.
struct DevScratch {
    std::mutex mu;
    bool ready = false;
    double* partials = nullptr;
    QMatTable<double>* table = nullptr;
    QMatTable<double> host_table;      // staging copy of the last table uploaded on this device
};

DevScratch g_na_dev[64];

__global__ void na_finalize(const double* __restrict__ part, long long nb, double* __restrict__ sums) {
    __shared__ double sh[32];
    for (int q = 0; q < 4; q++) {
        double acc = 0.0;
        for (long long t = threadIdx.x; t < nb; t += blockDim.x) acc += part[q * nb + t];
        double s = qBlockSum(acc, sh);
        if (threadIdx.x == 0) sums[q] = s;
    }
}

}  // namespace

extern "C" int qms_residual_noalloc_fits(int xs, int ys, int zs) {
    if (xs < 4 || ys < 4 || zs < 4) return 0;
    return qms_op_num_blocks(qms_make_grid(xs, ys, zs, 1.0, 1.0, 1.0)) <= QMS_NOALLOC_MAX_BLOCKS ? 1 : 0;
}

extern "C" int qms_residual_noalloc(int xs, int ys, int zs, double dx, double dy, double dz, double dt,
                                    int transient, const double v[3], const uint8_t* d_slots, const double* rows,
                                    int nmat, const double* d_x, const double* d_b, double* d_r, double* d_sums,
                                    void* stream) {
    if (xs < 4 || ys < 4 || zs < 4 || !(dx > 0 && dy > 0 && dz > 0 && dt > 0) || !v || !d_slots ||
        (nmat > 0 && !rows) || nmat < 0 || nmat > QMS_MAX_SLOTS - 1 || !d_x || !d_b || !d_r || !d_sums)
        return QMS_ERR_ARG;
    const QGrid g = qms_make_grid(xs, ys, zs, dx, dy, dz);
    const long long nb = qms_op_num_blocks(g);
    if (nb > QMS_NOALLOC_MAX_BLOCKS) return QMS_ERR_ARG;      // grid above the fixed scratch size
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return QMS_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    // an error the caller has not collected yet stays theirs: refuse to run rather than clear it
    if (cudaPeekAtLastError() != cudaSuccess) return QMS_ERR_CUDA;
    DevScratch& S = g_na_dev[dev];
    std::lock_guard<std::mutex> lk(S.mu);
    if (!S.ready) {
        // Host code cannot use the arrays' names as device addresses: resolve them once per
        // device, with that device current.  This first call must not be inside a stream capture.
        if (cudaGetSymbolAddress((void**)&S.partials, g_na_partials) != cudaSuccess) return QMS_ERR_CUDA;
        if (cudaGetSymbolAddress((void**)&S.table, g_na_table) != cudaSuccess) return QMS_ERR_CUDA;
        S.ready = true;
    }
    qms_fill_table(S.host_table, rows, nmat);
    if (cudaMemcpyAsync(S.table, &S.host_table, sizeof(S.host_table), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return QMS_ERR_CUDA;
    const bool adv = v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0;
    const QStepPar<double> P = qms_step_par<double>(g, v[0], v[1], v[2], dt, transient != 0);
    const QCoef<double> c{g, d_slots, S.table, 1.0 / QMS_MU0};
    qms_launch_operator<double>(g, c, P, adv, QOPH_RESID, d_x, d_b, d_r, nullptr, S.partials, st);
    na_finalize<<<1, 512, 0, st>>>(S.partials, nb, d_sums);
    // no error was pending before the launches (checked above): this one is theirs
    if (cudaGetLastError() != cudaSuccess) return QMS_ERR_CUDA;
    // the staging table is reused by the next call on this device
    if (cudaStreamSynchronize(st) != cudaSuccess) return QMS_ERR_CUDA;
    return 0;
}
