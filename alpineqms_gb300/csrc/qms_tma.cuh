// qms_tma.cuh -- the padded node layout of the inner solver's vectors and the TMA /
// mbarrier primitives (inline PTX) that stage its tiles in shared memory.
//
// Padded layout ("PL"): the four unknown blocks (Ax, Ay, Az, V) are stored as one 4-D
// array [4][Nz][Ny][P]: unknown (q, i, j, k) (1-based) at
//     q * comp + ((k - 1) * Ny + (j - 1)) * P + i,   comp = Nz * Ny * P,
// P = the node count along x rounded up to a multiple of 4 (16-byte rows).  Column 0,
// the columns past each block's own extent (Ax has xs = Nx - 1 columns), Ay's row Ny and
// Az's plane Nz are padding and stay zero.  The node coefficients use the same layout
// with six planes of arrays ([6][Nz][Ny][P]).  Every CTA tile of the stencil kernels then
// starts at column 32 bx, a 16-byte boundary, so one cp.async.bulk.tensor copies a whole
// plane of a tile (all components, +-1 halo) and zero-fills whatever lies outside.
#pragma once
#include <cuda.h>
#include <cstdint>

#include "qms_common.cuh"

struct QPL {
    int P;            // row pitch (elements)
    long long comp;   // elements per block
    long long n;      // total elements (4 blocks)
};

__host__ __device__ __forceinline__ QPL qms_pl(const QGrid& g) {
    QPL L;
    L.P = (g.Nx + 1 + 3) & ~3;
    L.comp = (long long)g.Nz * g.Ny * L.P;
    L.n = 4 * L.comp;
    return L;
}

// offset of node (i, j, k) within a block
__host__ __device__ __forceinline__ long long qms_pl_node(const QGrid& g, const QPL& L, int i, int j, int k) {
    return ((long long)(k - 1) * g.Ny + (j - 1)) * L.P + i;
}

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ unsigned qms_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(qms_smem(bar)), "r"(count) : "memory");
}

// makes the barrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// orders this thread's earlier generic-proxy accesses to shared memory before later
// async-proxy (TMA) writes to it
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(qms_smem(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(qms_smem(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `parity` to complete.  Every wait is bounded: try_wait suspends
// for a hardware time limit per call, and after QMS_MBAR_SPINS calls the wait gives up,
// flags QMS_ST_TIMEOUT in *err and returns false (the caller then stops using the tile).
#define QMS_MBAR_SPINS (1 << 22)
__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, unsigned parity, unsigned* err, int spins) {
    for (int it = 0; it < spins; it++)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicOr(err, (unsigned)QMS_ST_TIMEOUT);
    return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned* err) {
    return mbar_wait_n(bar, parity, err, QMS_MBAR_SPINS);
}

// one 4-D tiled bulk tensor copy global -> shared, completion counted on `bar`
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(qms_smem(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(qms_smem(bar))
        : "memory");
}

// ---------------------------------------------------------------- tiles
// A plane of the x tile: NQ blocks (all four, or a subset), rows j0-1 .. j0+8, columns
// i0-1 .. i0+34 (36 columns: the box width must be a multiple of 16 bytes); coefficient plane:
// NC arrays (all six, or the three conductivities), rows j0-1 .. j0+7.  Slots are padded to
// 128 bytes.
#define PLX 36
#define PLX16 40      // 2-byte elements: a row of the box must be a multiple of 16 bytes (80 B)
#define PLXY 10
#define PLCY 9
// CT: element type of the coefficient tiles (2-byte coefficients use PLX16 columns)
template <typename T, int NQ = 4, int NC = 6, typename CT = T>
struct PLTiles {
    static constexpr int CX = sizeof(CT) == 2 ? PLX16 : PLX;             // coefficient tile row width
    static constexpr int XSLOT_RAW = NQ * PLXY * PLX;                     // elements per x plane
    static constexpr int XSLOT = ((XSLOT_RAW * (int)sizeof(T) + 127) / 128) * 128 / (int)sizeof(T);
    static constexpr int CSLOT_RAW = NC * PLCY * CX;
    static constexpr int CSLOT = ((CSLOT_RAW * (int)sizeof(CT) + 127) / 128) * 128 / (int)sizeof(CT);
    static constexpr unsigned XBYTES = XSLOT_RAW * sizeof(T);
    static constexpr unsigned CBYTES = CSLOT_RAW * sizeof(CT);
    static constexpr size_t SMEM = (size_t)4 * XSLOT * sizeof(T) + (size_t)3 * CSLOT * sizeof(CT);
};

// the 2-byte copy of the node coefficients: the same [6][Nz][Ny][P16] order with rows of
// P16 = Nx + 1 rounded up to a multiple of 8 (16-byte rows for a tensor map)
__host__ __device__ __forceinline__ int qms_pl16_pitch(const QGrid& g) { return (g.Nx + 1 + 7) & ~7; }

// host: tensor maps of a padded vector (4 blocks) and of the padded node coefficients (6 arrays)
bool qms_make_pl_map(CUtensorMap* map, const void* base, const QGrid& g, int elem_bytes, int arrays, int box_rows);
// ... and of the bf16 copy of the node coefficients (`arrays` of them from base, PLX16 x PLCY boxes)
bool qms_make_pl16_map(CUtensorMap* map, const void* base, const QGrid& g, int arrays);
