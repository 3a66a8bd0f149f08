// Shared pieces of the temporally blocked sweep kernels (kernels_sweep_tb.cu: the pressure
// form; kernels_vsweep_tb.cu: the reference scheme's in-place velocity form): TMA box loads of
// one plane into a shared-memory ring with mbarrier completion, bounded waits, and the placement
// of the x-y windows a CTA owns.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace smk {
namespace tb {

constexpr int TX = 32;                // threads per tile row (one warp) = 64 cells
constexpr int BOX_F = 68;             // float box width: 64 cells + up to 2 alignment cells, 16-B multiple
constexpr int BOX_U8 = 80;            // flag box width in bytes: 64 + up to 15 alignment bytes
constexpr unsigned WAIT_LIMIT = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned i = 0; i < WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// 4-byte asynchronous copy global -> shared (no register holds the value); completion by
// cp_async_commit / cp_async_wait_all of the issuing thread.
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// every committed group but the most recent one has completed
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Windows along an axis of n cells, W cells wide with a T-cell halo.  A side of a window that
// reaches the grid's first or last cell needs no halo: those cells (the boundary ring) and every
// cell outside the grid are never updated by a sweep, so they never change, and a wrong value
// beyond the window (a zero padding row, a shuffle that wrapped) only ever enters their own
// update, which keeps their value.  So in the edge placement the first window starts at cell 0
// and owns W - T cells, the middle ones start T cells before the cells they own and own W - 2T,
// and the last owns the rest (at most W - T, its window reaching the last cell); one window owns
// everything when n <= W.  The plain placement gives every window a halo on both sides (window k
// starts at k(W - 2T) - T).  The edge placement is used only where it needs fewer windows (small
// grids): at equal counts the plain one measured faster (256^3: 136.7 against 139.7 us a launch).
__host__ __device__ inline int edge_windows(int n, int W, int T) {
    if (n <= W) return 1;
    const int rest = n - 2 * (W - T);
    return 2 + (rest > 0 ? (rest + W - 2 * T - 1) / (W - 2 * T) : 0);
}
__host__ __device__ inline int plain_windows(int n, int W, int T) { return (n + W - 2 * T - 1) / (W - 2 * T); }
__host__ __device__ inline int sweep_windows(int n, int W, int T) {
    const int e = edge_windows(n, W, T), p = plain_windows(n, W, T);
    return e < p ? e : p;
}
// Window k of sweep_windows(n, W, T): its first cell (even for even T) and the cells [lo, hi) it owns.
__host__ __device__ inline void sweep_window(int n, int W, int T, int k, int& start, int& lo, int& hi) {
    const int nw = sweep_windows(n, W, T);
    if (edge_windows(n, W, T) < plain_windows(n, W, T)) {
        lo = k == 0 ? 0 : (W - T) + (k - 1) * (W - 2 * T);
        hi = k + 1 < nw ? (W - T) + k * (W - 2 * T) : n;
        start = k == 0 ? 0 : lo - T;
    } else {
        lo = k * (W - 2 * T);
        hi = k + 1 < nw ? lo + (W - 2 * T) : n;
        start = lo - T;
    }
}

// Host: a 3-D tiled TMA tensor map over one field of grid g (X x (ny+1) x (nz+1) elements, 4-byte
// floats or bytes), boxes of BOX_F (BOX_U8) x rows x 1; false when the base is null or not
// 16-byte aligned or cuTensorMapEncodeTiled refuses the map.  Defined in kernels_sweep_tb.cu.
bool encode_3d(CUtensorMap* m, const void* base, bool is_u8, const Grid& g, int rows);
// The same with a box box_w elements wide (box_w x element size a multiple of 16 bytes).
bool encode_3d_box(CUtensorMap* m, const void* base, bool is_u8, const Grid& g, int box_w, int rows);

}  // namespace tb
}  // namespace smk
