// Pressure-form projection: right-hand side, red-black SOR sweeps on P (one colour pass per
// launch; the temporally blocked kernel is kernels_sweep_tb.cu), the tolerance check, and the
// gradient subtract.
//
// The reference projects in velocity space (project/smokeSimulation.cu:356-394): every colour
// pass reads and rewrites all six faces of each cell (~25 B/cell/pass).  Accumulating its
// per-cell corrections p_t into a cell pressure P gives the identical iteration in exact
// arithmetic -- SOR on  acc_c*P_c - sum_{fluid nbrs} P_n = -div(u*)_c  -- whose passes touch
// only P, b and one flag byte, and one gradient subtract u -= grad P on faces whose two cells
// are fluid replaces the per-pass face updates.  Bodies: stage_bodies.cuh.
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "stage_bodies.cuh"

namespace smk {

namespace {

constexpr int BX = SB_BX, BY = SB_BY;

inline dim3 grid3(int rx, int ry, int rz) {
    return dim3((unsigned)((rx + BX - 1) / BX), (unsigned)((ry + BY - 1) / BY), (unsigned)rz);
}

template <typename T>
__global__ void k_rhs(Grid g, const T* __restrict__ u, const T* __restrict__ v,
                      const T* __restrict__ w, const uint8_t* __restrict__ flags,
                      float* __restrict__ b, float* __restrict__ P, const float* __restrict__ P2,
                      const int* __restrict__ pcur, int warm, float* __restrict__ Ph, float alpha) {
    body_rhs(g, u, v, w, flags, b, P, P2, pcur, warm, blockIdx, Ph, alpha);
}

// rhs with four consecutive x per thread (vector loads and stores; body_rhs_x4).
template <typename T>
__global__ void __launch_bounds__(256) k_rhs_x4(Grid g, const T* __restrict__ u, const T* __restrict__ v,
                                                const T* __restrict__ w, const uint8_t* __restrict__ flags,
                                                float* __restrict__ b, float* __restrict__ P,
                                                const float* __restrict__ P2, const int* __restrict__ pcur,
                                                int warm, float* __restrict__ Ph, float alpha) {
    body_rhs_x4(g, u, v, w, flags, b, P, P2, pcur, warm, 4 * ((int)blockIdx.x * 32 + (int)threadIdx.x),
                (int)blockIdx.y * 8 + (int)threadIdx.y, (int)blockIdx.z, Ph, alpha);
}

// FP32 gradient subtract with four consecutive x per thread (body_gradient_subtract_x4).
__global__ void __launch_bounds__(256) k_gradient_subtract_x4(Grid g, float* __restrict__ u, float* __restrict__ v,
                                                              float* __restrict__ w, const float* __restrict__ P0,
                                                              const float* __restrict__ P1,
                                                              const int* __restrict__ pcur,
                                                              const uint8_t* __restrict__ flags,
                                                              const int* __restrict__ skip) {
    if (skip != nullptr && *skip) return;
    const float* P = (pcur != nullptr && *pcur == 1) ? P1 : P0;
    body_gradient_subtract_x4(g, u, v, w, P, flags, 4 * ((int)blockIdx.x * 32 + (int)threadIdx.x),
                              1 + (int)blockIdx.y * 8 + (int)threadIdx.y, 1 + (int)blockIdx.z);
}

__global__ void k_gradient_subtract(Grid g, float* __restrict__ u, float* __restrict__ v,
                                    float* __restrict__ w, const float* __restrict__ P0,
                                    const float* __restrict__ P1, const int* __restrict__ pcur,
                                    const uint8_t* __restrict__ flags, const int* __restrict__ skip) {
    if (skip != nullptr && *skip) return;
    body_gradient_subtract(g, u, v, w, P0, P1, pcur, flags, blockIdx);
}

__global__ void k_sweep(Grid g, float* __restrict__ P, const float* __restrict__ b,
                        const uint8_t* __restrict__ flags, int colour, WAcc wa,
                        const StepStatus* __restrict__ status) {
    body_sweep(g, P, b, flags, colour, wa, status, blockIdx);
}

// Weighted Jacobi: every projectable interior cell from the previous iterate Pin, into Pout, with
// the colour pass's expressions (cell_sweep); other interior cells get 0, as P holds there.
// Skipped once the tolerance rule has ended the solve; the first thread records which buffer
// the launch wrote.
__global__ void k_jacobi(Grid g, const float* __restrict__ Pin, float* __restrict__ Pout,
                         const float* __restrict__ b, const uint8_t* __restrict__ flags, WAcc wa,
                         const StepStatus* __restrict__ status, int* __restrict__ pcur, int out_idx) {
    if (status && *(volatile const int*)&status->done) return;
    if (pcur && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        *pcur = out_idx;
    const int x = 1 + (int)blockIdx.x * BX + (int)threadIdx.x;
    const int y = 1 + (int)blockIdx.y * BY + (int)threadIdx.y;
    const int z = 1 + (int)blockIdx.z;
    if (x > g.nx - 2 || y > g.ny - 2) return;
    const int i = g.idx(x, y, z);
    const uint8_t f = flags[i];
    if (!(f & F_PROJ)) {
        Pout[i] = 0.0f;
        return;
    }
    const int acc = __popc((unsigned)(f & F_NBRS));
    const float sum = ((Pin[i - 1] + Pin[i + 1]) + (Pin[i - g.X] + Pin[i + g.X])) + (Pin[i - g.XY] + Pin[i + g.XY]);
    const float pc = Pin[i];
    const float r = fmaf(-(float)acc, pc, b[i] + sum);
    Pout[i] = fmaf(wa.w[acc], r, pc);
}

__global__ void k_resid_check(Grid g, const float* __restrict__ P, const float* __restrict__ b,
                              const uint8_t* __restrict__ flags, StepStatus* status, int group,
                              float tol) {
    body_resid_check(g, P, b, flags, status, group, tol, blockIdx, gridDim.x * gridDim.y * gridDim.z);
}


}  // namespace

template <typename T>
void launch_rhs(const Grid& g, const T* u, const T* v, const T* w, const uint8_t* flags,
                float* b, float* P, const float* P2, const int* pcur, int warm, cudaStream_t st, bool vec,
                float* Ph, float alpha) {
    if (vec && vec4_layout_of<T>(g, {u, v, w}, {b, P, P2, Ph}, flags)) {
        const int groups = (g.nx + 3) / 4;
        k_rhs_x4<T><<<dim3((unsigned)((groups + 31) / 32), (unsigned)((g.ny + 7) / 8), (unsigned)g.nz), dim3(32, 8),
                      0, st>>>(g, u, v, w, flags, b, P, P2, pcur, warm, Ph, alpha);
        return;
    }
    k_rhs<<<grid3(g.nx, g.ny, g.nz), dim3(BX, BY), 0, st>>>(g, u, v, w, flags, b, P, P2, pcur, warm, Ph, alpha);
}
template void launch_rhs<float>(const Grid&, const float*, const float*, const float*, const uint8_t*, float*,
                                float*, const float*, const int*, int, cudaStream_t, bool, float*, float);
template void launch_rhs<__nv_bfloat16>(const Grid&, const __nv_bfloat16*, const __nv_bfloat16*,
                                        const __nv_bfloat16*, const uint8_t*, float*, float*, const float*,
                                        const int*, int, cudaStream_t, bool, float*, float);

void launch_sweep(const Grid& g, float* P, const float* b, const uint8_t* flags, int colour,
                  const float* wacc7, const StepStatus* status, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    WAcc wa;
    for (int k = 0; k < 7; ++k) wa.w[k] = wacc7[k];
    wa.w[7] = 0.0f;
    int half = (g.nx - 2 + 1) / 2;
    k_sweep<<<grid3(half, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, P, b, flags, colour, wa,
                                                                      status);
}

void launch_jacobi(const Grid& g, const float* Pin, float* Pout, const float* b, const uint8_t* flags,
                   const float* wacc7, const StepStatus* status, int* pcur, int out_idx, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    WAcc wa;
    for (int k = 0; k < 7; ++k) wa.w[k] = wacc7[k];
    wa.w[7] = 0.0f;
    k_jacobi<<<grid3(g.nx - 2, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, Pin, Pout, b, flags, wa, status, pcur,
                                                                           out_idx);
}

void launch_resid_check(const Grid& g, const float* P, const float* b, const uint8_t* flags,
                        StepStatus* status, int group, float tol, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    k_resid_check<<<grid3(g.nx - 2, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, P, b, flags, status,
                                                                               group, tol);
}

void launch_gradient_subtract(const Grid& g, float* u, float* v, float* w, const float* P0,
                              const float* P1, const int* pcur, const uint8_t* flags,
                              cudaStream_t st, bool vec, const int* skip) {
    if (g.nx < 2 || g.ny < 2 || g.nz < 2) return;
    if (!vec || !vec4_layout(g, {u, v, w, P0, P1}, flags)) {
        k_gradient_subtract<<<grid3(g.nx - 1, g.ny - 1, g.nz - 1), dim3(BX, BY), 0, st>>>(
            g, u, v, w, P0, P1, pcur, flags, skip);
        return;
    }
    const int groups = (g.nx + 3) / 4;  // x in [1, nx): groups of 4 from x = 0
    k_gradient_subtract_x4<<<dim3((unsigned)((groups + 31) / 32), (unsigned)((g.ny - 1 + 7) / 8), (unsigned)(g.nz - 1)),
                             dim3(32, 8), 0, st>>>(g, u, v, w, P0, P1, pcur, flags, skip);
}

}  // namespace smk

// ---- FP64-checked refinement of the projection ----------------------------------------------
//
// After the FP32 solve and gradient subtract, the divergence of the projected velocity is
// measured with FP64 accumulation: d = ((((-u0 + u1) + -v0) + v1) + -w0) + w1 over the six FP32
// face values in double.  While some projectable cell has |d| > tol, a correction round solves
// A e = b' with b' = (float)(-d) from e = 0 (the same FP32 red-black passes, a fixed number of
// sweeps), subtracts grad e from the velocity on fluid-fluid faces (the gradient subtract's rule)
// and adds e to the pressure, so the next warm start keeps the correction.  e lives in the
// pressure buffer that does not hold the solution (*pcur selects).  Every kernel returns at
// entry once a measurement was within tolerance.

namespace smk {
namespace {

__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v) {
    __shared__ unsigned long long red[32];
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nw = (blockDim.x * blockDim.y + 31) >> 5;
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    unsigned long long m = 0ull;
    if (tid == 0)
        for (int k = 0; k < nw; ++k) m = red[k] > m ? red[k] : m;
    return m;  // valid in thread 0
}

__global__ void k_refine_reset(RefineStatus* rs, int start) {
    if (start) {
        rs->rounds = 0;
        rs->stop = 0;
    }
    if (!rs->stop) {
        rs->div_bits = 0ull;
        rs->need = 0;
    }
}

// The refinement kernels are persistent: a fixed grid (a few CTAs per SM) walks the stage's
// 64 x 4 blocks, so a round that is not needed costs only that grid's exit, not a full-size launch.
__device__ __forceinline__ uint3 vblock(int vb, int nbx, int nby) {
    uint3 b;
    b.x = (unsigned)(vb % nbx);
    b.y = (unsigned)((vb / nbx) % nby);
    b.z = (unsigned)(vb / (nbx * nby));
    return b;
}

// FP64 |div u| per projectable cell (read only): the max (as IEEE bits) and whether any cell
// exceeds tol.
__global__ void k_refine_measure(Grid g, const float* u, const float* v, const float* w,
                                 const uint8_t* __restrict__ flags, RefineStatus* rs, double tol, int nbx,
                                 int nby, int nvb) {
    if (*(volatile int*)&rs->stop) return;
    double m = 0.0;
    for (int vb = (int)blockIdx.x; vb < nvb; vb += (int)gridDim.x) {
        const uint3 bid = vblock(vb, nbx, nby);
        const int x = (int)bid.x * BX + (int)threadIdx.x;
        const int y = (int)bid.y * BY + (int)threadIdx.y;
        const int z = (int)bid.z;
        if (x < g.nx && y < g.ny && z < g.nz) {
            const int i = g.idx(x, y, z);
            if (flags[i] & F_PROJ) {
                const double d = ((((-(double)u[i] + (double)u[i + 1]) + -(double)v[i]) + (double)v[i + g.X]) +
                                  -(double)w[i]) + (double)w[i + g.XY];
                const double a = fabs(d);
                if (!(a <= m)) m = a;  // NaN propagates as the largest value
            }
        }
    }
    // one flag store and at most one atomic per CTA, each only when it changes the stored value
    const int any = __syncthreads_or(m > tol);
    const unsigned long long bm = block_max_u64((unsigned long long)__double_as_longlong(m));
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        if (any && *(volatile int*)&rs->need == 0) rs->need = 1;
        if (bm > *(volatile unsigned long long*)&rs->div_bits) atomicMax(&rs->div_bits, bm);
    }
}

// A round that is needed: b = (float)(-d) (0 off the projectable set) and e = 0 over every cell.
__global__ void k_refine_prepare(Grid g, const float* u, const float* v, const float* w,
                                 const uint8_t* __restrict__ flags, float* b, float* P0, float* P1,
                                 const int* pcur, const RefineStatus* rs, int nbx, int nby, int nvb) {
    if (*(volatile const int*)&rs->stop) return;
    float* e = (*pcur == 1) ? P0 : P1;
    for (int vb = (int)blockIdx.x; vb < nvb; vb += (int)gridDim.x) {
        const uint3 bid = vblock(vb, nbx, nby);
        const int x = (int)bid.x * BX + (int)threadIdx.x;
        const int y = (int)bid.y * BY + (int)threadIdx.y;
        const int z = (int)bid.z;
        if (x >= g.nx || y >= g.ny || z >= g.nz) continue;
        const int i = g.idx(x, y, z);
        if (flags[i] & F_PROJ) {
            const double d = ((((-(double)u[i] + (double)u[i + 1]) + -(double)v[i]) + (double)v[i + g.X]) +
                              -(double)w[i]) + (double)w[i + g.XY];
            b[i] = (float)(-d);
        } else {
            b[i] = 0.0f;
        }
        e[i] = 0.0f;
    }
}

__global__ void k_refine_decide(RefineStatus* rs) {
    if (!rs->stop && !rs->need) rs->stop = 1;
}

__global__ void k_refine_sweep(Grid g, float* P0, float* P1, const int* pcur, const float* b,
                               const uint8_t* __restrict__ flags, int colour, WAcc wa,
                               const RefineStatus* rs, int nbx, int nby, int nvb) {
    if (*(volatile const int*)&rs->stop) return;
    float* e = (*pcur == 1) ? P0 : P1;
    for (int vb = (int)blockIdx.x; vb < nvb; vb += (int)gridDim.x)
        body_sweep(g, e, b, flags, colour, wa, nullptr, vblock(vb, nbx, nby));
}

template <typename Tv>
__global__ void k_refine_apply(Grid g, float* u, float* v, float* w, Tv* us, Tv* vs, Tv* ws, float* P0,
                               float* P1, const int* pcur, const uint8_t* __restrict__ flags,
                               RefineStatus* rs, int nbx, int nby, int nvb) {
    if (*(volatile int*)&rs->stop) return;
    const bool second = *pcur == 1;
    float* Pc = second ? P1 : P0;
    const float* e = second ? P0 : P1;
    if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) rs->rounds += 1;
    for (int vb = (int)blockIdx.x; vb < nvb; vb += (int)gridDim.x) {
        const uint3 bid = vblock(vb, nbx, nby);
        const int x = 1 + (int)bid.x * BX + (int)threadIdx.x;
        const int y = 1 + (int)bid.y * BY + (int)threadIdx.y;
        const int z = 1 + (int)bid.z;
        if (x >= g.nx || y >= g.ny || z >= g.nz) continue;
        const int i = g.idx(x, y, z);
        const uint8_t f = flags[i];
        if (!(f & F_SELF)) continue;
        const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2, inz = z <= g.nz - 2;
        const float ec = e[i];
        if (iny && inz && (f & F_XM)) {
            u[i] = u[i] - (ec - e[i - 1]);
            if (us) stv(us, i, u[i]);
        }
        if (inx && inz && (f & F_YM)) {
            v[i] = v[i] - (ec - e[i - g.X]);
            if (vs) stv(vs, i, v[i]);
        }
        if (inx && iny && (f & F_ZM)) {
            w[i] = w[i] - (ec - e[i - g.XY]);
            if (ws) stv(ws, i, w[i]);
        }
        if (inx && iny && inz) Pc[i] = Pc[i] + ec;
    }
}

int refine_ctas() {
    static int ctas = 0;
    if (ctas == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        ctas = (sms > 0 ? sms : 132) * 8;
    }
    return ctas;
}

}  // namespace

template <typename Tv>
void launch_refine(const Grid& g, float* u, float* v, float* w, Tv* us, Tv* vs, Tv* ws, float* b, float* P0,
                   float* P1, const int* pcur, const uint8_t* flags, const float* wacc7, int rounds,
                   int sweeps, double tol, RefineStatus* rs, long long* launches, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    WAcc wa;
    for (int k = 0; k < 7; ++k) wa.w[k] = wacc7[k];
    wa.w[7] = 0.0f;
    const dim3 blk(BX, BY);
    const int ctas = refine_ctas();
    auto grid_of = [ctas](int nvb) { return dim3((unsigned)(nvb < ctas ? nvb : ctas)); };
    // block ranges of the single-grid launches of each stage
    const dim3 cells = grid3(g.nx, g.ny, g.nz);
    const int cbx = (int)cells.x, cby = (int)cells.y, cnv = cbx * cby * (int)cells.z;
    const int half = (g.nx - 2 + 1) / 2;
    const dim3 sw = grid3(half, g.ny - 2, g.nz - 2);
    const int sbx = (int)sw.x, sby = (int)sw.y, snv = sbx * sby * (int)sw.z;
    const dim3 fc = grid3(g.nx - 1, g.ny - 1, g.nz - 1);
    const int fbx = (int)fc.x, fby = (int)fc.y, fnv = fbx * fby * (int)fc.z;
    k_refine_reset<<<1, 1, 0, st>>>(rs, 1);
    k_refine_measure<<<grid_of(cnv), blk, 0, st>>>(g, u, v, w, flags, rs, tol, cbx, cby, cnv);
    k_refine_decide<<<1, 1, 0, st>>>(rs);
    *launches += 3;
    for (int r = 0; r < rounds; ++r) {
        k_refine_prepare<<<grid_of(cnv), blk, 0, st>>>(g, u, v, w, flags, b, P0, P1, pcur, rs, cbx, cby, cnv);
        for (int s = 0; s < sweeps; ++s)
            for (int colour = 0; colour < 2; ++colour)
                k_refine_sweep<<<grid_of(snv), blk, 0, st>>>(g, P0, P1, pcur, b, flags, colour, wa, rs, sbx, sby, snv);
        k_refine_apply<Tv><<<grid_of(fnv), blk, 0, st>>>(g, u, v, w, us, vs, ws, P0, P1, pcur, flags, rs, fbx, fby,
                                                         fnv);
        k_refine_reset<<<1, 1, 0, st>>>(rs, 0);
        k_refine_measure<<<grid_of(cnv), blk, 0, st>>>(g, u, v, w, flags, rs, tol, cbx, cby, cnv);
        k_refine_decide<<<1, 1, 0, st>>>(rs);
        *launches += 2 * sweeps + 5;
    }
}
template void launch_refine<float>(const Grid&, float*, float*, float*, float*, float*, float*, float*, float*,
                                   float*, const int*, const uint8_t*, const float*, int, int, double,
                                   RefineStatus*, long long*, cudaStream_t);
template void launch_refine<__nv_bfloat16>(const Grid&, float*, float*, float*, __nv_bfloat16*, __nv_bfloat16*,
                                           __nv_bfloat16*, float*, float*, float*, const int*, const uint8_t*,
                                           const float*, int, int, double, RefineStatus*, long long*,
                                           cudaStream_t);

}  // namespace smk
