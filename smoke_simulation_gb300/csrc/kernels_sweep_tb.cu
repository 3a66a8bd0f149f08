// Temporally blocked red-black SOR sweeps on the cell pressure (the projection's hot loop).
//
// One launch applies `nhalf` <= T half-sweeps (colour passes) to P in a single pass over HBM:
// read P_in, b and the flag byte once, write P_out once -- 13 bytes per cell for T/2 sweeps,
// where one colour pass per launch would move ~9-11 bytes per pass.
//
// Decomposition.  A CTA owns an x-y tile of 64 x 32 columns (T-cell halo on each side, so the
// interior is (64-2T) x (32-2T)) and a z-range [za, zb) of output planes.  It marches z as a
// wavefront: at iteration q it loads plane q, computes the residual of plane q-1 (time 0, for
// the tolerance check) and brings plane q-1-t from time t-1 to time t for t = 1..T, so plane
// q-1-T leaves the pipeline finished.  Colour-t cells of a plane read only opposite-colour
// neighbours, whose values at time t-1 are what the neighbouring planes hold at that moment,
// so one copy of each plane suffices.  Halo cells are recomputed redundantly; cells within
// T - t of the interior are exact after half-sweep t, which is all the interior needs.
//
// Storage per thread (2 x-adjacent columns): the z-ring of P, b and flags in registers.
// Neighbours: z from registers, x from the thread's own pair or a warp shuffle (a tile row is
// one warp), y from a shared-memory copy of the plane published once per iteration
// (double-buffered, one barrier per iteration).
//
// Every update is  r = fma(-acc, P_c, b_c + (((((P_x- + P_x+) + P_y-) + P_y+) + P_z-) + P_z+));
// P_c = fma(omega/acc, r, P_c), the oracle's order, so results equal the one-pass-per-colour
// kernel bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"

namespace smk {

namespace {

constexpr int TB_TX = 32;            // threads per tile row (one warp)
constexpr int TB_TY = 32;            // tile rows
constexpr int TB_CX = 2 * TB_TX;     // columns per tile row (2 per thread)

struct WAcc8 { float w[8]; };

__device__ __forceinline__ float2 ld2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }

template <int T>
__global__ void __launch_bounds__(TB_TX * TB_TY, 1)
k_sweep_tb(Grid g, const float* __restrict__ Pin, float* __restrict__ Pout,
           const float* __restrict__ B, const uint8_t* __restrict__ F, int nhalf, int colour0,
           int zchunk, WAcc8 wa, StepStatus* status, int check, int group, float tol,
           int* __restrict__ pcur, int out_idx) {
    extern __shared__ float2 smem_tb[];
    __shared__ float wacc[8];

    if (status != nullptr) {
        if (*(volatile int*)&status->done) return;
        if (check && group > 0 && __uint_as_float(status->rmax_bits[group - 1]) <= tol) {
            if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 &&
                threadIdx.y == 0) {
                status->done = 1;
                status->done_group = group;
            }
            return;
        }
    }
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (ty == 0 && tx < 8) wacc[tx] = wa.w[tx];
    if (pcur != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tx == 0 && ty == 0)
        *pcur = out_idx;

    constexpr int IX = TB_CX - 2 * T, IY = TB_TY - 2 * T;
    const int xA = (int)blockIdx.x * IX - T + 2 * tx;  // even
    const int y = (int)blockIdx.y * IY - T + ty;
    const int za = (int)blockIdx.z * zchunk;
    const int zb = min(za + zchunk, g.nz);
    const bool colok = xA >= 0 && xA < g.X && y >= 0 && y <= g.ny;
    const bool interior = (2 * tx >= T) && (2 * tx < T + IX) && (ty >= T) && (ty < T + IY) &&
                          xA < g.nx && y < g.ny && y >= 0 && xA >= 0;
    const int rowoff = xA + g.X * y;

    // z-rings: index j holds plane q - j
    float2 p[T + 3];
    float2 bb[T + 2];
    unsigned ff[T + 2];
#pragma unroll
    for (int j = 0; j < T + 3; ++j) p[j] = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < T + 2; ++j) { bb[j] = make_float2(0.f, 0.f); ff[j] = 0u; }

    unsigned rmax = 0u;
    int par = 0;
    const int qbeg = za - T;
    const int qlast_load = min(zb - 1 + T, g.nz);
    const int qend = zb + T;

    // prefetch registers for the next plane
    float2 np_ = make_float2(0.f, 0.f), nb_ = make_float2(0.f, 0.f);
    unsigned nf_ = 0u;
    if (colok && qbeg >= 0 && qbeg <= qlast_load) {
        const int i = rowoff + g.XY * qbeg;
        np_ = ld2(Pin + i);
        nb_ = ld2(B + i);
        nf_ = __ldg(reinterpret_cast<const unsigned short*>(F + i));
    }
    __syncthreads();  // wacc visible

    for (int q = qbeg; q <= qend; ++q) {
#pragma unroll
        for (int j = T + 2; j > 0; --j) p[j] = p[j - 1];
#pragma unroll
        for (int j = T + 1; j > 0; --j) { bb[j] = bb[j - 1]; ff[j] = ff[j - 1]; }
        p[0] = np_;
        bb[0] = nb_;
        ff[0] = nf_;
        // issue the next plane's loads now; they complete while this plane computes
        np_ = make_float2(0.f, 0.f);
        nb_ = make_float2(0.f, 0.f);
        nf_ = 0u;
        const int qn = q + 1;
        if (colok && qn >= 0 && qn <= qlast_load) {
            const int i = rowoff + g.XY * qn;
            np_ = ld2(Pin + i);
            nb_ = ld2(B + i);
            nf_ = __ldg(reinterpret_cast<const unsigned short*>(F + i));
        }

        // publish planes q-1-s (s = 0..T) at their current time for the y-neighbours
        float2* buf = smem_tb + par * (T + 1) * TB_TY * TB_TX;
#pragma unroll
        for (int s = 0; s <= T; ++s) buf[(s * TB_TY + ty) * TB_TX + tx] = p[1 + s];
        __syncthreads();

        // stage 0: residual of plane q-1 at time 0 (tolerance check launches only)
        if (check) {
            const int zp = q - 1;
            const float2 cur = p[1];
            const float left = __shfl_up_sync(0xffffffffu, cur.y, 1);
            const float right = __shfl_down_sync(0xffffffffu, cur.x, 1);
            if (interior && zp >= za && zp < zb) {
                const float2 ym = buf[(0 * TB_TY + ty - 1) * TB_TX + tx];
                const float2 yp = buf[(0 * TB_TY + ty + 1) * TB_TX + tx];
                const float2 up = p[0], dn = p[2];
                const unsigned f2 = ff[1];
                const unsigned fa = f2 & 0xffu, fb = (f2 >> 8) & 0xffu;
                if (fa & F_PROJ) {
                    const int acc = __popc(fa & F_NBRS);
                    const float sum = left + cur.y + ym.x + yp.x + dn.x + up.x;
                    const float r = fmaf(-(float)acc, cur.x, bb[1].x + sum);
                    rmax = max(rmax, __float_as_uint(fabsf(r)));
                }
                if (fb & F_PROJ) {
                    const int acc = __popc(fb & F_NBRS);
                    const float sum = cur.x + right + ym.y + yp.y + dn.y + up.y;
                    const float r = fmaf(-(float)acc, cur.y, bb[1].y + sum);
                    rmax = max(rmax, __float_as_uint(fabsf(r)));
                }
            }
        }

        // stages 1..T: plane q-1-t from time t-1 to t (colour c_t cells)
#pragma unroll
        for (int t = 1; t <= T; ++t) {
            if (t <= nhalf) {
                const int zp = q - 1 - t;
                const int ct = colour0 ^ ((t - 1) & 1);
                const bool updA = ((y + zp) & 1) == ct;  // cell A (even x) has colour (y+zp)&1
                const float2 cur = p[1 + t];
                const float left = __shfl_up_sync(0xffffffffu, cur.y, 1);
                const float right = __shfl_down_sync(0xffffffffu, cur.x, 1);
                const float2 ym = ty > 0 ? buf[(t * TB_TY + ty - 1) * TB_TX + tx] : make_float2(0.f, 0.f);
                const float2 yp = ty < TB_TY - 1 ? buf[(t * TB_TY + ty + 1) * TB_TX + tx]
                                                 : make_float2(0.f, 0.f);
                const float2 up = p[t], dn = p[2 + t];
                const unsigned f = updA ? (ff[1 + t] & 0xffu) : ((ff[1 + t] >> 8) & 0xffu);
                if (f & F_PROJ) {
                    const int acc = __popc(f & F_NBRS);
                    const float pc = updA ? cur.x : cur.y;
                    const float xm = updA ? left : cur.x;
                    const float xp = updA ? cur.y : right;
                    const float sum = xm + xp + (updA ? ym.x : ym.y) + (updA ? yp.x : yp.y) +
                                      (updA ? dn.x : dn.y) + (updA ? up.x : up.y);
                    const float bc = updA ? bb[1 + t].x : bb[1 + t].y;
                    const float r = fmaf(-(float)acc, pc, bc + sum);
                    const float pn = fmaf(wacc[acc], r, pc);
                    if (updA) p[1 + t].x = pn; else p[1 + t].y = pn;
                }
            }
        }

        // plane q-1-T is finished
        const int zo = q - 1 - T;
        if (interior && zo >= za && zo < zb)
            *reinterpret_cast<float2*>(Pout + rowoff + g.XY * zo) = p[1 + T];
        par ^= 1;
    }

    if (check) block_max_to(rmax, &status->rmax_bits[group]);
}

template <int T>
void launch_tb(const Grid& g, const float* Pin, float* Pout, const float* b, const uint8_t* flags,
               int nhalf, int colour0, int zchunk, const float* wacc7, StepStatus* status, int check,
               int group, float tol, int* pcur, int out_idx, cudaStream_t st) {
    static bool configured = false;
    const size_t smem = sizeof(float2) * 2 * (T + 1) * TB_TY * TB_TX;
    if (!configured) {
        cudaFuncSetAttribute(k_sweep_tb<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    WAcc8 wa;
    for (int k = 0; k < 7; ++k) wa.w[k] = wacc7[k];
    wa.w[7] = 0.0f;
    constexpr int IX = TB_CX - 2 * T, IY = TB_TY - 2 * T;
    dim3 grid((unsigned)((g.nx + IX - 1) / IX), (unsigned)((g.ny + IY - 1) / IY),
              (unsigned)((g.nz + zchunk - 1) / zchunk));
    k_sweep_tb<T><<<grid, dim3(TB_TX, TB_TY), smem, st>>>(g, Pin, Pout, b, flags, nhalf, colour0, zchunk,
                                                         wa, status, check, group, tol, pcur, out_idx);
}

}  // namespace

int sweep_tb_depth_supported(int T) { return T == 2 || T == 4 || T == 6 || T == 8; }

void launch_sweep_tb(const Grid& g, const float* Pin, float* Pout, const float* b,
                     const uint8_t* flags, int T, int nhalf, int colour0, int zchunk,
                     const float* wacc7, StepStatus* status, int check, int group, float tol,
                     int* pcur, int out_idx, cudaStream_t st) {
    switch (T) {
        case 2: launch_tb<2>(g, Pin, Pout, b, flags, nhalf, colour0, zchunk, wacc7, status, check, group, tol, pcur, out_idx, st); break;
        case 4: launch_tb<4>(g, Pin, Pout, b, flags, nhalf, colour0, zchunk, wacc7, status, check, group, tol, pcur, out_idx, st); break;
        case 6: launch_tb<6>(g, Pin, Pout, b, flags, nhalf, colour0, zchunk, wacc7, status, check, group, tol, pcur, out_idx, st); break;
        default: launch_tb<8>(g, Pin, Pout, b, flags, nhalf, colour0, zchunk, wacc7, status, check, group, tol, pcur, out_idx, st); break;
    }
}

}  // namespace smk
