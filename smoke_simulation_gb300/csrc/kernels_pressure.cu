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
                      const int* __restrict__ pcur, int warm) {
    body_rhs(g, u, v, w, flags, b, P, P2, pcur, warm, blockIdx);
}

__global__ void k_sweep(Grid g, float* __restrict__ P, const float* __restrict__ b,
                        const uint8_t* __restrict__ flags, int colour, WAcc wa,
                        const StepStatus* __restrict__ status) {
    body_sweep(g, P, b, flags, colour, wa, status, blockIdx);
}

__global__ void k_resid_check(Grid g, const float* __restrict__ P, const float* __restrict__ b,
                              const uint8_t* __restrict__ flags, StepStatus* status, int group,
                              float tol) {
    body_resid_check(g, P, b, flags, status, group, tol, blockIdx);
}

__global__ void k_gradient_subtract(Grid g, float* __restrict__ u, float* __restrict__ v,
                                    float* __restrict__ w, const float* __restrict__ P0,
                                    const float* __restrict__ P1, const int* __restrict__ pcur,
                                    const uint8_t* __restrict__ flags) {
    body_gradient_subtract(g, u, v, w, P0, P1, pcur, flags, blockIdx);
}

}  // namespace

template <typename T>
void launch_rhs(const Grid& g, const T* u, const T* v, const T* w, const uint8_t* flags,
                float* b, float* P, const float* P2, const int* pcur, int warm, cudaStream_t st) {
    k_rhs<<<grid3(g.nx, g.ny, g.nz), dim3(BX, BY), 0, st>>>(g, u, v, w, flags, b, P, P2, pcur, warm);
}
template void launch_rhs<float>(const Grid&, const float*, const float*, const float*, const uint8_t*, float*,
                                float*, const float*, const int*, int, cudaStream_t);
template void launch_rhs<__nv_bfloat16>(const Grid&, const __nv_bfloat16*, const __nv_bfloat16*,
                                        const __nv_bfloat16*, const uint8_t*, float*, float*, const float*,
                                        const int*, int, cudaStream_t);

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

void launch_resid_check(const Grid& g, const float* P, const float* b, const uint8_t* flags,
                        StepStatus* status, int group, float tol, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    k_resid_check<<<grid3(g.nx - 2, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, P, b, flags, status,
                                                                               group, tol);
}

void launch_gradient_subtract(const Grid& g, float* u, float* v, float* w, const float* P0,
                              const float* P1, const int* pcur, const uint8_t* flags,
                              cudaStream_t st) {
    if (g.nx < 2 || g.ny < 2 || g.nz < 2) return;
    k_gradient_subtract<<<grid3(g.nx - 1, g.ny - 1, g.nz - 1), dim3(BX, BY), 0, st>>>(
        g, u, v, w, P0, P1, pcur, flags);
}

}  // namespace smk
