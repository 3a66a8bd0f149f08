// Pressure-form projection: right-hand side, red-black SOR sweeps on P, the tolerance check,
// and the gradient subtract.
//
// The reference projects in velocity space (project/smokeSimulation.cu:356-394): every colour
// pass reads and rewrites all six faces of each cell (~25 B/cell/pass).  Accumulating its
// per-cell corrections p_t into a cell pressure P gives the identical iteration in exact
// arithmetic -- SOR on  acc_c*P_c - sum_{fluid nbrs} P_n = -div(u*)_c  -- whose passes touch
// only P, b and one flag byte, and one gradient subtract u -= grad P on faces whose two cells
// are fluid replaces the per-pass face updates.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"

namespace smk {

namespace {

constexpr int BX = 64, BY = 4;

inline dim3 grid3(int rx, int ry, int rz) {
    return dim3((unsigned)((rx + BX - 1) / BX), (unsigned)((ry + BY - 1) / BY), (unsigned)rz);
}

struct WAcc { float w[8]; };

// b = -div(u*) on projectable cells; P = 0 off them (and everywhere on a cold start).  P is
// the first of the two pressure buffers; on a warm start whose previous solve ended in the
// second buffer (*pcur == 1) the previous pressure is taken from there.
__global__ void k_rhs(Grid g, const float* __restrict__ u, const float* __restrict__ v,
                      const float* __restrict__ w, const uint8_t* __restrict__ flags,
                      float* __restrict__ b, float* __restrict__ P, const float* __restrict__ P2,
                      const int* __restrict__ pcur, int warm) {
    int x = blockIdx.x * BX + threadIdx.x;
    int y = blockIdx.y * BY + threadIdx.y;
    int z = blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    int i = g.idx(x, y, z);
    if (flags[i] & F_PROJ) {
        float div = -u[i] + u[i + 1] + -v[i] + v[i + g.X] + -w[i] + w[i + g.XY];
        b[i] = -div;
        if (!warm) P[i] = 0.0f;
        else if (pcur != nullptr && P2 != nullptr && *pcur == 1) P[i] = P2[i];
    } else {
        b[i] = 0.0f;
        P[i] = 0.0f;
    }
}

// One colour pass:  r = fma(-acc, P_c, b_c + (((P_x-+P_x+)+(P_y-+P_y+))+(P_z-+P_z+)));
// P_c = fma(omega/acc, r, P_c).
__global__ void k_sweep(Grid g, float* __restrict__ P, const float* __restrict__ b,
                        const uint8_t* __restrict__ flags, int colour, WAcc wa,
                        const StepStatus* __restrict__ status) {
    if (status && *(volatile const int*)&status->done) return;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    int x = 1 + ((1 + y + z + colour) & 1) + 2 * (int)(blockIdx.x * BX + threadIdx.x);
    if (x > g.nx - 2 || y > g.ny - 2) return;
    int i = g.idx(x, y, z);
    uint8_t f = flags[i];
    if (!(f & F_PROJ)) return;
    int acc = __popc((unsigned)(f & F_NBRS));
    float sum = ((P[i - 1] + P[i + 1]) + (P[i - g.X] + P[i + g.X])) + (P[i - g.XY] + P[i + g.XY]);
    float pc = P[i];
    float r = fmaf(-(float)acc, pc, b[i] + sum);
    P[i] = fmaf(wa.w[acc], r, pc);
}

// Residual check at the start of sweep group `group`.  If the previous group's residual was
// within tolerance the solve is over: set `done` (later sweeps and checks return at once).
// Otherwise record max |r| of the current state for this group.
__global__ void k_resid_check(Grid g, const float* __restrict__ P, const float* __restrict__ b,
                              const uint8_t* __restrict__ flags, StepStatus* status, int group,
                              float tol) {
    if (*(volatile int*)&status->done) return;
    if (group > 0 && __uint_as_float(status->rmax_bits[group - 1]) <= tol) {
        if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 &&
            threadIdx.y == 0) {
            status->done = 1;
            status->done_group = group;
        }
        return;
    }
    int x = 1 + blockIdx.x * BX + threadIdx.x;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    float m = 0.0f;
    if (x <= g.nx - 2 && y <= g.ny - 2) {
        int i = g.idx(x, y, z);
        uint8_t f = flags[i];
        if (f & F_PROJ) {
            int acc = __popc((unsigned)(f & F_NBRS));
            float sum = ((P[i - 1] + P[i + 1]) + (P[i - g.X] + P[i + g.X])) + (P[i - g.XY] + P[i + g.XY]);
            float r = fmaf(-(float)acc, P[i], b[i] + sum);
            m = fabsf(r);
        }
    }
    block_max_to(__float_as_uint(m), &status->rmax_bits[group]);
}

// u -= P(x) - P(x-1) on faces whose two cells are fluid (P is 0 off the projectable set, so
// this reproduces exactly which faces the reference's passes move).
// The pressure is the first buffer, or the second when *pcur == 1 (the temporally blocked
// sweeps ping-pong between the two and record where the last executed launch wrote).
__global__ void k_gradient_subtract(Grid g, float* __restrict__ u, float* __restrict__ v,
                                    float* __restrict__ w, const float* __restrict__ P0,
                                    const float* __restrict__ P1, const int* __restrict__ pcur,
                                    const uint8_t* __restrict__ flags) {
    const float* __restrict__ P = (pcur != nullptr && *pcur == 1) ? P1 : P0;
    int x = 1 + blockIdx.x * BX + threadIdx.x;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    int i = g.idx(x, y, z);
    uint8_t f = flags[i];
    if (!(f & F_SELF)) return;
    const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2, inz = z <= g.nz - 2;
    float pc = P[i];
    if (iny && inz && (f & F_XM)) u[i] = u[i] - (pc - P[i - 1]);
    if (inx && inz && (f & F_YM)) v[i] = v[i] - (pc - P[i - g.X]);
    if (inx && iny && (f & F_ZM)) w[i] = w[i] - (pc - P[i - g.XY]);
}

}  // namespace

void launch_rhs(const Grid& g, const float* u, const float* v, const float* w, const uint8_t* flags,
                float* b, float* P, const float* P2, const int* pcur, int warm, cudaStream_t st) {
    k_rhs<<<grid3(g.nx, g.ny, g.nz), dim3(BX, BY), 0, st>>>(g, u, v, w, flags, b, P, P2, pcur, warm);
}

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
