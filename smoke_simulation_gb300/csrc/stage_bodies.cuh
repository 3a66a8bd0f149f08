// Bodies of the per-step stage kernels, shared by the single-grid kernels (one launch per grid
// and stage) and the grouped kernels (one launch per stage over every grid of a batch).
//
// A body receives its block coordinates explicitly (`bid`), checks every axis against its own
// range, and evaluates the reference's expressions in the reference's order (see the single-
// grid kernels in kernels_step.cu / kernels_pressure.cu for the reference lines each restates).
// Blocks are 64 x 4 threads over x and y, one z plane per block.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace smk {

constexpr int SB_BX = 64, SB_BY = 4;

struct WAcc { float w[8]; };

// ---- emitters ---------------------------------------------------------------------------------

// One cell of the box emitters (in list order, so the last box containing the cell decides):
// density into both buffers, and the box's upward velocity on the cell's two v faces.
template <typename T, typename Tv>
__device__ __forceinline__ void cell_emit_boxes(const Grid& g, T* __restrict__ rho0, T* __restrict__ rho1,
                                                Tv* __restrict__ v_now, const BoxObj* boxes, int nb,
                                                int x, int y, int z) {
    for (int k = 0; k < nb; ++k) {
        const BoxObj& b = boxes[k];
        if (x >= b.x0 && x < b.x1 && y >= b.y0 && y < b.y1 && z >= b.z0 && z < b.z1) {
            const int i = g.idx(x, y, z);
            stv(rho0, i, b.density);
            stv(rho1, i, b.density);
            if (b.set_vy) {
                stv(v_now, i, b.vy);
                stv(v_now, i + g.X, b.vy);
            }
        }
    }
}

// Box emitters restricted to [x0,x1)x[y0,..)x[z0,..): density into both buffers, optional v.
template <typename T, typename Tv>
__device__ __forceinline__ void body_emit_boxes(const Grid& g, T* __restrict__ rho0,
                                                T* __restrict__ rho1, Tv* __restrict__ v_now,
                                                const BoxObj* boxes, int nb, int x0, int y0, int z0,
                                                int x1, int y1, int z1, uint3 bid) {
    const int x = x0 + (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = y0 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = z0 + (int)bid.z;
    if (x >= x1 || y >= y1 || z >= z1) return;
    cell_emit_boxes(g, rho0, rho1, v_now, boxes, nb, x, y, z);
}

// One cell of fillSmoke (smokeSimulation.cu:251-273): float squared distance from the integer
// corner, strict test, both buffers = 1.
template <typename T>
__device__ __forceinline__ void cell_fill_smoke(const Grid& g, T* __restrict__ rho0, T* __restrict__ rho1,
                                                const SphereObj* sp, int ns, int x, int y, int z) {
    for (int k = 0; k < ns; ++k) {
        const float dx = (float)x - sp[k].x, dy = (float)y - sp[k].y, dz = (float)z - sp[k].z;
        const float dist = dx * dx + dy * dy + dz * dz;
        if (dist < sp[k].r * sp[k].r) {
            const int i = g.idx(x, y, z);
            stv(rho0, i, 1.0f);
            stv(rho1, i, 1.0f);
        }
    }
}

// fillSmoke over the box [x0,x1)x[y0,y1)x[z0,z1) (within the interior).
template <typename T>
__device__ __forceinline__ void body_fill_smoke(const Grid& g, T* __restrict__ rho0,
                                                T* __restrict__ rho1, const SphereObj* sp, int ns,
                                                int x0, int y0, int z0, int x1, int y1, int z1,
                                                uint3 bid) {
    const int x = x0 + (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = y0 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = z0 + (int)bid.z;
    if (x >= x1 || y >= y1 || z >= z1) return;
    cell_fill_smoke(g, rho0, rho1, sp, ns, x, y, z);
}

// ---- forcing: integrate (smokeSimulation.cu:315-329) + velocityConfinement (:331-352) -------

// One face index of the forcing: buoyancy/gravity on v where the cell and the one below are
// fluid, then the velocity clamp (x >= 1, z >= 1).  Updates (ut, vt, wt) in place; returns bit 0
// when v is to be stored, bit 1 when u and w are (the clamp scaled them).
__device__ __forceinline__ unsigned cell_forcing(uint8_t f, int x, int z, float r, float& ut, float& vt,
                                                 float& wt, float dt, float gravity, float alpha, float lim_sq,
                                                 float lim, int clamp_mode) {
    const bool force = (f & F_SELF) && (f & F_YM);
    const bool clamp = x >= 1 && z >= 1 && clamp_mode != 2;
    const float buoy = alpha * (r - 0.0f);
    if (force) vt = vt + (r * gravity * dt + buoy * dt);
    unsigned wr = (force || clamp) ? 1u : 0u;
    if (clamp) {
        const float len = ut * ut + vt * vt + wt * wt;
        if (clamp_mode == 0) {
            if (len * dt > lim_sq) {
                const float s = lim_sq / (len * dt);
                ut = ut * s;
                vt = vt * s;
                wt = wt * s;
                wr |= 2u;
            }
        } else if (len > lim * lim) {
            const float s = lim / sqrtf(len);
            ut = ut * s;
            vt = vt * s;
            wt = wt * s;
            wr |= 2u;
        }
    }
    return wr;
}

template <typename Tv, typename T>
__device__ __forceinline__ void body_forcing(const Grid& g, Tv* __restrict__ u, Tv* __restrict__ v,
                                             Tv* __restrict__ w, const T* __restrict__ rho,
                                             const uint8_t* __restrict__ flags, float dt, float gravity,
                                             float alpha, float lim_sq, float lim, int clamp_mode,
                                             uint3 bid) {
    const int x = (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = 1 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = (int)bid.z;
    if (x >= g.nx || y >= g.ny || z >= g.nz) return;
    const int i = g.idx(x, y, z);
    // every input is loaded before the flag byte is tested (the clamp reads u and w of the
    // same index; the buoyancy reads the density): one memory round trip per cell
    const uint8_t f = flags[i];
    float vt = ldv(v, i), ut = ldv(u, i), wt = ldv(w, i);
    const float r = ldv(rho, i);
    const unsigned wr = cell_forcing(f, x, z, r, ut, vt, wt, dt, gravity, alpha, lim_sq, lim, clamp_mode);
    if (wr & 2u) {
        stv(u, i, ut);
        stv(w, i, wt);
    }
    if (wr & 1u) stv(v, i, vt);
}

// ---- pressure scheme ------------------------------------------------------------------------
//
// The projection bodies take plain (not __restrict__) pointers: the grouped projection runs
// them as phases of one cooperative launch, where a phase reads what other CTAs wrote in an
// earlier phase (after a grid barrier), so no load of P, b or the velocities may go through
// the non-coherent read-only path.

// b = -div(u*) on projectable cells; P = 0 off them (and everywhere on a cold start); on a warm
// start whose previous solve ended in the second buffer (*pcur == 1) P is taken from there.
// With a pressure history Ph (smk_params.warm_extrapolate): Ph takes the last pressure Pl of
// every cell, and a projectable cell starts from Pl + alpha * (Pl - Ph_before) (alpha = 0: Pl).
__device__ __forceinline__ float warm_extrapolated(float pl, float ph, float alpha) {
    return alpha != 0.0f ? __fadd_rn(pl, __fmul_rn(alpha, __fsub_rn(pl, ph))) : pl;
}

template <typename T>
__device__ __forceinline__ void body_rhs(const Grid& g, const T* u, const T* v, const T* w,
                                         const uint8_t* __restrict__ flags, float* b, float* P,
                                         const float* P2, const int* pcur, int warm, uint3 bid,
                                         float* Ph = nullptr, float alpha = 0.0f) {
    const int x = (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = (int)bid.z;
    if (x >= g.nx || y >= g.ny || z >= g.nz) return;
    const int i = g.idx(x, y, z);
    // the six faces are loaded for every cell (all indices stay inside the face arrays) and the
    // flag selects the result, so the loads do not wait on the flag byte
    const uint8_t f = flags[i];
    const float u0 = ldv(u, i), u1 = ldv(u, i + 1), v0 = ldv(v, i), v1 = ldv(v, i + g.X),
                w0 = ldv(w, i), w1 = ldv(w, i + g.XY);
    const float div = -u0 + u1 + -v0 + v1 + -w0 + w1;
    const bool proj = (f & F_PROJ) != 0;
    b[i] = proj ? -div : 0.0f;
    const bool from2 = pcur != nullptr && P2 != nullptr && *pcur == 1;
    if (Ph != nullptr) {
        const float pl = warm ? (from2 ? P2[i] : P[i]) : 0.0f;
        const float ph = Ph[i];
        Ph[i] = pl;
        P[i] = proj ? warm_extrapolated(pl, ph, alpha) : 0.0f;
        return;
    }
    if (!proj || !warm) P[i] = 0.0f;
    else if (from2) P[i] = P2[i];
}

// One cell of a colour pass:  r = fma(-acc, P_c, b_c + (((P_x-+P_x+)+(P_y-+P_y+))+(P_z-+P_z+)));
// P_c = fma(omega/acc, r, P_c).
__device__ __forceinline__ void cell_sweep(const Grid& g, float* P, const float* b,
                                           const uint8_t* __restrict__ flags, int i, const float* wacc) {
    const uint8_t f = flags[i];
    if (!(f & F_PROJ)) return;
    const int acc = __popc((unsigned)(f & F_NBRS));
    const float sum = ((P[i - 1] + P[i + 1]) + (P[i - g.X] + P[i + g.X])) + (P[i - g.XY] + P[i + g.XY]);
    const float pc = P[i];
    const float r = fmaf(-(float)acc, pc, b[i] + sum);
    P[i] = fmaf(wacc[acc], r, pc);
}

// |residual| of one cell (0 off the projectable set), the expression of cell_sweep.
__device__ __forceinline__ float cell_resid(const Grid& g, const float* P, const float* b,
                                            const uint8_t* __restrict__ flags, int i) {
    const uint8_t f = flags[i];
    if (!(f & F_PROJ)) return 0.0f;
    const int acc = __popc((unsigned)(f & F_NBRS));
    const float sum = ((P[i - 1] + P[i + 1]) + (P[i - g.X] + P[i + g.X])) + (P[i - g.XY] + P[i + g.XY]);
    const float r = fmaf(-(float)acc, P[i], b[i] + sum);
    return fabsf(r);
}

// |div u| of one cell (0 off the projectable set).
__device__ __forceinline__ float cell_div(const Grid& g, const float* u, const float* v, const float* w,
                                          const uint8_t* __restrict__ flags, int i) {
    if (!(flags[i] & F_PROJ)) return 0.0f;
    const float div = -u[i] + u[i + 1] + -v[i] + v[i + g.X] + -w[i] + w[i + g.XY];
    return fabsf(div);
}

// One colour pass.  bid.x counts same-colour cells of a row.
__device__ __forceinline__ void body_sweep(const Grid& g, float* P, const float* b,
                                           const uint8_t* __restrict__ flags, int colour, const WAcc& wa,
                                           const StepStatus* __restrict__ status, uint3 bid) {
    if (status && *(volatile const int*)&status->done) return;
    const int y = 1 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = 1 + (int)bid.z;
    const int x = 1 + ((1 + y + z + colour) & 1) + 2 * ((int)bid.x * SB_BX + (int)threadIdx.x);
    if (x > g.nx - 2 || y > g.ny - 2 || z > g.nz - 2) return;
    cell_sweep(g, P, b, flags, g.idx(x, y, z), wa.w);
}

// Residual check at the start of sweep group `group`: record max |r| of the current pressure;
// the last block to finish decides (check_decide): within tolerance, the solve ends here and
// the group's sweeps, which test `done`, do nothing.  Contains a block barrier: every thread of
// the block must call it.  nblocks: the blocks of the launch.
__device__ __forceinline__ void body_resid_check(const Grid& g, const float* P, const float* b,
                                                 const uint8_t* __restrict__ flags, StepStatus* status,
                                                 int group, float tol, uint3 bid, unsigned nblocks) {
    if (*(volatile int*)&status->done) return;
    const int x = 1 + (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = 1 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = 1 + (int)bid.z;
    float m = 0.0f;
    if (x <= g.nx - 2 && y <= g.ny - 2 && z <= g.nz - 2) m = cell_resid(g, P, b, flags, g.idx(x, y, z));
    block_max_to(__float_as_uint(m), &status->rmax_bits[group]);
    if (threadIdx.x == 0 && threadIdx.y == 0) check_decide(status, group, tol, nblocks, nullptr, -1);
}

// u -= P(x) - P(x-1) on faces whose two cells are fluid (P is 0 off the projectable set).  The
// pressure is the first buffer, or the second when *pcur == 1.
__device__ __forceinline__ void body_gradient_subtract(const Grid& g, float* u, float* v, float* w,
                                                       const float* P0, const float* P1, const int* pcur,
                                                       const uint8_t* __restrict__ flags, uint3 bid) {
    const float* P = (pcur != nullptr && *pcur == 1) ? P1 : P0;
    const int x = 1 + (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = 1 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = 1 + (int)bid.z;
    if (x >= g.nx || y >= g.ny || z >= g.nz) return;
    const int i = g.idx(x, y, z);
    // loads first, then the flag decides which faces change; every face of the range is
    // written (unchanged ones with their own value), so no load waits on the flag byte
    const uint8_t f = flags[i];
    const float pc = P[i], px = P[i - 1], py = P[i - g.X], pz = P[i - g.XY];
    const float uu = u[i], vv = v[i], ww = w[i];
    const bool self = (f & F_SELF) != 0;
    const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2, inz = z <= g.nz - 2;
    u[i] = (self && iny && inz && (f & F_XM)) ? uu - (pc - px) : uu;
    v[i] = (self && inx && inz && (f & F_YM)) ? vv - (pc - py) : vv;
    w[i] = (self && inx && iny && (f & F_ZM)) ? ww - (pc - pz) : ww;
}

// ---- four consecutive x per thread (FP32 storage, 16-byte aligned rows) ----------------------
//
// The thread's group is x0..x0+3 (x0 a multiple of 4) of row (y, z); a group not entirely inside
// the stage's x range takes the per-element path.  Same expressions, in the same order, as the
// per-cell bodies above, so every result is the same.  Plain pointers, as for the projection
// bodies (the grouped projection runs the rhs and the subtract as phases of one launch).

// Forcing (body_forcing, cell_forcing) for velocities stored as Tv and density as T: a group's
// faces that do not change keep their bits (st4).  Rows y >= 1.
template <typename Tv, typename T>
__device__ __forceinline__ void body_forcing_x4(const Grid& g, Tv* u, Tv* v, Tv* w, const T* rho,
                                                const uint8_t* flags, float dt, float gravity, float alpha,
                                                float lim_sq, float lim, int clamp_mode, int x0, int y, int z) {
    if (x0 >= g.nx || y >= g.ny || z >= g.nz) return;
    const int i = g.idx(x0, y, z);
    if (x0 + 3 < g.nx) {
        const uchar4 f = *reinterpret_cast<const uchar4*>(flags + i);
        const typename Raw4<Tv>::type ru = ld4raw(u + i), rv = ld4raw(v + i), rw = ld4raw(w + i);
        float4 uu = to4(ru), vv = to4(rv), ww = to4(rw);
        const float4 r = to4(ld4raw(rho + i));
        const unsigned w0 = cell_forcing(f.x, x0, z, r.x, uu.x, vv.x, ww.x, dt, gravity, alpha, lim_sq, lim, clamp_mode);
        const unsigned w1 =
            cell_forcing(f.y, x0 + 1, z, r.y, uu.y, vv.y, ww.y, dt, gravity, alpha, lim_sq, lim, clamp_mode);
        const unsigned w2 =
            cell_forcing(f.z, x0 + 2, z, r.z, uu.z, vv.z, ww.z, dt, gravity, alpha, lim_sq, lim, clamp_mode);
        const unsigned w3 =
            cell_forcing(f.w, x0 + 3, z, r.w, uu.w, vv.w, ww.w, dt, gravity, alpha, lim_sq, lim, clamp_mode);
        const unsigned mv = (w0 & 1u) | ((w1 & 1u) << 1) | ((w2 & 1u) << 2) | ((w3 & 1u) << 3);
        const unsigned muw = ((w0 >> 1) & 1u) | (w1 & 2u) | ((w2 & 2u) << 1) | ((w3 & 2u) << 2);
        if (mv) st4(v + i, rv, vv, mv);
        if (muw) {
            st4(u + i, ru, uu, muw);
            st4(w + i, rw, ww, muw);
        }
        return;
    }
    for (int c = 0; c < 4 && x0 + c < g.nx; ++c) {
        float ut = ldv(u, i + c), vt = ldv(v, i + c), wt = ldv(w, i + c);
        const unsigned wr = cell_forcing(flags[i + c], x0 + c, z, ldv(rho, i + c), ut, vt, wt, dt, gravity, alpha,
                                         lim_sq, lim, clamp_mode);
        if (wr & 2u) {
            stv(u, i + c, ut);
            stv(w, i + c, wt);
        }
        if (wr & 1u) stv(v, i + c, vt);
    }
}

// rhs (body_rhs) for velocities stored as T.  Rows y >= 0, planes z >= 0.
template <typename T>
__device__ __forceinline__ void body_rhs_x4(const Grid& g, const T* u, const T* v, const T* w,
                                            const uint8_t* flags, float* b, float* P, const float* P2,
                                            const int* pcur, int warm, int x0, int y, int z,
                                            float* Ph = nullptr, float alpha = 0.0f) {
    if (x0 >= g.nx || y >= g.ny || z >= g.nz) return;
    const int i = g.idx(x0, y, z);
    const bool from2 = warm && pcur != nullptr && P2 != nullptr && *pcur == 1;
    if (x0 + 3 < g.nx) {
        const uchar4 f = *reinterpret_cast<const uchar4*>(flags + i);
        const float4 u0 = to4(ld4raw(u + i));
        const float u4 = ldv(u, i + 4);  // x0 + 4 <= nx: a face of the same row
        const float4 v0 = to4(ld4raw(v + i));
        const float4 v1 = to4(ld4raw(v + i + g.X));
        const float4 w0 = to4(ld4raw(w + i));
        const float4 w1 = to4(ld4raw(w + i + g.XY));
        const bool p0 = (f.x & F_PROJ) != 0, p1 = (f.y & F_PROJ) != 0, p2 = (f.z & F_PROJ) != 0,
                   p3 = (f.w & F_PROJ) != 0;
        const float d0 = -u0.x + u0.y + -v0.x + v1.x + -w0.x + w1.x;
        const float d1 = -u0.y + u0.z + -v0.y + v1.y + -w0.y + w1.y;
        const float d2 = -u0.z + u0.w + -v0.z + v1.z + -w0.z + w1.z;
        const float d3 = -u0.w + u4 + -v0.w + v1.w + -w0.w + w1.w;
        *reinterpret_cast<float4*>(b + i) =
            make_float4(p0 ? -d0 : 0.0f, p1 ? -d1 : 0.0f, p2 ? -d2 : 0.0f, p3 ? -d3 : 0.0f);
        if (Ph != nullptr) {
            const float4 pl = warm ? *reinterpret_cast<const float4*>((from2 ? P2 : P) + i)
                                   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const float4 ph = *reinterpret_cast<const float4*>(Ph + i);
            *reinterpret_cast<float4*>(Ph + i) = pl;
            *reinterpret_cast<float4*>(P + i) = make_float4(
                p0 ? warm_extrapolated(pl.x, ph.x, alpha) : 0.0f, p1 ? warm_extrapolated(pl.y, ph.y, alpha) : 0.0f,
                p2 ? warm_extrapolated(pl.z, ph.z, alpha) : 0.0f, p3 ? warm_extrapolated(pl.w, ph.w, alpha) : 0.0f);
            return;
        }
        if (!warm) {
            *reinterpret_cast<float4*>(P + i) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else if (from2) {
            const float4 q = *reinterpret_cast<const float4*>(P2 + i);
            *reinterpret_cast<float4*>(P + i) =
                make_float4(p0 ? q.x : 0.0f, p1 ? q.y : 0.0f, p2 ? q.z : 0.0f, p3 ? q.w : 0.0f);
        } else {
            if (!p0) P[i] = 0.0f;
            if (!p1) P[i + 1] = 0.0f;
            if (!p2) P[i + 2] = 0.0f;
            if (!p3) P[i + 3] = 0.0f;
        }
        return;
    }
    for (int c = 0; c < 4 && x0 + c < g.nx; ++c) {
        const int k = i + c;
        const float div = -ldv(u, k) + ldv(u, k + 1) + -ldv(v, k) + ldv(v, k + g.X) + -ldv(w, k) + ldv(w, k + g.XY);
        const bool proj = (flags[k] & F_PROJ) != 0;
        b[k] = proj ? -div : 0.0f;
        if (Ph != nullptr) {
            const float pl = warm ? (from2 ? P2[k] : P[k]) : 0.0f;
            const float ph = Ph[k];
            Ph[k] = pl;
            P[k] = proj ? warm_extrapolated(pl, ph, alpha) : 0.0f;
            continue;
        }
        if (!proj || !warm) P[k] = 0.0f;
        else if (from2) P[k] = P2[k];
    }
}

// BF16 projection (body_project_bf16) with the pressure P already chosen: every index of
// [0, nx] x [0, ny] x [0, nz] gets its FP32 projected velocities in pu, pv, pw; the BF16 faces a
// cell changes are rounded back into u, v, w (the others keep their bits).
__device__ __forceinline__ void body_project_bf16_x4(const Grid& g, __nv_bfloat16* u, __nv_bfloat16* v,
                                                     __nv_bfloat16* w, const float* P, const uint8_t* flags,
                                                     float* pu, float* pv, float* pw, int x0, int y, int z) {
    if (x0 > g.nx || y > g.ny || z > g.nz) return;
    const int i = g.idx(x0, y, z);
    if (x0 >= 4 && x0 + 3 <= g.nx - 1 && y >= 1 && y <= g.ny - 1 && z >= 1 && z <= g.nz - 1) {
        // four cells: x0..x0+3 in [1, nx), y in [1, ny), z in [1, nz)
        const uchar4 f = *reinterpret_cast<const uchar4*>(flags + i);
        const Raw4h ru = ld4raw(u + i), rv = ld4raw(v + i), rw = ld4raw(w + i);
        const float4 u4 = to4(ru), v4 = to4(rv), w4 = to4(rw);
        const float4 pc = *reinterpret_cast<const float4*>(P + i);
        const float pxm = P[i - 1];
        const float4 py = *reinterpret_cast<const float4*>(P + i - g.X);
        const float4 pz = *reinterpret_cast<const float4*>(P + i - g.XY);
        const float pcs[4] = {pc.x, pc.y, pc.z, pc.w}, pxs[4] = {pxm, pc.x, pc.y, pc.z},
                    pys[4] = {py.x, py.y, py.z, py.w}, pzs[4] = {pz.x, pz.y, pz.z, pz.w};
        const uint8_t fs[4] = {f.x, f.y, f.z, f.w};
        float us[4] = {u4.x, u4.y, u4.z, u4.w}, vs[4] = {v4.x, v4.y, v4.z, v4.w}, ws[4] = {w4.x, w4.y, w4.z, w4.w};
        const bool iny = y <= g.ny - 2, inz = z <= g.nz - 2;
        unsigned mu = 0u, mv = 0u, mw = 0u;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (!(fs[c] & F_SELF)) continue;
            const bool inx = x0 + c <= g.nx - 2;
            if (iny && inz && (fs[c] & F_XM)) { us[c] = us[c] - (pcs[c] - pxs[c]); mu |= 1u << c; }
            if (inx && inz && (fs[c] & F_YM)) { vs[c] = vs[c] - (pcs[c] - pys[c]); mv |= 1u << c; }
            if (inx && iny && (fs[c] & F_ZM)) { ws[c] = ws[c] - (pcs[c] - pzs[c]); mw |= 1u << c; }
        }
        const float4 uo = make_float4(us[0], us[1], us[2], us[3]), vo = make_float4(vs[0], vs[1], vs[2], vs[3]),
                     wo = make_float4(ws[0], ws[1], ws[2], ws[3]);
        if (mu) st4(u + i, ru, uo, mu);
        if (mv) st4(v + i, rv, vo, mv);
        if (mw) st4(w + i, rw, wo, mw);
        *reinterpret_cast<float4*>(pu + i) = uo;
        *reinterpret_cast<float4*>(pv + i) = vo;
        *reinterpret_cast<float4*>(pw + i) = wo;
        return;
    }
    for (int c = 0; c < 4 && x0 + c <= g.nx; ++c) {
        const int x = x0 + c, k = i + c;
        float uu = ldv(u, k), vv = ldv(v, k), ww = ldv(w, k);
        if (x < g.nx && y < g.ny && z < g.nz && x >= 1 && y >= 1 && z >= 1) {
            const uint8_t f = flags[k];
            if (f & F_SELF) {
                const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2, inz = z <= g.nz - 2;
                const float pc = P[k];
                if (iny && inz && (f & F_XM)) { uu = uu - (pc - P[k - 1]); stv(u, k, uu); }
                if (inx && inz && (f & F_YM)) { vv = vv - (pc - P[k - g.X]); stv(v, k, vv); }
                if (inx && iny && (f & F_ZM)) { ww = ww - (pc - P[k - g.XY]); stv(w, k, ww); }
            }
        }
        pu[k] = uu;
        pv[k] = vv;
        pw[k] = ww;
    }
}

// Gradient subtract (body_gradient_subtract) with the pressure P already chosen: every face of
// the range [1, nx) x [1, ny) x [1, nz) is stored, unchanged ones with their own value.
__device__ __forceinline__ void body_gradient_subtract_x4(const Grid& g, float* u, float* v, float* w,
                                                          const float* P, const uint8_t* flags, int x0, int y,
                                                          int z) {
    if (x0 >= g.nx || y >= g.ny || z >= g.nz || y < 1 || z < 1) return;
    const int i = g.idx(x0, y, z);
    const bool iny = y <= g.ny - 2, inz = z <= g.nz - 2;
    if (x0 >= 1 && x0 + 3 <= g.nx - 1) {
        const uchar4 f = *reinterpret_cast<const uchar4*>(flags + i);
        const float4 pc = *reinterpret_cast<const float4*>(P + i);
        const float pxm = P[i - 1];
        const float4 py = *reinterpret_cast<const float4*>(P + i - g.X);
        const float4 pz = *reinterpret_cast<const float4*>(P + i - g.XY);
        float4 uu = *reinterpret_cast<const float4*>(u + i);
        float4 vv = *reinterpret_cast<const float4*>(v + i);
        float4 ww = *reinterpret_cast<const float4*>(w + i);
        const float pcs[4] = {pc.x, pc.y, pc.z, pc.w}, pxs[4] = {pxm, pc.x, pc.y, pc.z},
                    pys[4] = {py.x, py.y, py.z, py.w}, pzs[4] = {pz.x, pz.y, pz.z, pz.w};
        const uint8_t fs[4] = {f.x, f.y, f.z, f.w};
        float us[4] = {uu.x, uu.y, uu.z, uu.w}, vs[4] = {vv.x, vv.y, vv.z, vv.w}, ws[4] = {ww.x, ww.y, ww.z, ww.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const bool self = (fs[c] & F_SELF) != 0;
            const bool inx = x0 + c <= g.nx - 2;
            if (self && iny && inz && (fs[c] & F_XM)) us[c] = us[c] - (pcs[c] - pxs[c]);
            if (self && inx && inz && (fs[c] & F_YM)) vs[c] = vs[c] - (pcs[c] - pys[c]);
            if (self && inx && iny && (fs[c] & F_ZM)) ws[c] = ws[c] - (pcs[c] - pzs[c]);
        }
        *reinterpret_cast<float4*>(u + i) = make_float4(us[0], us[1], us[2], us[3]);
        *reinterpret_cast<float4*>(v + i) = make_float4(vs[0], vs[1], vs[2], vs[3]);
        *reinterpret_cast<float4*>(w + i) = make_float4(ws[0], ws[1], ws[2], ws[3]);
        return;
    }
    for (int c = 0; c < 4; ++c) {
        const int x = x0 + c;
        if (x < 1 || x >= g.nx) continue;
        const int k = i + c;
        const uint8_t f = flags[k];
        const bool self = (f & F_SELF) != 0;
        const bool inx = x <= g.nx - 2;
        const float pc = P[k];
        if (self && iny && inz && (f & F_XM)) u[k] = u[k] - (pc - P[k - 1]);
        if (self && inx && inz && (f & F_YM)) v[k] = v[k] - (pc - P[k - g.X]);
        if (self && inx && iny && (f & F_ZM)) w[k] = w[k] - (pc - P[k - g.XY]);
    }
}

// max |div u| over projectable cells.  Contains a block barrier.
__device__ __forceinline__ void body_div_max(const Grid& g, const float* u, const float* v,
                                             const float* w, const uint8_t* __restrict__ flags,
                                             StepStatus* status, uint3 bid) {
    const int x = 1 + (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = 1 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = 1 + (int)bid.z;
    float m = 0.0f;
    if (x <= g.nx - 2 && y <= g.ny - 2 && z <= g.nz - 2) m = cell_div(g, u, v, w, flags, g.idx(x, y, z));
    block_max_to(__float_as_uint(m), &status->div_bits);
}

// BF16 storage form: the projected velocity is written in FP32 to (pu, pv, pw) over every face
// (advection reads it there, and max|div u| is measured there), and rounded into the BF16
// state where the gradient changed it, so the state holds the projected velocity as in the
// FP32 form.  Storing only the rounded value would leave a divergence of order 1e-2 |u|.
__device__ __forceinline__ void body_project_bf16(const Grid& g, __nv_bfloat16* u, __nv_bfloat16* v,
                                                  __nv_bfloat16* w, const float* P0, const float* P1,
                                                  const int* pcur, const uint8_t* __restrict__ flags,
                                                  float* pu, float* pv, float* pw, uint3 bid) {
    const float* P = (pcur != nullptr && *pcur == 1) ? P1 : P0;
    const int x = (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = (int)bid.z;
    if (x > g.nx || y > g.ny || z > g.nz) return;
    const int i = g.idx(x, y, z);
    float uu = ldv(u, i), vv = ldv(v, i), ww = ldv(w, i);
    const bool cell = x < g.nx && y < g.ny && z < g.nz && x >= 1 && y >= 1 && z >= 1;
    if (cell) {
        const uint8_t f = flags[i];
        if (f & F_SELF) {
            const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2, inz = z <= g.nz - 2;
            const float pc = P[i];
            if (iny && inz && (f & F_XM)) { uu = uu - (pc - P[i - 1]); stv(u, i, uu); }
            if (inx && inz && (f & F_YM)) { vv = vv - (pc - P[i - g.X]); stv(v, i, vv); }
            if (inx && iny && (f & F_ZM)) { ww = ww - (pc - P[i - g.XY]); stv(w, i, ww); }
        }
    }
    pu[i] = uu;
    pv[i] = vv;
    pw[i] = ww;
}

// ---- advection --------------------------------------------------------------------------------

// velocityAdvectionU/V/W (smokeSimulation.cu:527-615), the three fused per staggered index.
template <typename Ti, typename To>
__device__ __forceinline__ void body_advect_velocity(const Grid& g, const Ti* __restrict__ u0,
                                                     const Ti* __restrict__ v0,
                                                     const Ti* __restrict__ w0, To* __restrict__ u1,
                                                     To* __restrict__ v1, To* __restrict__ w1,
                                                     const uint8_t* __restrict__ flags, float dt,
                                                     uint3 bid) {
    const int x = 1 + (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = 1 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = 1 + (int)bid.z;
    if (x >= g.nx || y >= g.ny || z >= g.nz) return;
    const int i = g.idx(x, y, z);
    const uint8_t f = flags[i];
    if (!(f & F_SELF)) return;
    const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2, inz = z <= g.nz - 2;
    const bool du = iny && inz && (f & F_XM), dv = inx && inz && (f & F_YM),
               dw = inx && iny && (f & F_ZM);
    if (!(du || dv || dw)) return;
    // The three 8-point averages at one index serve two faces each (avgU: v and w faces, avgV:
    // u and w, avgW: u and v), so each is evaluated once.
    const float au = avgU(u0, g, i), av = avgV(v0, g, i), aw = avgW(w0, g, i);
    if (du) {
        float xt = (float)x, yt = (float)y + 0.5f, zt = (float)z + 0.5f;
        xt = xt - dt * ldv(u0, i);
        yt = yt - dt * av;
        zt = zt - dt * aw;
        stv(u1, i, sample_ref<0, 1, 1>(u0, g, xt, yt, zt));
    }
    if (dv) {
        float xt = (float)x + 0.5f, yt = (float)y, zt = (float)z + 0.5f;
        xt = xt - dt * au;
        yt = yt - dt * ldv(v0, i);
        zt = zt - dt * aw;
        stv(v1, i, sample_ref<1, 0, 1>(v0, g, xt, yt, zt));
    }
    if (dw) {
        float xt = (float)x + 0.5f, yt = (float)y + 0.5f, zt = (float)z;
        xt = xt - dt * au;
        yt = yt - dt * av;
        zt = zt - dt * ldv(w0, i);
        stv(w1, i, sample_ref<1, 1, 0>(w0, g, xt, yt, zt));
    }
}

// advectSmoke (smokeSimulation.cu:617-638) with the NEW velocities.  The reference evaluates
// the backtrace x + 0.5 - u*dt in double and rounds to float.  With a = x + 0.5 (exact, lowest
// bit 2^-1) and b = u*dt (a float), the exact a - b needs at most max(e_a - e_b, 0) + 24 bits,
// so it is exact in double unless |b| < a*2^-29; then a - b lies strictly inside a's float
// rounding interval, in double too.  Either way float(double(a) - double(b)) equals the single-
// rounded float subtraction, which avoids GB300's slow FP64 pipe (golden-vector tests pin it).
template <typename T, typename Tv>
__device__ __forceinline__ void body_advect_density(const Grid& g, const T* __restrict__ r0,
                                                    T* __restrict__ r1, const Tv* __restrict__ u,
                                                    const Tv* __restrict__ v,
                                                    const Tv* __restrict__ w,
                                                    const uint8_t* __restrict__ flags, float dt,
                                                    uint3 bid) {
    const int x = 1 + (int)bid.x * SB_BX + (int)threadIdx.x;
    const int y = 1 + (int)bid.y * SB_BY + (int)threadIdx.y;
    const int z = 1 + (int)bid.z;
    if (x > g.nx - 2 || y > g.ny - 2 || z > g.nz - 2) return;
    const int i = g.idx(x, y, z);
    // the face velocities are loaded with the flag byte, not after it (ld_eager)
    const float ua = ld_eager(u + i), ub = ld_eager(u + i + 1), va = ld_eager(v + i),
                vb = ld_eager(v + i + g.X), wa = ld_eager(w + i), wb = ld_eager(w + i + g.XY);
    if (!(flags[i] & F_SELF)) return;
    const float ut = (ua + ub) / 2.0f;
    const float vt = (va + vb) / 2.0f;
    const float wt = (wa + wb) / 2.0f;
    const float xt = __fsub_rn((float)x + 0.5f, ut * dt);
    const float yt = __fsub_rn((float)y + 0.5f, vt * dt);
    const float zt = __fsub_rn((float)z + 0.5f, wt * dt);
    stv(r1, i, sample_ref<1, 1, 1>(r0, g, xt, yt, zt));
}

}  // namespace smk
