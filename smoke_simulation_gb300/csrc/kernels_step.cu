// Stage kernels shared by both projection schemes, plus the reference-scheme projection.
//
// Each kernel restates one stage of the reference step (project/smokeSimulation.cu) with the
// reference's exact floating-point expression order, on the library's pitched layout
// (common.cuh) and with x-contiguous, coalesced thread mapping (one thread per x, a warp per
// row segment) instead of the reference's 8x8x8 cubes.
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

constexpr int MAX_OBJ_PER_LAUNCH = 64;
struct SphereList { int n; SphereObj s[MAX_OBJ_PER_LAUNCH]; };
struct ObstacleList { int n; ObstacleObj o[MAX_OBJ_PER_LAUNCH]; };
struct BoxList { int n; BoxObj b[MAX_OBJ_PER_LAUNCH]; };

// ---- a4: emitters ---------------------------------------------------------------------------

// Box emitters over the union box [lo, hi): density into both buffers, optional v-faces.
__global__ void k_emit_boxes(Grid g, float* __restrict__ rho0, float* __restrict__ rho1,
                             float* __restrict__ v_now, BoxList L, int x0, int y0, int z0, int x1,
                             int y1) {
    int x = x0 + blockIdx.x * BX + threadIdx.x;
    int y = y0 + blockIdx.y * BY + threadIdx.y;
    int z = z0 + blockIdx.z;
    if (x >= x1 || y >= y1) return;
    for (int k = 0; k < L.n; ++k) {
        const BoxObj& b = L.b[k];
        if (x >= b.x0 && x < b.x1 && y >= b.y0 && y < b.y1 && z >= b.z0 && z < b.z1) {
            int i = g.idx(x, y, z);
            rho0[i] = b.density;
            rho1[i] = b.density;
            if (b.set_vy) {
                v_now[i] = b.vy;
                v_now[i + g.X] = b.vy;
            }
        }
    }
}

// fillSmoke (smokeSimulation.cu:251-273): interior cells, float squared distance from the
// integer corner, strict test, density 1 in both buffers.
__global__ void k_fill_smoke(Grid g, float* __restrict__ rho0, float* __restrict__ rho1, SphereList L,
                             int x0, int y0, int z0, int x1, int y1) {
    int x = x0 + blockIdx.x * BX + threadIdx.x;
    int y = y0 + blockIdx.y * BY + threadIdx.y;
    int z = z0 + blockIdx.z;
    if (x >= x1 || y >= y1) return;
    for (int k = 0; k < L.n; ++k) {
        float dx = (float)x - L.s[k].x, dy = (float)y - L.s[k].y, dz = (float)z - L.s[k].z;
        float dist = dx * dx + dy * dy + dz * dz;
        if (dist < L.s[k].r * L.s[k].r) {
            int i = g.idx(x, y, z);
            rho0[i] = 1.0f;
            rho1[i] = 1.0f;
        }
    }
}

// fillObstacle (smokeSimulation.cu:289-313): interior cells; each obstacle overwrites the
// cell, so the last one decides.  `first` marks the first chunk of obstacles.
__global__ void k_fill_obstacles(Grid g, uint8_t* __restrict__ s, ObstacleList L) {
    int x = 1 + blockIdx.x * BX + threadIdx.x;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    if (x >= g.nx - 1 || y >= g.ny - 1) return;
    uint8_t val = 2;
    for (int k = 0; k < L.n; ++k) {
        float dx = (float)x - L.o[k].x, dy = (float)y - L.o[k].y, dz = (float)z - L.o[k].z;
        float dist = dx * dx + dy * dy + dz * dz;
        val = (dist < L.o[k].r * L.o[k].r) ? 0 : 1;
    }
    if (val != 2) s[g.idx(x, y, z)] = val;
}

__global__ void k_build_flags(Grid g, const uint8_t* __restrict__ s, uint8_t* __restrict__ flags,
                              float* __restrict__ P) {
    int x = blockIdx.x * BX + threadIdx.x;
    int y = blockIdx.y * BY + threadIdx.y;
    int z = blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    int i = g.idx(x, y, z);
    unsigned f = s[i] ? F_SELF : 0u;
    if (x > 0 && s[i - 1]) f |= F_XM;
    if (x < g.nx - 1 && s[i + 1]) f |= F_XP;
    if (y > 0 && s[i - g.X]) f |= F_YM;
    if (y < g.ny - 1 && s[i + g.X]) f |= F_YP;
    if (z > 0 && s[i - g.XY]) f |= F_ZM;
    if (z < g.nz - 1 && s[i + g.XY]) f |= F_ZP;
    bool interior = x >= 1 && y >= 1 && z >= 1 && x <= g.nx - 2 && y <= g.ny - 2 && z <= g.nz - 2;
    if (interior && (f & F_SELF) && (f & F_NBRS)) f |= F_PROJ;
    flags[i] = (uint8_t)f;
    if (!(f & F_PROJ) && P) P[i] = 0.0f;
}

// ---- b: integrate (smokeSimulation.cu:315-329) + velocityConfinement (:331-352) ------------
// Both are pointwise on the shared staggered index, so one pass applies integrate then clamp.
__global__ void k_forcing(Grid g, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                          const float* __restrict__ rho, const uint8_t* __restrict__ flags, float dt,
                          float gravity, float alpha, float lim_sq, float lim, int clamp_mode) {
    int x = blockIdx.x * BX + threadIdx.x;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    int i = g.idx(x, y, z);
    uint8_t f = flags[i];
    float vt = v[i];
    if ((f & F_SELF) && (f & F_YM)) {
        float r = rho[i];
        float buoy = alpha * (r - 0.0f);
        vt = vt + (r * gravity * dt + buoy * dt);
        if (!(x >= 1 && z >= 1 && clamp_mode != 2)) v[i] = vt;
    }
    if (x >= 1 && z >= 1 && clamp_mode != 2) {
        float ut = u[i], wt = w[i];
        float len = ut * ut + vt * vt + wt * wt;
        if (clamp_mode == 0) {
            if (len * dt > lim_sq) {
                float s = lim_sq / (len * dt);
                u[i] = ut * s;
                vt = vt * s;
                w[i] = wt * s;
            }
        } else if (len > lim * lim) {
            float s = lim / sqrtf(len);
            u[i] = ut * s;
            vt = vt * s;
            w[i] = wt * s;
        }
        v[i] = vt;
    }
}

// ---- d (reference scheme): divergence kernel (smokeSimulation.cu:356-394) ------------------
// Colour k covers cells with (x+y+z+k) even; one thread per cell of the colour, consecutive
// threads on consecutive same-colour cells of a row.  Within a colour no two cells share a
// face, so the in-place face updates are race-free.
__global__ void k_project_velocity(Grid g, float* __restrict__ u, float* __restrict__ v,
                                   float* __restrict__ w, const uint8_t* __restrict__ flags,
                                   int colour, double omega) {
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    int x = 1 + ((1 + y + z + colour) & 1) + 2 * (int)(blockIdx.x * BX + threadIdx.x);
    if (x > g.nx - 2 || y > g.ny - 2) return;
    int i = g.idx(x, y, z);
    uint8_t f = flags[i];
    if (!(f & F_SELF)) return;
    int sx0 = (f >> 1) & 1, sx1 = (f >> 2) & 1, sy0 = (f >> 3) & 1, sy1 = (f >> 4) & 1,
        sz0 = (f >> 5) & 1, sz1 = (f >> 6) & 1;
    int acc = sx0 + sx1 + sy0 + sy1 + sz0 + sz1;
    if (acc == 0) return;
    const int ix = i + 1, iy = i + g.X, iz = i + g.XY;
    float div = -u[i] + u[ix] + -v[i] + v[iy] + -w[i] + w[iz];
    float q = (-div) / (float)acc;
    float pt = __double2float_rn((double)q * omega);
    u[i] = u[i] - pt * (float)sx0;
    u[ix] = u[ix] + pt * (float)sx1;
    v[i] = v[i] - pt * (float)sy0;
    v[iy] = v[iy] + pt * (float)sy1;
    w[i] = w[i] - pt * (float)sz0;
    w[iz] = w[iz] + pt * (float)sz1;
}

// ---- a: velocityAdvectionU/V/W (smokeSimulation.cu:527-615), fused -------------------------
// One thread per staggered index computes whichever of the three face updates apply there.
__global__ void k_advect_velocity(Grid g, const float* __restrict__ u0, const float* __restrict__ v0,
                                  const float* __restrict__ w0, float* __restrict__ u1,
                                  float* __restrict__ v1, float* __restrict__ w1,
                                  const uint8_t* __restrict__ flags, float dt) {
    int x = 1 + blockIdx.x * BX + threadIdx.x;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    const int i = g.idx(x, y, z);
    const uint8_t f = flags[i];
    if (!(f & F_SELF)) return;
    const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2, inz = z <= g.nz - 2;
    if (iny && inz && (f & F_XM)) {
        float xt = (float)x, yt = (float)y + 0.5f, zt = (float)z + 0.5f;
        float uu = u0[i];
        float vv = avgV(v0, g, i);
        float ww = avgW(w0, g, i);
        xt = xt - dt * uu;
        yt = yt - dt * vv;
        zt = zt - dt * ww;
        u1[i] = sample_ref(u0, g, xt, yt, zt, 0.0f, 0.5f, 0.5f);
    }
    if (inx && inz && (f & F_YM)) {
        float xt = (float)x + 0.5f, yt = (float)y, zt = (float)z + 0.5f;
        float uu = avgU(u0, g, i);
        float vv = v0[i];
        float ww = avgW(w0, g, i);
        xt = xt - dt * uu;
        yt = yt - dt * vv;
        zt = zt - dt * ww;
        v1[i] = sample_ref(v0, g, xt, yt, zt, 0.5f, 0.0f, 0.5f);
    }
    if (inx && iny && (f & F_ZM)) {
        float xt = (float)x + 0.5f, yt = (float)y + 0.5f, zt = (float)z;
        float uu = avgU(u0, g, i);
        float vv = avgV(v0, g, i);
        float ww = w0[i];
        xt = xt - dt * uu;
        yt = yt - dt * vv;
        zt = zt - dt * ww;
        w1[i] = sample_ref(w0, g, xt, yt, zt, 0.5f, 0.5f, 0.0f);
    }
}

// ---- a: advectSmoke (smokeSimulation.cu:617-638) --------------------------------------------
// Uses the NEW velocities.  The reference evaluates the backtrace x + 0.5 - u*dt in double
// (int + double literal) and rounds to float.  With a = x + 0.5 (exact, lowest bit 2^-1) and
// b = u*dt (a float), the exact a - b needs at most max(e_a - e_b, 0) + 24 bits, so it is exact
// in double unless |b| < a*2^-29; then a - b lies strictly inside a's float rounding interval,
// in double too.  Either way float(double(a) - double(b)) equals the single-rounded float
// subtraction, which avoids GB300's slow FP64 pipe (the golden-vector tests pin this).
__global__ void k_advect_density(Grid g, const float* __restrict__ r0, float* __restrict__ r1,
                                 const float* __restrict__ u, const float* __restrict__ v,
                                 const float* __restrict__ w, const uint8_t* __restrict__ flags,
                                 float dt) {
    int x = 1 + blockIdx.x * BX + threadIdx.x;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    if (x > g.nx - 2 || y > g.ny - 2) return;
    const int i = g.idx(x, y, z);
    if (!(flags[i] & F_SELF)) return;
    float ut = (u[i] + u[i + 1]) / 2.0f;
    float vt = (v[i] + v[i + g.X]) / 2.0f;
    float wt = (w[i] + w[i + g.XY]) / 2.0f;
    float xt = __fsub_rn((float)x + 0.5f, ut * dt);
    float yt = __fsub_rn((float)y + 0.5f, vt * dt);
    float zt = __fsub_rn((float)z + 0.5f, wt * dt);
    r1[i] = sample_ref(r0, g, xt, yt, zt, 0.5f, 0.5f, 0.5f);
}

// max |div u| over projectable cells (post-projection diagnostic).
__global__ void k_div_max(Grid g, const float* __restrict__ u, const float* __restrict__ v,
                          const float* __restrict__ w, const uint8_t* __restrict__ flags,
                          StepStatus* status) {
    int x = 1 + blockIdx.x * BX + threadIdx.x;
    int y = 1 + blockIdx.y * BY + threadIdx.y;
    int z = 1 + blockIdx.z;
    float m = 0.0f;
    if (x <= g.nx - 2 && y <= g.ny - 2) {
        int i = g.idx(x, y, z);
        if (flags[i] & F_PROJ) {
            float div = -u[i] + u[i + 1] + -v[i] + v[i + g.X] + -w[i] + w[i + g.XY];
            m = fabsf(div);
        }
    }
    block_max_to(__float_as_uint(m), &status->div_bits);
}

}  // namespace

// ---- launchers ------------------------------------------------------------------------------

void launch_emit_boxes(const Grid& g, float* rho0, float* rho1, float* v_now, const BoxObj* boxes,
                       int nb, cudaStream_t st) {
    for (int base = 0; base < nb; base += MAX_OBJ_PER_LAUNCH) {
        BoxList L;
        L.n = nb - base < MAX_OBJ_PER_LAUNCH ? nb - base : MAX_OBJ_PER_LAUNCH;
        int x0 = g.nx, y0 = g.ny, z0 = g.nz, x1 = 0, y1 = 0, z1 = 0;
        for (int k = 0; k < L.n; ++k) {
            BoxObj b = boxes[base + k];
            b.x0 = b.x0 < 0 ? 0 : b.x0; b.y0 = b.y0 < 0 ? 0 : b.y0; b.z0 = b.z0 < 0 ? 0 : b.z0;
            b.x1 = b.x1 > g.nx ? g.nx : b.x1; b.y1 = b.y1 > g.ny ? g.ny : b.y1;
            b.z1 = b.z1 > g.nz ? g.nz : b.z1;
            L.b[k] = b;
            if (b.x0 < b.x1 && b.y0 < b.y1 && b.z0 < b.z1) {
                x0 = b.x0 < x0 ? b.x0 : x0; y0 = b.y0 < y0 ? b.y0 : y0; z0 = b.z0 < z0 ? b.z0 : z0;
                x1 = b.x1 > x1 ? b.x1 : x1; y1 = b.y1 > y1 ? b.y1 : y1; z1 = b.z1 > z1 ? b.z1 : z1;
            }
        }
        if (x0 >= x1 || y0 >= y1 || z0 >= z1) continue;
        k_emit_boxes<<<grid3(x1 - x0, y1 - y0, z1 - z0), dim3(BX, BY), 0, st>>>(g, rho0, rho1, v_now,
                                                                                L, x0, y0, z0, x1, y1);
    }
}

void launch_fill_smoke(const Grid& g, float* rho0, float* rho1, const SphereObj* sp, int ns,
                       cudaStream_t st) {
    for (int base = 0; base < ns; base += MAX_OBJ_PER_LAUNCH) {
        SphereList L;
        L.n = ns - base < MAX_OBJ_PER_LAUNCH ? ns - base : MAX_OBJ_PER_LAUNCH;
        // union bounding box (one cell of margin), clipped to the interior [1, n-2]
        double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
        for (int k = 0; k < L.n; ++k) {
            L.s[k] = sp[base + k];
            double c[3] = {L.s[k].x, L.s[k].y, L.s[k].z};
            double r = L.s[k].r < 0 ? -L.s[k].r : L.s[k].r;
            for (int a = 0; a < 3; ++a) {
                lo[a] = c[a] - r - 1 < lo[a] ? c[a] - r - 1 : lo[a];
                hi[a] = c[a] + r + 1 > hi[a] ? c[a] + r + 1 : hi[a];
            }
        }
        int n3[3] = {g.nx, g.ny, g.nz};
        int a0[3], a1[3];
        bool empty = false;
        for (int a = 0; a < 3; ++a) {
            double l = lo[a] < 1 ? 1 : lo[a];
            double h = hi[a] > n3[a] - 2 ? n3[a] - 2 : hi[a];
            if (!(l <= h)) { empty = true; break; }
            a0[a] = (int)l;
            a1[a] = (int)h + 1;
        }
        if (empty) continue;
        k_fill_smoke<<<grid3(a1[0] - a0[0], a1[1] - a0[1], a1[2] - a0[2]), dim3(BX, BY), 0, st>>>(
            g, rho0, rho1, L, a0[0], a0[1], a0[2], a1[0], a1[1]);
    }
}

void launch_fill_obstacles(const Grid& g, uint8_t* s, const ObstacleObj* ob, int no, cudaStream_t st) {
    if (no <= 0 || g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    // Only the last obstacle decides a cell (each one overwrites every interior cell).
    ObstacleList L;
    L.n = 1;
    L.o[0] = ob[no - 1];
    k_fill_obstacles<<<grid3(g.nx - 2, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, s, L);
}

void launch_build_flags(const Grid& g, const uint8_t* s, uint8_t* flags, float* P, cudaStream_t st) {
    k_build_flags<<<grid3(g.nx, g.ny, g.nz), dim3(BX, BY), 0, st>>>(g, s, flags, P);
}

void launch_forcing(const Grid& g, float* u, float* v, float* w, const float* rho,
                    const uint8_t* flags, float dt, float gravity, float buoyancy, float clamp_const,
                    int clamp_mode, cudaStream_t st) {
    if (g.ny < 2) return;
    float lim_sq = clamp_const * clamp_const;
    k_forcing<<<grid3(g.nx, g.ny - 1, g.nz), dim3(BX, BY), 0, st>>>(
        g, u, v, w, rho, flags, dt, gravity, buoyancy, lim_sq, clamp_const, clamp_mode);
}

void launch_project_velocity(const Grid& g, float* u, float* v, float* w, const uint8_t* flags,
                             int colour, double omega, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    int half = (g.nx - 2 + 1) / 2;
    k_project_velocity<<<grid3(half, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, u, v, w, flags,
                                                                                 colour, omega);
}

void launch_advect_velocity(const Grid& g, const float* u0, const float* v0, const float* w0,
                            float* u1, float* v1, float* w1, const uint8_t* flags, float dt,
                            cudaStream_t st) {
    if (g.nx < 2 || g.ny < 2 || g.nz < 2) return;
    k_advect_velocity<<<grid3(g.nx - 1, g.ny - 1, g.nz - 1), dim3(BX, BY), 0, st>>>(
        g, u0, v0, w0, u1, v1, w1, flags, dt);
}

void launch_advect_density(const Grid& g, const float* r0, float* r1, const float* u1,
                           const float* v1, const float* w1, const uint8_t* flags, float dt,
                           cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    k_advect_density<<<grid3(g.nx - 2, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, r0, r1, u1, v1,
                                                                                   w1, flags, dt);
}

void launch_div_max(const Grid& g, const float* u, const float* v, const float* w,
                    const uint8_t* flags, StepStatus* status, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    k_div_max<<<grid3(g.nx - 2, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, u, v, w, flags, status);
}

}  // namespace smk
