// Stage kernels shared by both projection schemes, plus the reference-scheme projection.
//
// Each kernel restates one stage of the reference step (project/smokeSimulation.cu) with the
// reference's exact floating-point expression order, on the library's pitched layout
// (common.cuh) and with x-contiguous, coalesced thread mapping (one thread per x, a warp per
// row segment) instead of the reference's 8x8x8 cubes.  The per-step stage bodies live in
// stage_bodies.cuh, shared with the grouped (batch) kernels.
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "stage_bodies.cuh"

namespace smk {

namespace {

constexpr int BX = SB_BX, BY = SB_BY;
constexpr int ADV_ZC = 4;  // z planes per advection block

inline dim3 grid3(int rx, int ry, int rz) {
    return dim3((unsigned)((rx + BX - 1) / BX), (unsigned)((ry + BY - 1) / BY), (unsigned)rz);
}

constexpr int MAX_OBJ_PER_LAUNCH = 64;
struct SphereList { int n; SphereObj s[MAX_OBJ_PER_LAUNCH]; };
struct ObstacleList { int n; ObstacleObj o[MAX_OBJ_PER_LAUNCH]; };
struct BoxList { int n; BoxObj b[MAX_OBJ_PER_LAUNCH]; };

// ---- a4: emitters and obstacles ---------------------------------------------------------------

template <typename T, typename Tv>
__global__ void k_emit_boxes(Grid g, T* __restrict__ rho0, T* __restrict__ rho1,
                             Tv* __restrict__ v_now, const __grid_constant__ BoxList L, int x0,
                             int y0, int z0, int x1, int y1, int z1) {
    body_emit_boxes(g, rho0, rho1, v_now, L.b, L.n, x0, y0, z0, x1, y1, z1, blockIdx);
}

template <typename T>
__global__ void k_fill_smoke(Grid g, T* __restrict__ rho0, T* __restrict__ rho1,
                             const __grid_constant__ SphereList L, int x0, int y0, int z0, int x1,
                             int y1, int z1) {
    body_fill_smoke(g, rho0, rho1, L.s, L.n, x0, y0, z0, x1, y1, z1, blockIdx);
}

// A cell the obstacle makes solid: interior, and inside its sphere by fillObstacle's test.
__device__ __forceinline__ bool obstacle_cell(const Grid& g, const ObstacleObj& o, int x, int y, int z) {
    if (x < 1 || y < 1 || z < 1 || x > g.nx - 2 || y > g.ny - 2 || z > g.nz - 2) return false;
    const float dx = (float)x - o.x, dy = (float)y - o.y, dz = (float)z - o.z;
    const float dist = dx * dx + dy * dy + dz * dz;
    return dist < o.r * o.r;
}

// Moving-obstacle boundary: every face with a cell of obstacle `o` on either side takes the
// obstacle's velocity component.  One thread per staggered index (x, y, z) <= (nx, ny, nz).
template <typename Tv>
__global__ void k_obstacle_velocity(Grid g, Tv* __restrict__ u, Tv* __restrict__ v, Tv* __restrict__ w,
                                    ObstacleObj o) {
    const int x = blockIdx.x * BX + threadIdx.x;
    const int y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    if (x > g.nx || y > g.ny || z > g.nz) return;
    const int i = g.idx(x, y, z);
    const bool c = obstacle_cell(g, o, x, y, z);
    if (x >= 1 && x <= g.nx - 1 && y < g.ny && z < g.nz && (c || obstacle_cell(g, o, x - 1, y, z))) stv(u, i, o.vx);
    if (y >= 1 && y <= g.ny - 1 && x < g.nx && z < g.nz && (c || obstacle_cell(g, o, x, y - 1, z))) stv(v, i, o.vy);
    if (z >= 1 && z <= g.nz - 1 && x < g.nx && y < g.ny && (c || obstacle_cell(g, o, x, y, z - 1))) stv(w, i, o.vz);
}

// fillObstacle (smokeSimulation.cu:289-313): interior cells; each obstacle overwrites the
// cell, so the last one decides.
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

// The pressure is left alone: the rhs pass zeroes it on the cells that are not projectable before
// a solve reads it, so the last solution keeps its values until then (the warm start's history
// saves it as the solve left it).
__global__ void k_build_flags(Grid g, const uint8_t* __restrict__ s, uint8_t* __restrict__ flags) {
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
}

// ---- b: integrate (smokeSimulation.cu:315-329) + velocityConfinement (:331-352) ------------
template <typename Tv, typename T>
__global__ void k_forcing(Grid g, Tv* __restrict__ u, Tv* __restrict__ v, Tv* __restrict__ w,
                          const T* __restrict__ rho, const uint8_t* __restrict__ flags, float dt,
                          float gravity, float alpha, float lim_sq, float lim, int clamp_mode) {
    body_forcing(g, u, v, w, rho, flags, dt, gravity, alpha, lim_sq, lim, clamp_mode, blockIdx);
}

// Forcing with four consecutive x per thread (vector loads and stores; body_forcing_x4).
template <typename Tv, typename T>
__global__ void __launch_bounds__(256) k_forcing_x4(Grid g, Tv* __restrict__ u, Tv* __restrict__ v,
                                                    Tv* __restrict__ w, const T* __restrict__ rho,
                                                    const uint8_t* __restrict__ flags, float dt, float gravity,
                                                    float alpha, float lim_sq, float lim, int clamp_mode) {
    body_forcing_x4(g, u, v, w, rho, flags, dt, gravity, alpha, lim_sq, lim, clamp_mode,
                    4 * ((int)blockIdx.x * 32 + (int)threadIdx.x), 1 + (int)blockIdx.y * 8 + (int)threadIdx.y,
                    (int)blockIdx.z);
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

// ---- a: advectSmoke (:617-638); the velocity advection is kernels_advect_tile.cu -------------
// The density advection is a latency-bound gather: the register cap keeps 8 blocks of 8 warps
// per SM (32 registers).  Each block walks ADV_ZC consecutive planes in ascending z: the planes
// a cell's sample reads overlap the next cell's and stay in L1 between them (3% faster than one
// plane per block at 256^3).
template <typename T, typename Tv>
__global__ void __launch_bounds__(BX * BY, 8) k_advect_density(Grid g, const T* __restrict__ r0, T* __restrict__ r1,
                                 const Tv* __restrict__ u, const Tv* __restrict__ v,
                                 const Tv* __restrict__ w, const uint8_t* __restrict__ flags,
                                 float dt, int z0, int z1) {
    for (int k = 0; k < ADV_ZC; ++k) {
        const int zz = z0 + (int)blockIdx.z * ADV_ZC + k;
        if (zz >= z1) break;
        body_advect_density(g, r0, r1, u, v, w, flags, dt, make_uint3(blockIdx.x, blockIdx.y, (unsigned)zz));
    }
}

// The BF16 projection with four consecutive x per thread (body_project_bf16_x4).
__global__ void __launch_bounds__(256) k_project_bf16_x4(Grid g, __nv_bfloat16* __restrict__ u,
                                                         __nv_bfloat16* __restrict__ v, __nv_bfloat16* __restrict__ w,
                                                         const float* __restrict__ P0, const float* __restrict__ P1,
                                                         const int* __restrict__ pcur,
                                                         const uint8_t* __restrict__ flags, float* __restrict__ pu,
                                                         float* __restrict__ pv, float* __restrict__ pw) {
    const float* P = (pcur != nullptr && *pcur == 1) ? P1 : P0;
    body_project_bf16_x4(g, u, v, w, P, flags, pu, pv, pw, 4 * ((int)blockIdx.x * 32 + (int)threadIdx.x),
                         (int)blockIdx.y * 8 + (int)threadIdx.y, (int)blockIdx.z);
}

__global__ void k_project_bf16(Grid g, __nv_bfloat16* __restrict__ u, __nv_bfloat16* __restrict__ v,
                               __nv_bfloat16* __restrict__ w, const float* __restrict__ P0,
                               const float* __restrict__ P1, const int* __restrict__ pcur,
                               const uint8_t* __restrict__ flags, float* __restrict__ pu,
                               float* __restrict__ pv, float* __restrict__ pw) {
    body_project_bf16(g, u, v, w, P0, P1, pcur, flags, pu, pv, pw, blockIdx);
}

__global__ void k_bf16_to_f32(const __nv_bfloat16* __restrict__ a, float* __restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = __bfloat162float(a[i]);
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, __nv_bfloat16* __restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16_rn(a[i]);
}

// max |div u| over projectable cells (post-projection diagnostic).
__global__ void k_div_max(Grid g, const float* __restrict__ u, const float* __restrict__ v,
                          const float* __restrict__ w, const uint8_t* __restrict__ flags,
                          StepStatus* status) {
    body_div_max(g, u, v, w, flags, status, blockIdx);
}

}  // namespace

// ---- launchers ------------------------------------------------------------------------------

template <typename T, typename Tv>
void launch_emit_boxes(const Grid& g, T* rho0, T* rho1, Tv* v_now, const BoxObj* boxes,
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
                                                                                L, x0, y0, z0, x1, y1, z1);
    }
}

// Union bounding box (one cell of margin) of a list of spheres, clipped to the interior
// [1, n-2]; returns false when empty.
bool sphere_bounds(const Grid& g, const SphereObj* sp, int ns, int a0[3], int a1[3]) {
    double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
    for (int k = 0; k < ns; ++k) {
        double c[3] = {sp[k].x, sp[k].y, sp[k].z};
        double r = sp[k].r < 0 ? -sp[k].r : sp[k].r;
        for (int a = 0; a < 3; ++a) {
            lo[a] = c[a] - r - 1 < lo[a] ? c[a] - r - 1 : lo[a];
            hi[a] = c[a] + r + 1 > hi[a] ? c[a] + r + 1 : hi[a];
        }
    }
    int n3[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; ++a) {
        double l = lo[a] < 1 ? 1 : lo[a];
        double h = hi[a] > n3[a] - 2 ? n3[a] - 2 : hi[a];
        if (!(l <= h)) return false;
        a0[a] = (int)l;
        a1[a] = (int)h + 1;
    }
    return true;
}

template <typename T>
void launch_fill_smoke(const Grid& g, T* rho0, T* rho1, const SphereObj* sp, int ns,
                       cudaStream_t st) {
    for (int base = 0; base < ns; base += MAX_OBJ_PER_LAUNCH) {
        SphereList L;
        L.n = ns - base < MAX_OBJ_PER_LAUNCH ? ns - base : MAX_OBJ_PER_LAUNCH;
        for (int k = 0; k < L.n; ++k) L.s[k] = sp[base + k];
        int a0[3], a1[3];
        if (!sphere_bounds(g, L.s, L.n, a0, a1)) continue;
        k_fill_smoke<<<grid3(a1[0] - a0[0], a1[1] - a0[1], a1[2] - a0[2]), dim3(BX, BY), 0, st>>>(
            g, rho0, rho1, L, a0[0], a0[1], a0[2], a1[0], a1[1], a1[2]);
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

template <typename Tv>
void launch_obstacle_velocity(const Grid& g, Tv* u, Tv* v, Tv* w, const ObstacleObj& last, cudaStream_t st) {
    k_obstacle_velocity<Tv><<<grid3(g.nx + 1, g.ny + 1, g.nz + 1), dim3(BX, BY), 0, st>>>(g, u, v, w, last);
}
template void launch_obstacle_velocity<float>(const Grid&, float*, float*, float*, const ObstacleObj&, cudaStream_t);
template void launch_obstacle_velocity<__nv_bfloat16>(const Grid&, __nv_bfloat16*, __nv_bfloat16*, __nv_bfloat16*,
                                                      const ObstacleObj&, cudaStream_t);

void launch_build_flags(const Grid& g, const uint8_t* s, uint8_t* flags, cudaStream_t st) {
    k_build_flags<<<grid3(g.nx, g.ny, g.nz), dim3(BX, BY), 0, st>>>(g, s, flags);
}

template <typename Tv, typename T>
void launch_forcing(const Grid& g, Tv* u, Tv* v, Tv* w, const T* rho,
                    const uint8_t* flags, float dt, float gravity, float buoyancy, float clamp_const,
                    int clamp_mode, cudaStream_t st, bool vec) {
    if (g.ny < 2) return;
    float lim_sq = clamp_const * clamp_const;
    if (vec && vec4_layout_of<Tv>(g, {u, v, w}, {}, flags) && vec4_layout_of<T>(g, {rho}, {}, flags)) {
        const int groups = (g.nx + 3) / 4;
        k_forcing_x4<Tv, T><<<dim3((unsigned)((groups + 31) / 32), (unsigned)((g.ny - 1 + 7) / 8), (unsigned)g.nz),
                              dim3(32, 8), 0, st>>>(g, u, v, w, rho, flags, dt, gravity, buoyancy, lim_sq,
                                                    clamp_const, clamp_mode);
        return;
    }
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

template <typename T, typename Tv>
void launch_advect_density(const Grid& g, const T* r0, T* r1, const Tv* u1,
                           const Tv* v1, const Tv* w1, const uint8_t* flags, float dt,
                           cudaStream_t st, int z0, int z1) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    if (z1 < 0 || z1 > g.nz - 2) z1 = g.nz - 2;
    if (z0 < 0) z0 = 0;
    if (z1 <= z0) return;
    k_advect_density<<<grid3(g.nx - 2, g.ny - 2, (z1 - z0 + ADV_ZC - 1) / ADV_ZC), dim3(BX, BY), 0, st>>>(
        g, r0, r1, u1, v1, w1, flags, dt, z0, z1);
}

void launch_div_max(const Grid& g, const float* u, const float* v, const float* w,
                    const uint8_t* flags, StepStatus* status, cudaStream_t st) {
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return;
    k_div_max<<<grid3(g.nx - 2, g.ny - 2, g.nz - 2), dim3(BX, BY), 0, st>>>(g, u, v, w, flags, status);
}

void launch_project_bf16(const Grid& g, __nv_bfloat16* u, __nv_bfloat16* v, __nv_bfloat16* w,
                         const float* P0, const float* P1, const int* pcur, const uint8_t* flags,
                         float* pu, float* pv, float* pw, cudaStream_t st, bool vec) {
    if (vec && vec4_layout_of<__nv_bfloat16>(g, {u, v, w}, {P0, P1, pu, pv, pw}, flags)) {
        const int groups = (g.nx + 1 + 3) / 4;
        k_project_bf16_x4<<<dim3((unsigned)((groups + 31) / 32), (unsigned)((g.ny + 1 + 7) / 8), (unsigned)(g.nz + 1)),
                            dim3(32, 8), 0, st>>>(g, u, v, w, P0, P1, pcur, flags, pu, pv, pw);
        return;
    }
    k_project_bf16<<<grid3(g.nx + 1, g.ny + 1, g.nz + 1), dim3(BX, BY), 0, st>>>(g, u, v, w, P0, P1, pcur,
                                                                               flags, pu, pv, pw);
}

void launch_convert(const __nv_bfloat16* src, float* dst, size_t n, cudaStream_t st) {
    k_bf16_to_f32<<<(unsigned)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536), 256, 0, st>>>(src, dst, n);
}

void launch_convert(const float* src, __nv_bfloat16* dst, size_t n, cudaStream_t st) {
    k_f32_to_bf16<<<(unsigned)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536), 256, 0, st>>>(src, dst, n);
}

// explicit instantiations: FP32 storage and BF16 storage
template void launch_emit_boxes<float, float>(const Grid&, float*, float*, float*, const BoxObj*, int,
                                              cudaStream_t);
template void launch_emit_boxes<__nv_bfloat16, __nv_bfloat16>(const Grid&, __nv_bfloat16*, __nv_bfloat16*,
                                                              __nv_bfloat16*, const BoxObj*, int, cudaStream_t);
template void launch_emit_boxes<float, __nv_bfloat16>(const Grid&, float*, float*, __nv_bfloat16*,
                                                      const BoxObj*, int, cudaStream_t);
template void launch_fill_smoke<float>(const Grid&, float*, float*, const SphereObj*, int, cudaStream_t);
template void launch_fill_smoke<__nv_bfloat16>(const Grid&, __nv_bfloat16*, __nv_bfloat16*, const SphereObj*,
                                               int, cudaStream_t);
template void launch_forcing<float, float>(const Grid&, float*, float*, float*, const float*, const uint8_t*,
                                           float, float, float, float, int, cudaStream_t, bool);
template void launch_forcing<__nv_bfloat16, __nv_bfloat16>(const Grid&, __nv_bfloat16*, __nv_bfloat16*,
                                                           __nv_bfloat16*, const __nv_bfloat16*, const uint8_t*,
                                                           float, float, float, float, int, cudaStream_t, bool);
template void launch_forcing<__nv_bfloat16, float>(const Grid&, __nv_bfloat16*, __nv_bfloat16*, __nv_bfloat16*,
                                                   const float*, const uint8_t*, float, float, float, float, int,
                                                   cudaStream_t, bool);
template void launch_advect_density<float, float>(const Grid&, const float*, float*, const float*,
                                                  const float*, const float*, const uint8_t*, float,
                                                  cudaStream_t, int, int);
template void launch_advect_density<float, __nv_bfloat16>(const Grid&, const float*, float*,
                                                          const __nv_bfloat16*, const __nv_bfloat16*,
                                                          const __nv_bfloat16*, const uint8_t*, float,
                                                          cudaStream_t, int, int);
template void launch_advect_density<__nv_bfloat16, __nv_bfloat16>(const Grid&, const __nv_bfloat16*,
                                                                  __nv_bfloat16*, const __nv_bfloat16*,
                                                                  const __nv_bfloat16*, const __nv_bfloat16*,
                                                                  const uint8_t*, float, cudaStream_t, int, int);

}  // namespace smk
