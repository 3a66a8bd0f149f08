// Grouped kernels of a batch step: one persistent launch per stage over every grid (group.h).
//
//   k_group_objects     emitters (boxes, then spheres) of every grid
//   k_group_forcing     integrate + clamp
//   k_group_project     the whole projection as ONE cooperative kernel: b and the pressure
//                       start, every red-black colour pass of every grid with the per-grid
//                       tolerance rule, the gradient subtract (or the BF16 projection), and
//                       max |div u|; phases are separated by a bounded grid barrier
//   k_group_adv_vel     velocity advection
//   k_group_adv_rho     density advection
// The grid-stride kernels are sized to the resident CTAs of the device; every tile runs the
// stage body of the single-grid kernel, so a grid's results are the same alone and batched.
//
// Tolerance rule (the single-grid sweep loop's): at the start of check group k (sweep k*G) a
// grid whose residual recorded at the start of group k-1 is within tolerance is done; any other
// grid records max |r| of its current pressure for group k and runs the group's passes.  Every
// CTA makes the same decision from the same recorded residuals (written before a barrier), so
// all CTAs agree on the set of active grids without further communication.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "common.cuh"
#include "group.h"
#include "kernels.h"
#include "sim_internal.h"
#include "stage_bodies.cuh"

namespace smk {

namespace {

constexpr unsigned long long GROUP_WAIT_NS = 2000000000ull;  // a barrier wait gives up after 2 s

// Testing (smk_inject_barrier_timeout): the next cooperative projection launch made outside a
// capture gets a skipped arrival and a short wait; its barrier state is remembered for the report.
std::mutex g_inject_mutex;
int g_inject_barrier = 0;
unsigned long long g_inject_wait_ns = 0;
GroupSync* g_injected_sync = nullptr;
int g_injected_ctas = 0;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int tid256() { return (int)threadIdx.x + SB_BX * (int)threadIdx.y; }

// Block index of tile `local` of a 64 x 4 block launch over an rx x ry x rz range.
__device__ __forceinline__ uint3 tile_bid(int local, int rx, int ry) {
    const int nbx = group_div_up(rx, SB_BX), nby = group_div_up(ry, SB_BY);
    uint3 b;
    b.x = (unsigned)(local % nbx);
    b.y = (unsigned)((local / nbx) % nby);
    b.z = (unsigned)(local / (nbx * nby));
    return b;
}

// Group of 4 x, row and plane of this thread in tile `local` of a 4-wide stage (group_x4_tiles).
__device__ __forceinline__ void x4_coords(int local, int gx, int ry, int y0, int z0, int& x, int& y, int& z) {
    const int nbx = group_div_up(gx, GX4_GX), nby = group_div_up(ry, GX4_GY);
    const int t = tid256();
    x = 4 * ((local % nbx) * GX4_GX + t % GX4_GX);
    y = y0 + ((local / nbx) % nby) * GX4_GY + t / GX4_GX;
    z = z0 + local / (nbx * nby);
}

// f(j, local) for every tile of `stage` this CTA owns (grid-stride over the batch's tiles).
// With `mask` (shared memory, one byte per grid), grids whose byte has none of the bits
// `need` are skipped as a whole.  j is uniform over the CTA, so f may contain block barriers.
template <class F>
__device__ __forceinline__ void for_tiles(const GroupArgs& a, int stage, const uint8_t* mask, int need, F&& f) {
    const int* st = a.starts + stage * (a.n + 1);
    const int total = st[a.n];
    const int step = (int)gridDim.x;
    int j = 0;
    if ((int)blockIdx.x < total) {  // the grid of this CTA's first tile (binary search)
        int lo = 0, hi = a.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (st[mid] <= (int)blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        j = lo;
    }
    for (int t = (int)blockIdx.x; t < total; t += step) {
        while (st[j + 1] <= t) ++j;
        if (mask != nullptr && !(mask[j] & need)) {
            const int end = st[j + 1];
            t += ((end - t + step - 1) / step - 1) * step;  // the loop's += lands on the first t >= end
            continue;
        }
        f(j, t - st[j]);
    }
}

// ---- grid-stride stages ---------------------------------------------------------------------

template <typename T, typename Tv>
__device__ __forceinline__ void objects_cell(const GroupGrid& d, const GroupArgs& a, int x, int y, int z) {
    const Grid gg = d.g;
    if (x >= d.bx0 && x < d.bx1 && y >= d.by0 && y < d.by1 && z >= d.bz0 && z < d.bz1)
        cell_emit_boxes(gg, (T*)d.rho0, (T*)d.rho1, (Tv*)d.v_now, a.boxes + d.box0, d.nbox, x, y, z);
    if (x >= d.sx0 && x < d.sx1 && y >= d.sy0 && y < d.sy1 && z >= d.sz0 && z < d.sz1)
        cell_fill_smoke(gg, (T*)d.rho0, (T*)d.rho1, a.spheres + d.sph0, d.nsph, x, y, z);
}

__global__ void __launch_bounds__(GROUP_TILE) k_group_objects(const GroupArgs a) {
    for_tiles(a, GS_OBJECTS, nullptr, 0, [&](int j, int local) {
        const GroupGrid& d = a.grids[j];
        const uint3 bid = tile_bid(local, d.ox1 - d.ox0, d.oy1 - d.oy0);
        const int x = d.ox0 + (int)bid.x * SB_BX + (int)threadIdx.x;
        const int y = d.oy0 + (int)bid.y * SB_BY + (int)threadIdx.y;
        const int z = d.oz0 + (int)bid.z;
        if (x >= d.ox1 || y >= d.oy1 || z >= d.oz1) return;
        if (d.kind == GK_BF16) objects_cell<__nv_bfloat16, __nv_bfloat16>(d, a, x, y, z);
        else if (d.kind == GK_BF16_VEL) objects_cell<float, __nv_bfloat16>(d, a, x, y, z);
        else objects_cell<float, float>(d, a, x, y, z);
    });
}

__global__ void __launch_bounds__(GROUP_TILE) k_group_forcing(const GroupArgs a) {
    for_tiles(a, GS_FORCE, nullptr, 0, [&](int j, int local) {
        const GroupGrid& d = a.grids[j];
        const Grid gg = d.g;  // in registers: the stores of the body cannot alias it
        int gx, ry, rz, y0, z0;
        typedef __nv_bfloat16 h;
        if (group_x4_extent(GS_FORCE, d, gx, ry, rz, y0, z0)) {
            int x, y, z;
            x4_coords(local, gx, ry, y0, z0, x, y, z);
            if (d.kind == GK_BF16)
                body_forcing_x4<h, h>(gg, (h*)d.u_now, (h*)d.v_now, (h*)d.w_now, (const h*)d.rho_now, d.flags, d.dt,
                                      d.gravity, d.alpha, d.lim_sq, d.lim, d.clamp_mode, x, y, z);
            else if (d.kind == GK_BF16_VEL)
                body_forcing_x4<h, float>(gg, (h*)d.u_now, (h*)d.v_now, (h*)d.w_now, (const float*)d.rho_now,
                                          d.flags, d.dt, d.gravity, d.alpha, d.lim_sq, d.lim, d.clamp_mode, x, y, z);
            else
                body_forcing_x4<float, float>(gg, (float*)d.u_now, (float*)d.v_now, (float*)d.w_now,
                                              (const float*)d.rho_now, d.flags, d.dt, d.gravity, d.alpha, d.lim_sq,
                                              d.lim, d.clamp_mode, x, y, z);
            return;
        }
        const uint3 bid = tile_bid(local, d.g.nx, d.g.ny - 1);
        if (d.kind == GK_BF16)
            body_forcing<h, h>(gg, (h*)d.u_now, (h*)d.v_now, (h*)d.w_now, (const h*)d.rho_now, d.flags, d.dt,
                               d.gravity, d.alpha, d.lim_sq, d.lim, d.clamp_mode, bid);
        else if (d.kind == GK_BF16_VEL)
            body_forcing<h, float>(gg, (h*)d.u_now, (h*)d.v_now, (h*)d.w_now, (const float*)d.rho_now, d.flags,
                                   d.dt, d.gravity, d.alpha, d.lim_sq, d.lim, d.clamp_mode, bid);
        else
            body_forcing<float, float>(gg, (float*)d.u_now, (float*)d.v_now, (float*)d.w_now,
                                       (const float*)d.rho_now, d.flags, d.dt, d.gravity, d.alpha, d.lim_sq,
                                       d.lim, d.clamp_mode, bid);
    });
}

// The advection tiles walk GROUP_ADV_ZC consecutive planes (the planes neighbouring cells'
// averages and samples share stay in L1); register caps of 8 CTAs per SM (32 registers: the
// velocity kernel spills 56 bytes there and the 64-grid batch step still runs 1.5% faster than
// with 5 CTAs and 48 registers).
__global__ void __launch_bounds__(GROUP_TILE, 8) k_group_adv_vel(const GroupArgs a) {
    for_tiles(a, GS_ADV_VEL, nullptr, 0, [&](int j, int local) {
        const GroupGrid& d = a.grids[j];
        const Grid gg = d.g;  // in registers: the stores of the body cannot alias it
        const uint3 bid = tile_bid(local, d.g.nx - 1, d.g.ny - 1);
        typedef __nv_bfloat16 h;
        for (int k = 0; k < GROUP_ADV_ZC; ++k) {
            const uint3 b = make_uint3(bid.x, bid.y, bid.z * GROUP_ADV_ZC + k);
            if ((int)b.z >= d.g.nz - 1) break;
            if (d.kind == GK_F32)
                body_advect_velocity<float, float>(gg, d.pu, d.pv, d.pw, (float*)d.u_past, (float*)d.v_past,
                                                   (float*)d.w_past, d.flags, d.dt, b);
            else
                body_advect_velocity<float, h>(gg, d.pu, d.pv, d.pw, (h*)d.u_past, (h*)d.v_past, (h*)d.w_past,
                                               d.flags, d.dt, b);
        }
    });
}

__global__ void __launch_bounds__(GROUP_TILE, 8) k_group_adv_rho(const GroupArgs a) {
    for_tiles(a, GS_ADV_RHO, nullptr, 0, [&](int j, int local) {
        const GroupGrid& d = a.grids[j];
        const Grid gg = d.g;  // in registers: the stores of the body cannot alias it
        const uint3 bid = tile_bid(local, d.g.nx - 2, d.g.ny - 2);
        typedef __nv_bfloat16 h;
        for (int k = 0; k < GROUP_ADV_ZC; ++k) {
            const uint3 b = make_uint3(bid.x, bid.y, bid.z * GROUP_ADV_ZC + k);
            if ((int)b.z >= d.g.nz - 2) break;
            if (d.kind == GK_BF16)
                body_advect_density<h, h>(gg, (const h*)d.rho_now, (h*)d.rho_past, (const h*)d.u_past,
                                          (const h*)d.v_past, (const h*)d.w_past, d.flags, d.dt, b);
            else if (d.kind == GK_BF16_VEL)
                body_advect_density<float, h>(gg, (const float*)d.rho_now, (float*)d.rho_past, (const h*)d.u_past,
                                              (const h*)d.v_past, (const h*)d.w_past, d.flags, d.dt, b);
            else
                body_advect_density<float, float>(gg, (const float*)d.rho_now, (float*)d.rho_past,
                                                  (const float*)d.u_past, (const float*)d.v_past,
                                                  (const float*)d.w_past, d.flags, d.dt, b);
        }
    });
}

// ---- cooperative projection -----------------------------------------------------------------

// Grid barrier over the cooperative launch (all CTAs co-resident).  Arrivals count up in one
// 64-bit counter that is zeroed before the launch; a CTA waits for `target` = its barrier
// number x gridDim.x.  The wait is bounded: after a.wait_ns (2 s unless a test shortened it) it
// raises `abort`, and a CTA that sees `abort` leaves too (each leaving CTA is counted in
// sync->left).  a.skip_barrier (testing, host-injected) makes CTA 0 not arrive at that barrier,
// so every wait on it runs out.  Returns false when the kernel must stop.
__device__ bool group_barrier(const GroupArgs& a, unsigned long long& target) {
    __shared__ int ok_s;
    __syncthreads();
    target += gridDim.x;
    if (tid256() == 0) {
        __threadfence();
        const bool skip = a.skip_barrier > 0 && blockIdx.x == 0 &&
                          target == (unsigned long long)a.skip_barrier * gridDim.x;
        if (!skip) atomicAdd(&a.sync->count, 1ull);
        int ok = 1;
        const unsigned long long t0 = global_ns();
        while (*(volatile unsigned long long*)&a.sync->count < target) {
            if (*(volatile int*)&a.sync->abort) {
                ok = 0;
                break;
            }
            if (global_ns() - t0 > a.wait_ns) {
                atomicExch(&a.sync->abort, 1);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        if (!ok) atomicAdd(&a.sync->left, 1);
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// A barrier gave up: flag every grid of the batch (the host reports it at the next sync).
__device__ void group_abort(const GroupArgs& a) {
    for (int j = tid256(); j < a.n; j += GROUP_TILE) atomicExch(a.grids[j].kerr, 1);
}

// Up to ZB cells of one same-colour (k, y) column of a colour pass: every load first, then the
// updates.  Nothing a colour pass reads is written during the pass (it writes only cells of
// its colour and reads the other colour's cells and the cell itself), so the loads of the ZB
// cells are independent of the stores and can all be in flight at once.  Cell q sits in plane
// z0 + q at x = xa + (par ^ (q & 1)); `count` cells are valid.  The arithmetic is cell_sweep's.
constexpr int ZB = 4;
__device__ __forceinline__ void sweep_column(const Grid& g, float* P, const float* b,
                                             const uint8_t* __restrict__ flags, const float* wacc, int base,
                                             int par, int xa, int count) {
    float c[ZB], sum[ZB], bb[ZB];
    int idx[ZB];
    uint8_t f[ZB];
#pragma unroll
    for (int q = 0; q < ZB; ++q) {
        const int pq = par ^ (q & 1);
        idx[q] = base + q * g.XY + pq;
        f[q] = 0;
        if (q < count && xa + pq <= g.nx - 2) {
            const int i = idx[q];
            f[q] = flags[i];
            sum[q] = ((P[i - 1] + P[i + 1]) + (P[i - g.X] + P[i + g.X])) + (P[i - g.XY] + P[i + g.XY]);
            c[q] = P[i];
            bb[q] = b[i];
        }
    }
#pragma unroll
    for (int q = 0; q < ZB; ++q) {
        if (f[q] & F_PROJ) {
            const int acc = __popc((unsigned)(f[q] & F_NBRS));
            const float r = fmaf(-(float)acc, c[q], bb[q] + sum[q]);
            P[idx[q]] = fmaf(wacc[acc], r, c[q]);
        }
    }
}

// max |residual| bits over up to ZB cells of an interior column (cell_resid's expression).
__device__ __forceinline__ unsigned resid_column(const Grid& g, const float* P, const float* b,
                                                 const uint8_t* __restrict__ flags, int i0, int count) {
    unsigned m = 0u;
    float v[ZB];
#pragma unroll
    for (int q = 0; q < ZB; ++q) v[q] = q < count ? cell_resid(g, P, b, flags, i0 + q * g.XY) : 0.0f;
#pragma unroll
    for (int q = 0; q < ZB; ++q) m = max(m, __float_as_uint(v[q]));
    return m;
}

// Per-grid byte of the active set (dynamic shared memory).
enum : uint8_t { GA_DONE = 1, GA_SWEEP = 2, GA_CHECK = 4 };

__global__ void __launch_bounds__(GROUP_TILE) k_group_project(const GroupArgs a) {
    extern __shared__ uint8_t gst[];
    const int tid = tid256();
    unsigned long long target = 0;
    for (int j = tid; j < a.n; j += GROUP_TILE) gst[j] = 0;

    if (!a.sweeps_only && (a.phases & GP_RHS)) {
        // this step's status words (zeroed by one CTA per grid), then b and the pressure start
        for (int j = (int)blockIdx.x; j < a.n; j += (int)gridDim.x) {
            unsigned* w = reinterpret_cast<unsigned*>(a.grids[j].status);
            for (int k = tid; k < a.grids[j].status_words; k += GROUP_TILE) w[k] = 0u;
        }
        for_tiles(a, GS_RHS, nullptr, 0, [&](int j, int local) {
            const GroupGrid& d = a.grids[j];
            const Grid gg = d.g;  // in registers: the stores of the body cannot alias it
            int gx, ry, rz, y0, z0;
            if (group_x4_extent(GS_RHS, d, gx, ry, rz, y0, z0)) {
                int x, y, z;
                x4_coords(local, gx, ry, y0, z0, x, y, z);
                if (d.kind == GK_F32)
                    body_rhs_x4<float>(gg, (const float*)d.u_now, (const float*)d.v_now, (const float*)d.w_now,
                                       d.flags, d.b, d.P, d.P2, d.pcur, d.warm, x, y, z, d.Ph, d.extrap);
                else
                    body_rhs_x4<__nv_bfloat16>(gg, (const __nv_bfloat16*)d.u_now, (const __nv_bfloat16*)d.v_now,
                                               (const __nv_bfloat16*)d.w_now, d.flags, d.b, d.P, d.P2, d.pcur,
                                               d.warm, x, y, z, d.Ph, d.extrap);
                return;
            }
            const uint3 bid = tile_bid(local, d.g.nx, d.g.ny);
            if (d.kind == GK_F32)
                body_rhs<float>(gg, (const float*)d.u_now, (const float*)d.v_now, (const float*)d.w_now, d.flags,
                                d.b, d.P, d.P2, d.pcur, d.warm, bid, d.Ph, d.extrap);
            else
                body_rhs<__nv_bfloat16>(gg, (const __nv_bfloat16*)d.u_now, (const __nv_bfloat16*)d.v_now,
                                        (const __nv_bfloat16*)d.w_now, d.flags, d.b, d.P, d.P2, d.pcur, d.warm,
                                        bid, d.Ph, d.extrap);
        });
        if (!group_barrier(a, target)) {
            group_abort(a);
            return;
        }
        // the solve runs in place in P: the next step's warm start reads it there
        if (blockIdx.x == 0)
            for (int j = tid; j < a.n; j += GROUP_TILE) *a.grids[j].pcur = 0;
    }

    // the solve waves run one after another; inside a wave every grid runs its own colour
    // passes and tolerance rule, pass by pass in lockstep with the wave's other grids
    const int nwaves = (a.phases & GP_SOLVE) ? a.nwaves : 0;
    for (int wave = 0; wave < nwaves; ++wave)
    for (int s = 0;; ++s) {
        // which grids sweep now, and which record a residual first (group starts)
        int act = 0, chk = 0;
        for (int j = tid; j < a.n; j += GROUP_TILE) {
            const GroupGrid& d = a.grids[j];
            uint8_t m = gst[j] & GA_DONE;
            if (!m && d.wave == wave && s < d.max_sweeps) {
                const bool check = !a.sweeps_only && d.tol > 0.0f && s % d.check_every == 0;
                m = check ? (GA_SWEEP | GA_CHECK) : GA_SWEEP;
            }
            gst[j] = m;
            act |= m & GA_SWEEP;
            chk |= m & GA_CHECK;
        }
        act = __syncthreads_or(act);
        chk = __syncthreads_or(chk);
        if (!act) break;

        if (chk) {
            int cur = -1;
            unsigned mb = 0u;
            auto flush = [&]() {
                const GroupGrid& d = a.grids[cur];
                block_max_to(mb, &d.status->rmax_bits[s / d.check_every]);
            };
            for_tiles(a, GS_RESID, gst, GA_CHECK, [&](int j, int local) {
                if (j != cur) {
                    if (cur >= 0) flush();
                    cur = j;
                    mb = 0u;
                }
                const GroupGrid& d = a.grids[j];
                const Grid g = d.g;  // in registers: the stores below cannot alias it
                const int tpp = group_interior_tpp(g);
                const int z0 = 1 + (local / tpp) * a.zslab;
                const int z1 = min(z0 + a.zslab, g.nz - 1);
                const int f = (local % tpp) * GROUP_TILE + tid;
                const int L = g.nx - 2;
                if (f < L * (g.ny - 2)) {
                    int i = g.idx(1 + f % L, 1 + f / L, z0);
                    for (int z = z0; z < z1; z += ZB, i += ZB * g.XY)
                        mb = max(mb, resid_column(g, d.P, d.b, d.flags, i, z1 - z));
                }
            });
            if (cur >= 0) flush();
            if (!group_barrier(a, target)) {
                group_abort(a);
                return;
            }
            // the tolerance rule: a grid whose residual is within tolerance ends its solve here,
            // before this group's sweeps
            act = 0;
            for (int j = tid; j < a.n; j += GROUP_TILE) {
                const GroupGrid& d = a.grids[j];
                uint8_t m = gst[j];
                if (m & GA_CHECK) {
                    const int k = s / d.check_every;
                    if (__uint_as_float(*(volatile unsigned*)&d.status->rmax_bits[k]) <= d.tol) {
                        m = GA_DONE;
                        if (blockIdx.x == 0) {
                            d.status->done = 1;
                            d.status->done_group = k;
                        }
                    }
                }
                gst[j] = m;
                act |= m & GA_SWEEP;
            }
            act = __syncthreads_or(act);
            if (!act) continue;  // every checked grid is done; the next pass finds none active
        }

        for (int colour = 0; colour < 2; ++colour) {
            for_tiles(a, GS_SWEEP, gst, GA_SWEEP, [&](int j, int local) {
                const GroupGrid& d = a.grids[j];
                const Grid g = d.g;  // in registers: the stores below cannot alias it
                const int tpp = group_sweep_tpp(g);
                const int z0 = 1 + (local / tpp) * a.zslab;
                const int z1 = min(z0 + a.zslab, g.nz - 1);
                const int f = (local % tpp) * GROUP_TILE + tid;
                const int H = (g.nx - 1) / 2;  // same-colour cells per row (rounded up)
                if (f < H * (g.ny - 2)) {
                    const int y = 1 + f / H;
                    // the colour's cell of this (k, y) column alternates between x and x +- 1 in z
                    const int xa = 1 + 2 * (f % H);
                    const int par = (1 + y + z0 + colour) & 1;  // ZB is even: same at every chunk start
                    int base = g.idx(xa, y, z0);
                    for (int z = z0; z < z1; z += ZB, base += ZB * g.XY)
                        sweep_column(g, d.P, d.b, d.flags, d.wacc, base, par, xa, z1 - z);
                }
            });
            if (!group_barrier(a, target)) {
                group_abort(a);
                return;
            }
        }
    }
    if (a.sweeps_only || !(a.phases & GP_FINISH)) return;

    // the pressure is the first buffer after the colour-pass solve (*pcur == 0), or where the
    // blocked solve's last launch left it
    for_tiles(a, GS_PROJECT, nullptr, 0, [&](int j, int local) {
        const GroupGrid& d = a.grids[j];
        const Grid gg = d.g;  // in registers: the stores of the body cannot alias it
        int gx, y0, z0, rx, ry, rz;
        if (group_x4_extent(GS_PROJECT, d, gx, ry, rz, y0, z0)) {
            int x, y, z;
            x4_coords(local, gx, ry, y0, z0, x, y, z);
            const float* P = (d.pcur != nullptr && *d.pcur == 1) ? d.P2 : d.P;
            if (d.kind == GK_F32)
                body_gradient_subtract_x4(gg, (float*)d.u_now, (float*)d.v_now, (float*)d.w_now, P, d.flags, x, y, z);
            else
                body_project_bf16_x4(gg, (__nv_bfloat16*)d.u_now, (__nv_bfloat16*)d.v_now, (__nv_bfloat16*)d.w_now, P,
                                     d.flags, d.pu, d.pv, d.pw, x, y, z);
            return;
        }
        group_extent(GS_PROJECT, d, rx, ry, rz);
        const uint3 bid = tile_bid(local, rx, ry);
        if (d.kind == GK_F32)
            body_gradient_subtract(gg, (float*)d.u_now, (float*)d.v_now, (float*)d.w_now, d.P, d.P2, d.pcur,
                                   d.flags, bid);
        else
            body_project_bf16(gg, (__nv_bfloat16*)d.u_now, (__nv_bfloat16*)d.v_now, (__nv_bfloat16*)d.w_now,
                              d.P, d.P2, d.pcur, d.flags, d.pu, d.pv, d.pw, bid);
    });

    if (a.starts[GS_DIV * (a.n + 1) + a.n] > 0) {
        if (!group_barrier(a, target)) {
            group_abort(a);
            return;
        }
        int cur = -1;
        unsigned mb = 0u;
        for_tiles(a, GS_DIV, nullptr, 0, [&](int j, int local) {
            if (j != cur) {
                if (cur >= 0) block_max_to(mb, &a.grids[cur].status->div_bits);
                cur = j;
                mb = 0u;
            }
            const GroupGrid& d = a.grids[j];
            const Grid g = d.g;  // in registers: the stores below cannot alias it
            const int tpp = group_interior_tpp(g);
            const int z0 = 1 + (local / tpp) * a.zslab;
            const int z1 = min(z0 + a.zslab, g.nz - 1);
            const int f = (local % tpp) * GROUP_TILE + tid;
            const int L = g.nx - 2;
            if (f < L * (g.ny - 2)) {
                int i = g.idx(1 + f % L, 1 + f / L, z0);
                for (int z = z0; z < z1; ++z, i += g.XY)
                    mb = max(mb, __float_as_uint(cell_div(g, d.pu, d.pv, d.pw, d.flags, i)));
            }
        });
        if (cur >= 0) block_max_to(mb, &a.grids[cur].status->div_bits);
    }
}

int g_sms = 0;
int g_occ[6] = {0, 0, 0, 0, 0, 0};  // resident CTAs per SM: project, objects, forcing, adv_vel, adv_rho

int ensure_occupancy() {
    if (g_sms > 0) return 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    const void* ks[5] = {(const void*)k_group_project, (const void*)k_group_objects, (const void*)k_group_forcing,
                         (const void*)k_group_adv_vel, (const void*)k_group_adv_rho};
    for (int k = 0; k < 5 && e == cudaSuccess; ++k)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_occ[k], ks[k], GROUP_TILE, k == 0 ? 16384 : 0);
    if (e != cudaSuccess) {
        g_sms = 0;
        return (int)e;
    }
    return 0;
}

// per_tile: one CTA per tile, so the block scheduler hands out tiles in index order as CTAs
// finish and the tiles in flight (and the planes they share) stay close together in L2, where a
// fixed set of grid-striding CTAs drifts apart; it pays for the gather-heavy velocity advection
// (1.00 -> 0.88 ms on the 64-grid batch) but not for the light stages, whose short CTAs then
// cost more to launch than they save (forcing 0.31 -> 0.46 ms).
int launch_grid_stride(const void* kernel, int total, int occ, const GroupArgs& a, cudaStream_t st,
                       bool per_tile = false) {
    if (total <= 0) return 0;
    const int cap = occ * g_sms;
    const int ctas = per_tile || total < cap ? total : cap;
    void* args[] = {(void*)&a};
    return (int)cudaLaunchKernel(kernel, dim3((unsigned)ctas), dim3(SB_BX, SB_BY), args, 0, st);
}

int launch_project(const GroupArgs& args, const GroupLaunch& L, cudaStream_t st) {
    GroupArgs a = args;
    a.wait_ns = GROUP_WAIT_NS;
    a.skip_barrier = 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return (int)cudaGetLastError();
    if (cap == cudaStreamCaptureStatusNone) {
        // a pending barrier-timeout injection (testing) applies to this launch, made outside any
        // graph capture (a captured launch would replay it), and is consumed
        std::lock_guard<std::mutex> lock(g_inject_mutex);
        if (g_inject_barrier > 0) {
            a.skip_barrier = g_inject_barrier;
            a.wait_ns = g_inject_wait_ns;
            g_inject_barrier = 0;
            g_injected_sync = a.sync;
            g_injected_ctas = L.coop_ctas;
        }
    }
    cudaError_t e = cudaMemsetAsync(a.sync, 0, sizeof(GroupSync), st);
    if (e != cudaSuccess) return (int)e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)L.coop_ctas);
    cfg.blockDim = dim3(SB_BX, SB_BY);
    cfg.dynamicSmemBytes = (size_t)a.n;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return (int)cudaLaunchKernelEx(&cfg, k_group_project, a);
}

}  // namespace

int group_occupancy(int* coop_per_sm, int* stage_per_sm, int* sms) {
    const int rc = ensure_occupancy();
    if (rc) return rc;
    if (coop_per_sm) *coop_per_sm = g_occ[0];
    if (stage_per_sm) *stage_per_sm = g_occ[2];
    if (sms) *sms = g_sms;
    return 0;
}

// The blocked solve's launches for groups [g0, g1): group k covers sweeps [k G, (k+1) G) (the
// last one may be partial), depth-6 launches, the first of each with the tolerance check.
// Inside a loop body (group_base set) the group index is relative to *group_base; `nl` counts
// launches so far (the input buffer alternates, starting from P).
int issue_tb_groups(const GroupTBLaunch& tb, int g0, int g1, const int* group_base, int& nl, cudaStream_t st) {
    constexpr int T = 6;
    for (int grp = g0; grp < g1; ++grp) {
        const int first = grp * tb.check_every;
        const int end = first + tb.check_every < tb.max_sweeps ? first + tb.check_every : tb.max_sweeps;
        for (int h = 2 * first; h < 2 * end; h += T) {
            const int nh = 2 * end - h < T ? 2 * end - h : T;
            const int rc = launch_group_sweep_tb(tb.grids, tb.starts, tb.n, tb.total, (nl & 1) == 0, nh, h & 1,
                                                 tb.zchunk, h == 2 * first ? 1 : 0, grp, group_base, st);
            if (rc) return rc;
            ++nl;
        }
    }
    return 0;
}

// The whole blocked solve: the full groups as a device-side WHILE loop when the stream is being
// captured (the loop stops when every grid's tolerance rule is satisfied), then the groups
// left (a partial last group), whose launches exit at entry for grids that are done.
int launch_tb_solve(GroupTBLaunch& tb, cudaStream_t st) {
    constexpr int T = 6;
    const int G = tb.check_every;
    const int nlg = (2 * G + T - 1) / T;
    const int U = (nlg % 2 == 0) ? 1 : 2;
    const int full = tb.max_sweeps / G;
    const int groups = (tb.max_sweeps + G - 1) / G;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return (int)e;
    const int loop_groups = (cs == cudaStreamCaptureStatusActive && tb.body) ? (full / U) * U : 0;
    int nl = 0, done_groups = 0;
    if (loop_groups > U) {
        e = cudaMemsetAsync(tb.counter, 0, sizeof(int), st);
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &ndeps);
        cudaGraphConditionalHandle handle;
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&handle, cg, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = handle;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &np);
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(tb.body, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return (int)e;
        int rc = issue_tb_groups(tb, 0, U, tb.counter, nl, tb.body);
        if (!rc)
            launch_group_tb_loop_next(tb.grids, tb.n, tb.counter, U, loop_groups, tb.launches, nl + 1, handle,
                                      tb.body);
        cudaGraph_t bg = nullptr;
        e = cudaStreamEndCapture(tb.body, &bg);
        if (rc) return rc;
        if (e != cudaSuccess) return (int)e;
        nl = 0;  // U groups launch an even number of times: every iteration starts from P
        done_groups = loop_groups;
    }
    const int rc = issue_tb_groups(tb, done_groups, groups, nullptr, nl, st);
    tb.issued = nl;
    return rc;
}

int launch_group_step(const GroupArgs& a, const GroupLaunch& L, cudaStream_t st, GroupTBLaunch* tb) {
    int rc = ensure_occupancy();
    if (!rc) rc = launch_grid_stride((const void*)k_group_objects, L.total[GS_OBJECTS], g_occ[1], a, st);
    if (!rc) rc = launch_grid_stride((const void*)k_group_forcing, L.total[GS_FORCE], g_occ[2], a, st);
    if (tb == nullptr) {
        if (!rc) rc = launch_project(a, L, st);
    } else {
        GroupArgs r = a;
        r.phases = GP_RHS;
        if (!rc) rc = launch_project(r, L, st);
        if (!rc) rc = launch_tb_solve(*tb, st);
        r.phases = GP_FINISH;
        if (!rc) rc = launch_project(r, L, st);
    }
    if (!rc) rc = launch_grid_stride((const void*)k_group_adv_vel, L.total[GS_ADV_VEL], g_occ[3], a, st, true);
    if (!rc) rc = launch_grid_stride((const void*)k_group_adv_rho, L.total[GS_ADV_RHO], g_occ[4], a, st);
    return rc;
}

int launch_group_tb_sweeps(const GroupTBLaunch& tb, int launches, cudaStream_t st) {
    // tuning: `launches` depth-6 launches without tolerance checks, each reading P and writing P2
    for (int k = 0; k < launches; ++k) {
        const int rc = launch_group_sweep_tb(tb.grids, tb.starts, tb.n, tb.total, true, 6, 0, tb.zchunk, 0, 0,
                                             nullptr, st);
        if (rc) return rc;
    }
    return 0;
}

int launch_group_sweeps_only(const GroupArgs& a, const GroupLaunch& L, cudaStream_t st) {
    int rc = ensure_occupancy();
    if (!rc) rc = launch_project(a, L, st);
    return rc;
}

}  // namespace smk

// ---- testing: a grid-barrier wait that runs out, without any fault ------------------------------

extern "C" int smk_inject_barrier_timeout(int barrier, int wait_ms) {
    if (barrier < 0 || wait_ms < 1 || wait_ms > 10000)
        return smk_fail(SMK_ERR_INVALID, "barrier must be >= 0 and wait_ms 1..10000");
    std::lock_guard<std::mutex> lock(smk::g_inject_mutex);
    smk::g_inject_barrier = barrier;
    smk::g_inject_wait_ns = (unsigned long long)wait_ms * 1000000ull;
    return SMK_OK;
}

extern "C" int smk_barrier_timeout_report(int* ctas_left, int* ctas) {
    smk::GroupSync* sync = nullptr;
    int n = 0;
    {
        std::lock_guard<std::mutex> lock(smk::g_inject_mutex);
        sync = smk::g_injected_sync;
        n = smk::g_injected_ctas;
    }
    if (sync == nullptr) return smk_fail(SMK_ERR_STATE, "no barrier-timeout injection has run");
    SMK_CUDA(cudaDeviceSynchronize());
    smk::GroupSync h;
    SMK_CUDA(cudaMemcpy(&h, sync, sizeof(h), cudaMemcpyDeviceToHost));
    if (ctas_left) *ctas_left = h.left;
    if (ctas) *ctas = n;
    return SMK_OK;
}
