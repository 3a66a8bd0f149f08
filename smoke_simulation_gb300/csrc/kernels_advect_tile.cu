// Velocity advection (velocityAdvectionU/V/W, smokeSimulation.cu:527-615) with the velocity
// planes staged in shared memory by TMA.
//
// A CTA of 32 x 8 threads owns a 32 x 8 tile of cells in x-y and a run of AT_ZC consecutive
// planes, and walks them in ascending z, one cell per thread and plane.  Each plane of u, v
// and w arrives as a 40 x 10 box (the tile plus one cell on every side, the x origin rounded
// down to a 16-byte boundary) in a four-slot ring: while plane z is computed, planes z - 1,
// z and z + 1 are resident and plane z + 2 is in flight.  The three 8-point averages of a cell
// read planes z - 1 and z at fixed offsets from one shared-memory address; a trilinear sample
// reads the window when its eight corners lie in planes z - 1 .. z + 1 of the window (every
// backtrace shorter than one cell does) and global memory otherwise.  The arithmetic is the
// reference's, term for term (avgU/V/W, sample_ref), so the results are the bits of the
// per-cell kernel.
//
// Each iteration has one barrier: after it every thread has finished plane z - 1, so thread 0
// refills the slot of plane z - 2 with plane z + 2.  Waits on the ring's mbarriers are bounded;
// on a timeout the CTA records the error, waits (bounded) for its own copies still in flight
// and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "tb_common.cuh"

namespace smk {

namespace {

using namespace tb;

constexpr int AT_TX = 32, AT_TY = 8;
constexpr int AT_W = 40;                  // window columns: x in [x_tile - 4, x_tile + 36)
constexpr int AT_H = AT_TY + 2;           // window rows: y in [y_tile - 1, y_tile + 9)
constexpr int AT_PSTR = 416;              // floats per field plane: 40 x 10, padded to 128 bytes
constexpr int AT_SLOTS = 4;
constexpr int AT_BOX_BYTES = AT_W * AT_H * 4;
constexpr int AT_ZC = 16;                 // planes per CTA
constexpr int AT_OX = 4;                  // a cell's column in the window = tx + AT_OX

static_assert(AT_PSTR * 4 % 128 == 0 && AT_PSTR >= AT_W * AT_H, "plane stride");

struct AdvMaps {
    CUtensorMap u, v, w;
};

// A trilinear sample of one field (sample_ref's arithmetic) whose corners are read from the
// window planes pm, pc, pp (planes z - 1, z, z + 1; the window's origin is (wx0, wy0)) when
// they lie there, else from global memory.
template <int HX, int HY, int HZ>
__device__ __forceinline__ float sample_win(const float* __restrict__ f, const Grid& g, const float* pm,
                                            const float* pc, const float* pp, int wx0, int wy0, int z, float px,
                                            float py, float pz) {
    const int lx = g.nx - 1, ly = g.ny - 1, lz = g.nz - 1;
    const float mx = (float)(unsigned)lx, my = (float)(unsigned)ly, mz = (float)(unsigned)lz;
    const float xs = fmaxf(fminf(px, mx), 1.0f) - (HX ? 0.5f : 0.0f);
    const float ys = fmaxf(fminf(py, my), 1.0f) - (HY ? 0.5f : 0.0f);
    const float zs = fmaxf(fminf(pz, mz), 1.0f) - (HZ ? 0.5f : 0.0f);
    const int x0 = __float2int_rz(xs);
    const float xw1 = xs - (float)x0;
    const float xw0 = 1.0f - xw1;
    const int y0 = __float2int_rz(ys);
    const float yw1 = ys - (float)y0;
    const float yw0 = 1.0f - yw1;
    const int z0 = __float2int_rz(zs);
    const float zw1 = zs - (float)z0;
    const float zw0 = 1.0f - zw1;
    // the upper corner repeats the lower one only on a delta-0 axis clamped to the last cell
    const bool sy = HY || y0 < ly;
    const bool sz = HZ || z0 < lz;
    const bool sx = HX || x0 < lx;
    const unsigned ux = (unsigned)(x0 - wx0), uy = (unsigned)(y0 - wy0), uz = (unsigned)(z0 - (z - 1));
    float a000, a010, a001, a011, b100, b110, b101, b111;
    if (ux <= (unsigned)(AT_W - 2) && uy <= (unsigned)(AT_H - 2) && uz <= 1u) {
        const int o = (int)(uy * AT_W + ux);
        const float* q0 = (uz ? pc : pm) + o;
        const float* q1 = sz ? (uz ? pp : pc) + o : q0;
        const int oy = sy ? AT_W : 0;
        a000 = q0[0];
        b100 = q0[1];
        a010 = q0[oy];
        b110 = q0[oy + 1];
        a001 = q1[0];
        b101 = q1[1];
        a011 = q1[oy];
        b111 = q1[oy + 1];
    } else {
        const float* r00 = f + (x0 + y0 * g.X + z0 * g.XY);
        const float* r10 = r00 + (sy ? g.X : 0);
        const float* r01 = r00 + (sz ? g.XY : 0);
        const float* r11 = r01 + (sy ? g.X : 0);
        a000 = r00[0];
        a010 = r10[0];
        a001 = r01[0];
        a011 = r11[0];
        b100 = r00[1];
        b110 = r10[1];
        b101 = r01[1];
        b111 = r11[1];
    }
    const float a100 = sx ? b100 : a000, a110 = sx ? b110 : a010, a101 = sx ? b101 : a001,
                a111 = sx ? b111 : a011;
    // trilinear_ref's products as packed pairs (each lane one IEEE product, the same bits).  The
    // products feed products and scalar sums only: ptxas contracts a packed product followed by a
    // packed add into a fused multiply-add, even with -fmad=false and explicit .rn forms
    const float2 xw = make_float2(xw0, xw1);
    const float2 xy0 = __fmul2_rn(xw, make_float2(yw0, yw0)), xy1 = __fmul2_rn(xw, make_float2(yw1, yw1));
    const float2 z0v = make_float2(zw0, zw0), z1v = make_float2(zw1, zw1);
    const float2 p0 = __fmul2_rn(__fmul2_rn(xy0, z0v), make_float2(a000, a100));
    const float2 p1 = __fmul2_rn(__fmul2_rn(xy1, z0v), make_float2(a010, a110));
    const float2 p2 = __fmul2_rn(__fmul2_rn(xy0, z1v), make_float2(a001, a101));
    const float2 p3 = __fmul2_rn(__fmul2_rn(xy1, z1v), make_float2(a011, a111));
    return p0.x + p0.y + p1.x + p1.y + p2.x + p2.y + p3.x + p3.y;
}

template <typename To>
__global__ void __launch_bounds__(AT_TX * AT_TY, 4)
k_advect_velocity_tile(const __grid_constant__ AdvMaps maps, Grid g, const float* __restrict__ u0,
                       const float* __restrict__ v0, const float* __restrict__ w0, To* __restrict__ u1,
                       To* __restrict__ v1, To* __restrict__ w1, const uint8_t* __restrict__ flags, float dt,
                       int* kerr, int cz0) {
    __shared__ alignas(128) float win[AT_SLOTS][3][AT_PSTR];
    __shared__ alignas(8) uint64_t mbar[AT_SLOTS];
    const int tx = (int)threadIdx.x, ty = (int)threadIdx.y;
    const bool leader = tx == 0 && ty == 0;
    const int xt = (int)blockIdx.x * AT_TX, yt = 1 + (int)blockIdx.y * AT_TY;
    const int zs = 1 + (cz0 + (int)blockIdx.z) * AT_ZC;
    const int ze = min(zs + AT_ZC, g.nz);  // planes [zs, ze) are advected; [zs - 1, ze] are read
    const int wx0 = xt - AT_OX, wy0 = yt - 1;

    // plane p goes to slot p & 3; its barrier phase counts the slot's earlier uses in this CTA
    auto issue = [&](int p) {
        const int s = p & (AT_SLOTS - 1);
        const uint32_t bar = smem_u32(&mbar[s]);
        mbar_expect_tx(bar, 3u * AT_BOX_BYTES);
        tma_load_3d(smem_u32(&win[s][0][0]), &maps.u, wx0, wy0, p, bar);
        tma_load_3d(smem_u32(&win[s][1][0]), &maps.v, wx0, wy0, p, bar);
        tma_load_3d(smem_u32(&win[s][2][0]), &maps.w, wx0, wy0, p, bar);
    };
    auto parity = [&](int p) { return (uint32_t)(((p - (zs - 1)) >> 2) & 1); };
    if (leader) {
        for (int s = 0; s < AT_SLOTS; ++s) mbar_init(smem_u32(&mbar[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int p = zs - 1; p <= min(zs + 1, ze); ++p) issue(p);
    }
    __syncthreads();

    const int x = xt + tx, y = yt + ty;
    const bool live = x >= 1 && x < g.nx && y < g.ny;
    const bool inx = x <= g.nx - 2, iny = y <= g.ny - 2;
    const int oc = (ty + 1) * AT_W + tx + AT_OX;  // the cell's offset in a window plane
    const float xf = (float)x, yf = (float)y;
    int issued = min(zs + 1, ze);  // last plane issued (leader)
    int waited = zs - 2;           // last plane this thread has seen complete
    if (mbar_wait(smem_u32(&mbar[(zs - 1) & 3]), parity(zs - 1))) {
        waited = zs - 1;
        if (mbar_wait(smem_u32(&mbar[zs & 3]), parity(zs))) waited = zs;
    }
    bool ok = waited == zs;

    for (int z = zs; z < ze; ++z) {
        if (z > zs) {
            // every thread is done with plane z - 2's slot; refill it with plane z + 2
            if (__syncthreads_or(!ok)) break;
            if (leader && z + 2 <= ze) issue(issued = z + 2);
        } else if (leader && z + 2 <= ze) {
            issue(issued = z + 2);
        }
        if (ok) ok = mbar_wait(smem_u32(&mbar[(z + 1) & 3]), parity(z + 1));
        if (!ok) continue;
        waited = z + 1;
        if (!live) continue;
        const int i = g.idx(x, y, z);
        const unsigned f = flags[i];
        if (!(f & F_SELF)) continue;
        const bool inz = z <= g.nz - 2;
        const bool du = iny && inz && (f & F_XM), dv = inx && inz && (f & F_YM), dw = inx && iny && (f & F_ZM);
        if (!(du || dv || dw)) continue;
        const float* um = &win[(z - 1) & 3][0][0];
        const float* uc = &win[z & 3][0][0];
        const float* up = &win[(z + 1) & 3][0][0];
        const float* vm = um + AT_PSTR;
        const float* vc = uc + AT_PSTR;
        const float* vp = up + AT_PSTR;
        const float* wm = vm + AT_PSTR;
        const float* wc = vc + AT_PSTR;
        const float* wp = vp + AT_PSTR;
        // avgU/avgV/avgW at this index, in the reference's order (common.cuh)
        // avgU and avgV as one packed chain of sums (lane x: u, lane y: v), avgW alone
        const float* a = um + oc;
        const float* b = uc + oc;
        const float* c = vm + oc;
        const float* d = vc + oc;
        float2 s2 = __fadd2_rn(make_float2(a[0], c[0]), make_float2(a[1], c[-1]));
        s2 = __fadd2_rn(s2, make_float2(a[-AT_W], c[AT_W]));
        s2 = __fadd2_rn(s2, make_float2(a[1 - AT_W], c[AT_W - 1]));
        s2 = __fadd2_rn(s2, make_float2(b[0], d[0]));
        s2 = __fadd2_rn(s2, make_float2(b[1], d[-1]));
        s2 = __fadd2_rn(s2, make_float2(b[-AT_W], d[AT_W]));
        s2 = __fadd2_rn(s2, make_float2(b[1 - AT_W], d[AT_W - 1]));
        const float au = s2.x / 8.0f, av = s2.y / 8.0f;
        a = wc + oc;
        b = wm + oc;
        const float aw = (a[0] + a[-1] + a[-AT_W] + a[-1 - AT_W] + b[0] + b[-1] + b[-AT_W] + b[-1 - AT_W]) / 8.0f;
        const float zf = (float)z;
        if (du) {
            float px = xf, py = yf + 0.5f, pz = zf + 0.5f;
            px = px - dt * uc[oc];
            py = py - dt * av;
            pz = pz - dt * aw;
            stv(u1, i, sample_win<0, 1, 1>(u0, g, um, uc, up, wx0, wy0, z, px, py, pz));
        }
        if (dv) {
            float px = xf + 0.5f, py = yf, pz = zf + 0.5f;
            px = px - dt * au;
            py = py - dt * vc[oc];
            pz = pz - dt * aw;
            stv(v1, i, sample_win<1, 0, 1>(v0, g, vm, vc, vp, wx0, wy0, z, px, py, pz));
        }
        if (dw) {
            float px = xf + 0.5f, py = yf + 0.5f, pz = zf;
            px = px - dt * au;
            py = py - dt * av;
            pz = pz - dt * wc[oc];
            stv(w1, i, sample_win<1, 1, 0>(w0, g, wm, wc, wp, wx0, wy0, z, px, py, pz));
        }
    }
    if (__syncthreads_or(!ok)) {
        // a plane never arrived: record it and wait (bounded) for this CTA's copies in flight
        if (leader) {
            atomicExch(kerr, 1);
            for (int p = waited + 1; p <= issued; ++p) mbar_wait(smem_u32(&mbar[p & 3]), parity(p));
        }
        __syncthreads();
    }
}

}  // namespace

struct AdvectMaps {
    AdvMaps set[2];
    int n;
};

AdvectMaps* create_advect_maps(const Grid& g, const float* const* u, const float* const* v, const float* const* w,
                               int n) {
    if (n < 1 || n > 2) return nullptr;
    AdvectMaps* m = new AdvectMaps();
    m->n = n;
    bool ok = true;
    for (int k = 0; k < n && ok; ++k)
        ok = tb::encode_3d_box(&m->set[k].u, u[k], false, g, AT_W, AT_H) &&
             tb::encode_3d_box(&m->set[k].v, v[k], false, g, AT_W, AT_H) &&
             tb::encode_3d_box(&m->set[k].w, w[k], false, g, AT_W, AT_H);
    if (!ok) {
        delete m;
        return nullptr;
    }
    return m;
}

void destroy_advect_maps(AdvectMaps* m) { delete m; }

template <typename To>
int launch_advect_velocity_tile(const AdvectMaps* m, int set, const Grid& g, const float* u0, const float* v0,
                                const float* w0, To* u1, To* v1, To* w1, const uint8_t* flags, float dt, int* kerr,
                                cudaStream_t st, int c0, int c1) {
    if (m == nullptr || set < 0 || set >= m->n) return -1;
    if (g.nx < 2 || g.ny < 2 || g.nz < 2) return 0;
    const int chunks = advect_velocity_chunks(g);
    if (c1 < 0 || c1 > chunks) c1 = chunks;
    if (c0 < 0) c0 = 0;
    if (c1 <= c0) return 0;
    const dim3 grid((unsigned)((g.nx + AT_TX - 1) / AT_TX), (unsigned)((g.ny - 1 + AT_TY - 1) / AT_TY),
                    (unsigned)(c1 - c0));
    k_advect_velocity_tile<To><<<grid, dim3(AT_TX, AT_TY), 0, st>>>(m->set[set], g, u0, v0, w0, u1, v1, w1, flags,
                                                                     dt, kerr, c0);
    return 0;
}

int advect_velocity_chunk_planes() { return AT_ZC; }

int advect_velocity_chunks(const Grid& g) { return g.nz < 2 ? 0 : (g.nz - 1 + AT_ZC - 1) / AT_ZC; }

template int launch_advect_velocity_tile<float>(const AdvectMaps*, int, const Grid&, const float*, const float*,
                                                const float*, float*, float*, float*, const uint8_t*, float, int*,
                                                cudaStream_t, int, int);
template int launch_advect_velocity_tile<__nv_bfloat16>(const AdvectMaps*, int, const Grid&, const float*,
                                                        const float*, const float*, __nv_bfloat16*,
                                                        __nv_bfloat16*, __nv_bfloat16*, const uint8_t*, float, int*,
                                                        cudaStream_t, int, int);

}  // namespace smk
