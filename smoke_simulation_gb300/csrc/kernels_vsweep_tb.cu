// Temporally blocked red-black SOR of the reference scheme: the reference's in-place velocity
// projection (project/smokeSimulation.cu:356-394, 30 iterations per step at :795-801) with T
// colour passes per pass over HBM, bit-exact with one pass per launch (k_project_velocity).
//
// The reference's pass over colour c updates every interior fluid cell with (x + y + z + c) even
// and at least one fluid neighbour: from its six faces, div = -u_x + u_x+1 + -v_y + v_y+1 + -w_z
// + w_z+1 (left to right), p_t = float(double(-div / acc) * omega), and then
// u_x -= p_t*s(x-1), u_x+1 += p_t*s(x+1), v_y -= p_t*s(y-1), v_y+1 += p_t*s(y+1), w_z -= p_t*s(z-1),
// w_z+1 += p_t*s(z+1).  Within a pass no two updated cells share a face, so every face changes at
// most once per pass, and a face between cells a (below/left) and b is changed either by b
// ("own" lower face) or by a (b's face as a's upper face): the value sequence of each face is
// fixed by the pass order alone.
//
// Decomposition (as the pressure-form kernel, kernels_sweep_tb.cu): a CTA of 32 x TY threads
// owns an x-y tile of 64 x 2TY face-grid positions (position i holds the three lower faces u_i,
// v_i, w_i of cell i, the library's shared index) and a z-range, and marches z: at iteration q it
// takes plane q and applies pass t (t = 1..T) to plane q - t.  Each thread owns a 2 x 2 patch
// (columns A = x0, B = x0+1 with x0 even; rows y0, y0+1 with y0 even), so the cells a pass
// updates are A of one row and B of the other, uniformly over the CTA and the same for every
// stage of an iteration.  Pass t on plane p reads faces of planes p and p+1 and writes faces of
// planes p and p+1 (w_z+1), which the same thread holds: the z-ring lives in registers (T + 2
// planes: the plane being loaded, T planes in passes, and the finished plane waiting for its last
// update from above).  In-plane:
//   - x: a B cell's u_x+1 is the next lane's A value (shuffle down); the A cell right of an updated
//     B receives p_t * s through a shuffle up within the same pass;
//   - y: an updated last-row cell reads the v of the thread below's row 0 at the previous pass's
//     end, published in shared memory at the previous iteration; the row-0 cell below an updated
//     last-row cell receives p_t * s one iteration later (the thread above publishes p_t, the
//     receiver applies it before its next pass on that plane: nothing reads that face in between).
// So one barrier per iteration (double-buffered published planes) suffices.  Predicates: a face
// changes only when its updating cell is projectable (the flag byte's bit 7); the receiver of a
// cross-thread update reads the sender's projectable bit from the flag boxes when it loads the
// plane (left neighbour: a shuffle of the flag word; row above: the shared-memory flag box).
//
// Halo, windows, z-chunks and the TMA ring with bounded mbarrier waits are those of the pressure
// form (tb_common.cuh); positions that no pass changes (the boundary ring and everything outside
// the grid) make windows that reach the grid's edge need no halo there.  A launch reads u, v, w
// and the flags and writes u, v, w to a second set of face arrays (the simulation's pressure and
// rhs buffers, unused by this scheme): 25 bytes per position for T/2 iterations.
//
// p_t = float(double(-div / acc) * omega) is evaluated exactly without the FP64 pipe, which bounds
// the one-pass kernel on GB300 (exact_scale.cuh: the quotient by the small integer acc with one
// FMA correction, the double product with integer arithmetic).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "common.cuh"
#include "exact_scale.cuh"
#include "kernels.h"
#include "tb_common.cuh"

namespace smk {

namespace {

using namespace tb;

// Tile geometry: TY warps (tile rows of threads) of 2-row patches, ROWS = 2 TY face-grid rows.
// TY = 16: one CTA of 16 warps per SM (T = 4 needs ~120 registers a thread); TY = 12: two CTAs
// of 12 warps per SM (T = 2 within 80 registers), more warps to hide the update chains' latency.
template <int TY>
struct VTGeom {
    static constexpr int ROWS = 2 * TY;
    static constexpr int BOX_F_BYTES = ROWS * BOX_F * 4;          // one float box
    static constexpr int BOX_B_BYTES = ROWS * BOX_U8;             // the flag box
    static constexpr int STAGE = 3 * BOX_F_BYTES + BOX_B_BYTES;   // u, v, w, flags of one plane
    static constexpr int PROW = (TY + 2) * TX;                    // floats per published plane
    static constexpr int THREADS = TX * TY;
    static constexpr int MAPS = TY == 16 ? 0 : 1;                 // tensor-map set (box height)
    static_assert(STAGE % 128 == 0, "TMA destinations stay 128-byte aligned");
};

struct VMaps {
    CUtensorMap u, v, w, f;
};

// ---- one pass on one cell ----------------------------------------------------------------------

__device__ __forceinline__ float fsel(unsigned f, unsigned bit) { return (f & bit) ? 1.0f : 0.0f; }

// Per neighbour pattern (the flag byte's six neighbour bits, e = (f >> 1) & 63): the divisor acc
// (>= 1, so a non-projectable cell's quotient stays finite) as a float, RN(1/acc), and the six 0/1
// face multipliers s(x-1), s(y-1), s(z-1) | s(x+1), s(y+1), s(z+1), from a shared table
// (two 16-byte reads instead of a population count, a conversion and six selects per update).
struct CellCoef {
    float4 a;  // acc, RN(1/acc), s(x-1), s(y-1)
    float4 b;  // s(z-1), s(x+1), s(y+1), s(z+1)
};

__device__ __forceinline__ CellCoef make_coef(int e) {
    const int acc = max(__popc((unsigned)e), 1);
    CellCoef c;
    c.a = make_float4((float)acc, 1.0f / (float)acc, (e & 1) ? 1.f : 0.f, (e & 4) ? 1.f : 0.f);
    c.b = make_float4((e & 16) ? 1.f : 0.f, (e & 2) ? 1.f : 0.f, (e & 8) ? 1.f : 0.f, (e & 32) ? 1.f : 0.f);
    return c;
}

// p_t of a cell from its six faces; 0 for a cell that is not projectable (every use of p_t is
// predicated on the projectable bit).
__device__ __forceinline__ float cell_pt(unsigned f, const CellCoef& c, float uc, float ux, float vc, float vy,
                                         float wc, float wz, const OmegaSplit& os, double omega) {
    const float div = -uc + ux + -vc + vy + -wc + wz;
    bool rare;
    float pt = div_scale_fast(-div, c.a.x, c.a.y, os, rare);
    if (rare) pt = div_scale_full(-div, c.a.x, c.a.y, os.mo_hi, os.mo_lo, os.eo, os.sign, os.emin, os.emax, omega);
    return (f & F_PROJ) ? pt : 0.0f;
}

// Own (lower) faces of an updated cell: u_x -= p_t*s(x-1), v_y -= p_t*s(y-1), w_z -= p_t*s(z-1).
__device__ __forceinline__ void own_faces(unsigned f, const CellCoef& c, float pt, float& u, float& v, float& w) {
    if (f & F_PROJ) {
        u = u - pt * c.a.z;
        v = v - pt * c.a.w;
        w = w - pt * c.b.x;
    }
}

// Predicate bits of the faces a plane's patch receives from cells held by another thread.
enum : unsigned {
    G_XA0 = 1u,  // A0's left neighbour (lane - 1's B0) is projectable
    G_XA1 = 2u,  // A1's left neighbour (lane - 1's B1)
    G_YA0 = 4u,  // A0's neighbour at y - 1 (the thread above's A1, or the row above the tile)
    G_YB0 = 8u,  // B0's neighbour at y - 1
};

__device__ __forceinline__ unsigned fbyte(unsigned f, int k) { return (f >> (8 * k)) & 0xffu; }

// One tile of a launch: T colour passes (nhalf of them when not FULL) starting at colour0.
template <int T, int TY, bool FULL>
__device__ __forceinline__ void vsweep_tile(const VMaps& maps, const Grid& g, float* __restrict__ uo,
                                            float* __restrict__ vo, float* __restrict__ wo, int nhalf,
                                            int colour0, int zchunk, const OmegaSplit& os, double omega,
                                            int* __restrict__ kerr) {
    using G = VTGeom<TY>;
    constexpr int VT_STAGE = G::STAGE, VT_BOX_F = G::BOX_F_BYTES, VT_PROW = G::PROW, VT_THREADS = G::THREADS,
                  VT_ROWS = G::ROWS;
    constexpr int R = T + 2;   // register ring: planes q-1-T .. q
    constexpr int S = R / 2;   // TMA stages (stage and phase fixed per unrolled iteration)
    constexpr int NPUB = 2 * (T + 1);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* stages = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    float* pub = reinterpret_cast<float*>(stages + S * VT_STAGE);
    __shared__ __align__(8) uint64_t mbar[S];
    __shared__ CellCoef ctab[64];  // per neighbour pattern (make_coef)

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TX + tx;
    const bool leader = tid == 0;
    if (tid < 64) ctab[tid] = make_coef(tid);
    // zero the padding rows of every published plane (never written afterwards)
    for (int i = tid; i < 2 * NPUB * 2 * TX; i += VT_THREADS) {
        const int lane = i % TX, edge = (i / TX) % 2, set = i / (2 * TX);
        pub[set * VT_PROW + (edge ? (TY + 1) * TX : 0) + lane] = 0.0f;
    }

    // windows over the face grid: (nx+1) x (ny+1) positions, planes 0..nz
    int X0, xlo, xhi, Y0, ylo, yhi;
    sweep_window(g.nx + 1, 2 * TX, T, (int)blockIdx.x, X0, xlo, xhi);
    sweep_window(g.ny + 1, VT_ROWS, T, (int)blockIdx.y, Y0, ylo, yhi);
    const int xf = X0 - (X0 & 3);    // 16-byte aligned float box start
    const int xb = X0 - (X0 & 15);   // 16-byte aligned flag box start
    const int of = X0 - xf + 2 * tx;
    const int ob = X0 - xb + 2 * tx;
    const int x0 = X0 + 2 * tx;
    const int y0 = Y0 + 2 * ty;
    const int za = (int)blockIdx.z * zchunk;
    const int zb = min(za + zchunk, g.nz + 1);
    const bool inx = x0 >= xlo && x0 < xhi;
    bool in[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) in[r] = inx && y0 + r >= ylo && y0 + r < yhi && y0 + r >= 0 && y0 + r <= g.ny;
    const int off0 = x0 + g.X * y0;

    // a plane q is finished at iteration q + 1 + T; planes below 0 are never changed and the
    // zero-initialised ring stands for them, so a chunk near z = 0 may start at plane 0 where that
    // saves a pass of the unrolled loop
    const int qend = zb + T;
    int qbeg = (za - T < 0 && (qend + R) / R < (qend - (za - T) + R) / R) ? 0 : za - T;
    // start one plane lower where needed so that iteration k of every unrolled pass has the
    // update pattern of k's parity (fixed at compile time: one pattern's code per iteration); the
    // extra plane is one more halo plane (zero-filled below plane 0)
    qbeg -= (qbeg + colour0 - 1) & 1;
    const int nouter = (qend - qbeg + R) / R;
    const int qfinal = qbeg + nouter * R - 1;

    auto issue = [&](int s, int z) {
        unsigned char* st = stages + s * VT_STAGE;
        const uint32_t bar = smem_u32(&mbar[s]);
        mbar_expect_tx(bar, (uint32_t)VT_STAGE);
        tma_load_3d(smem_u32(st), &maps.u, xf, Y0, z, bar);
        tma_load_3d(smem_u32(st + VT_BOX_F), &maps.v, xf, Y0, z, bar);
        tma_load_3d(smem_u32(st + 2 * VT_BOX_F), &maps.w, xf, Y0, z, bar);
        tma_load_3d(smem_u32(st + 3 * VT_BOX_F), &maps.f, xb, Y0, z, bar);
    };
    if (leader) {
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&mbar[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int s = 0; s < S; ++s) issue(s, qbeg + s);
    }

    float2 U[2][R], V[2][R], W[2][R];  // per patch row (x = column A, y = column B), slot = plane mod R
    unsigned ff[R], gg[R];               // flag bytes A0, B0, A1, B1 and the G_* predicate bits
#pragma unroll
    for (int j = 0; j < R; ++j) {
#pragma unroll
        for (int r = 0; r < 2; ++r) U[r][j] = V[r][j] = W[r][j] = make_float2(0.f, 0.f);
        ff[j] = gg[j] = 0u;
    }
    const int me0 = (ty + 1) * TX + tx;
    int par = 0;
    __syncthreads();  // barriers initialised, table and padding visible

    for (int base = qbeg; base <= qend; base += R) {
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int q = base + k;
            const int st = k % S;
            const uint32_t phase = (uint32_t)((k / S) & 1);
            // updated cells of every stage of this iteration: A0 and B1 (sA), else B0 and A1; the
            // pattern follows (q + colour0 - 1), which qbeg's choice makes k's parity
            const bool sA = (k & 1) == 0;
            float* cur = pub + par * NPUB * VT_PROW;              // written this iteration
            const float* prv = pub + (par ^ 1) * NPUB * VT_PROW;  // written by the last one

            // ---- plane q into slot k, with the predicates of the faces it receives
            const bool ok = mbar_wait(smem_u32(&mbar[st]), phase);
            {
                const unsigned char* S_ = stages + st * VT_STAGE;
                const float* su = reinterpret_cast<const float*>(S_);
                const float* sv = reinterpret_cast<const float*>(S_ + VT_BOX_F);
                const float* sw = reinterpret_cast<const float*>(S_ + 2 * VT_BOX_F);
                const unsigned char* sf = S_ + 3 * VT_BOX_F;
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const int rr = (2 * ty + r) * BOX_F + of;
                    U[r][k] = *reinterpret_cast<const float2*>(su + rr);
                    V[r][k] = *reinterpret_cast<const float2*>(sv + rr);
                    W[r][k] = *reinterpret_cast<const float2*>(sw + rr);
                }
                const unsigned f0 = *reinterpret_cast<const unsigned short*>(sf + (2 * ty) * BOX_U8 + ob);
                const unsigned f1 = *reinterpret_cast<const unsigned short*>(sf + (2 * ty + 1) * BOX_U8 + ob);
                const unsigned f = f0 | (f1 << 16);
                ff[k] = f;
                const unsigned fl = __shfl_up_sync(0xffffffffu, f, 1);  // lane - 1's A0, B0, A1, B1
                const unsigned fa = ty > 0 ? *reinterpret_cast<const unsigned short*>(sf + (2 * ty - 1) * BOX_U8 + ob)
                                           : 0u;  // the row above: A, B
                unsigned gb = 0u;
                if (tx > 0) {
                    if (fbyte(fl, 1) & F_PROJ) gb |= G_XA0;
                    if (fbyte(fl, 3) & F_PROJ) gb |= G_XA1;
                }
                if (fa & F_PROJ) gb |= G_YA0;
                if ((fa >> 8) & F_PROJ) gb |= G_YB0;
                gg[k] = gb;
            }
            if (__syncthreads_or(!ok)) {
                // a TMA stage never completed: record it, drain what is in flight, stop
                if (leader) {
                    atomicExch(kerr, 1);
                    const int last = min(q + S - 1, qfinal);
                    for (int pq = q; pq <= last; ++pq) {
                        const int d = pq - qbeg;
                        mbar_wait(smem_u32(&mbar[d % S]), (uint32_t)((d / S) & 1));
                    }
                }
                __syncthreads();
                return;
            }
            // every thread has read stage st: refill it with plane q + S
            if (leader && q + S <= qfinal) issue(st, q + S);
            // "pass 0": the v of this plane's row-0 cell that this iteration's pattern updates, read
            // by the thread above at its first pass on this plane (next iteration).  Written after
            // the barrier: the previous iteration's reads of this buffer are all done.
            cur[me0] = sA ? V[0][k].x : V[0][k].y;

            // ---- passes t = 1..T on plane q - t (slot j), reaching into plane q - t + 1 (slot jn)
#pragma unroll
            for (int t = 1; t <= T; ++t) {
                const int j = (k - t + 2 * R) % R;
                const int jn = (k - t + 1 + 2 * R) % R;
                const unsigned f = ff[j], gb = gg[j];
                // the pass before (t - 1, at the previous iteration) changed the v face of this
                // plane's row-0 cell updated now through the thread above's last-row cell
                if (t >= 2 && (FULL || t - 1 <= nhalf)) {
                    const float pa = prv[(2 * (t - 1) + 1) * VT_PROW + me0 - TX];
                    if (sA) {
                        if (gb & G_YA0) V[0][j].x = V[0][j].x + pa * fsel(fbyte(f, 0), F_SELF);
                    } else {
                        if (gb & G_YB0) V[0][j].y = V[0][j].y + pa * fsel(fbyte(f, 1), F_SELF);
                    }
                }
                if (!(FULL || t <= nhalf)) continue;
                // v of the thread below's row-0 cell at the end of the previous pass
                const float vb = prv[(2 * (t - 1)) * VT_PROW + me0 + TX];
                if (sA) {
                    const unsigned fA0 = fbyte(f, 0), fB1 = fbyte(f, 3), fA1 = fbyte(f, 2);
                    const CellCoef cA0 = ctab[(fA0 >> 1) & 63u], cB1 = ctab[(fB1 >> 1) & 63u];
                    const float uR = __shfl_down_sync(0xffffffffu, U[1][j].x, 1);  // lane + 1's A1
                    const float pA0 = cell_pt(fA0, cA0, U[0][j].x, U[0][j].y, V[0][j].x, V[1][j].x, W[0][j].x,
                                              W[0][jn].x, os, omega);
                    const float pB1 = cell_pt(fB1, cB1, U[1][j].y, uR, V[1][j].y, vb, W[1][j].y, W[1][jn].y, os,
                                              omega);
                    own_faces(fA0, cA0, pA0, U[0][j].x, V[0][j].x, W[0][j].x);
                    own_faces(fB1, cB1, pB1, U[1][j].y, V[1][j].y, W[1][j].y);
                    const float pL = __shfl_up_sync(0xffffffffu, pB1, 1);  // lane - 1's B1
                    if (fA0 & F_PROJ) {
                        U[0][j].y = U[0][j].y + pA0 * cA0.b.y;    // B0's u
                        V[1][j].x = V[1][j].x + pA0 * cA0.b.z;    // A1's v
                        W[0][jn].x = W[0][jn].x + pA0 * cA0.b.w;  // w above A0
                    }
                    if (gb & G_XA1) U[1][j].x = U[1][j].x + pL * fsel(fA1, F_SELF);
                    if (fB1 & F_PROJ) W[1][jn].y = W[1][jn].y + pB1 * cB1.b.w;
                    cur[(2 * t) * VT_PROW + me0] = V[0][j].x;
                    cur[(2 * t + 1) * VT_PROW + me0] = pB1;
                } else {
                    const unsigned fB0 = fbyte(f, 1), fA1 = fbyte(f, 2), fA0 = fbyte(f, 0);
                    const CellCoef cB0 = ctab[(fB0 >> 1) & 63u], cA1 = ctab[(fA1 >> 1) & 63u];
                    const float uR = __shfl_down_sync(0xffffffffu, U[0][j].x, 1);  // lane + 1's A0
                    const float pB0 = cell_pt(fB0, cB0, U[0][j].y, uR, V[0][j].y, V[1][j].y, W[0][j].y, W[0][jn].y,
                                              os, omega);
                    const float pA1 = cell_pt(fA1, cA1, U[1][j].x, U[1][j].y, V[1][j].x, vb, W[1][j].x, W[1][jn].x,
                                              os, omega);
                    own_faces(fB0, cB0, pB0, U[0][j].y, V[0][j].y, W[0][j].y);
                    own_faces(fA1, cA1, pA1, U[1][j].x, V[1][j].x, W[1][j].x);
                    const float pL = __shfl_up_sync(0xffffffffu, pB0, 1);  // lane - 1's B0
                    if (fB0 & F_PROJ) {
                        V[1][j].y = V[1][j].y + pB0 * cB0.b.z;    // B1's v
                        W[0][jn].y = W[0][jn].y + pB0 * cB0.b.w;  // w above B0
                    }
                    if (gb & G_XA0) U[0][j].x = U[0][j].x + pL * fsel(fA0, F_SELF);
                    if (fA1 & F_PROJ) {
                        U[1][j].y = U[1][j].y + pA1 * cA1.b.y;    // B1's u
                        W[1][jn].x = W[1][jn].x + pA1 * cA1.b.w;  // w above A1
                    }
                    cur[(2 * t) * VT_PROW + me0] = V[0][j].y;
                    cur[(2 * t + 1) * VT_PROW + me0] = pA1;
                }
            }

            // ---- plane q - 1 - T: its last update (from the thread above's pass T) and the store
            {
                const int js = (k - 1 - T + 2 * R) % R;
                if (FULL) {
                    const float pa = prv[(2 * T + 1) * VT_PROW + me0 - TX];
                    const unsigned f = ff[js], gb = gg[js];
                    if (sA) {
                        if (gb & G_YA0) V[0][js].x = V[0][js].x + pa * fsel(fbyte(f, 0), F_SELF);
                    } else {
                        if (gb & G_YB0) V[0][js].y = V[0][js].y + pa * fsel(fbyte(f, 1), F_SELF);
                    }
                }
                const int zo = q - 1 - T;
                if (zo >= za && zo < zb) {
#pragma unroll
                    for (int r = 0; r < 2; ++r) {
                        if (!in[r]) continue;
                        const size_t o = (size_t)off0 + (size_t)r * g.X + (size_t)g.XY * zo;
                        *reinterpret_cast<float2*>(uo + o) = U[r][js];
                        *reinterpret_cast<float2*>(vo + o) = V[r][js];
                        *reinterpret_cast<float2*>(wo + o) = W[r][js];
                    }
                }
            }
            par ^= 1;
        }
    }
}

template <int T, int TY, bool FULL>
__global__ void __launch_bounds__(VTGeom<TY>::THREADS, TY == 16 ? 1 : 2)
k_vsweep_tb(const __grid_constant__ VMaps maps, Grid g, float* __restrict__ uo, float* __restrict__ vo,
            float* __restrict__ wo, int nhalf, int colour0, int zchunk, OmegaSplit os, double omega,
            int* __restrict__ kerr) {
    vsweep_tile<T, TY, FULL>(maps, g, uo, vo, wo, nhalf, colour0, zchunk, os, omega, kerr);
}

template <int T, int TY>
constexpr size_t vt_smem_bytes() {
    using G = VTGeom<TY>;
    return 128 + (size_t)((T + 2) / 2) * G::STAGE + sizeof(float) * 2 * 2 * (T + 1) * G::PROW;
}

// The tile height used with depth T: 12 warps (two CTAs per SM) for T = 2, 16 for T = 4.
constexpr int vt_ty(int T) { return T == 2 ? 12 : 16; }

}  // namespace

OmegaSplit omega_split(double w) {
    OmegaSplit s;
    memset(&s, 0, sizeof(s));
    uint64_t b;
    memcpy(&b, &w, 8);
    const int E = (int)((b >> 52) & 0x7ff);
    if (E == 0 || E == 0x7ff) {  // zero, subnormal or not finite: every q takes the double product
        s.emin = 256;
        s.emax = -1;
        return s;
    }
    const uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    s.mo_hi = (uint32_t)(m >> 32);
    s.mo_lo = (uint32_t)m;
    s.eo = E - 1023;
    s.sign = (uint32_t)(b >> 63);
    // the integer path keeps biased float exponents whose result stays a normal float: the
    // result lies in [2^(eq + eo), 2^(eq + eo + 2)], whose exponents must stay in [-126, 127]
    s.emin = -126 - s.eo + 127;
    s.emax = 125 - s.eo + 127;
    if (s.emin < 1) s.emin = 1;
    if (s.emax > 254) s.emax = 254;
    return s;
}

struct VSweepMaps {
    // per box height (0: 32 rows, 1: 24 rows)
    CUtensorMap su[2][2], sv[2][2], sw[2][2];  // [height][state buffer 0/1]
    CUtensorMap xu[2], xv[2], xw[2];           // the scratch face arrays
    CUtensorMap f[2];                          // neighbour flags
};

int vsweep_depth_supported(int T) { return T == 2 || T == 4; }

int prepare_vsweep_kernels() {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const bool ok =
        cudaFuncSetAttribute(k_vsweep_tb<2, 12, true>, a, (int)vt_smem_bytes<2, 12>()) == cudaSuccess &&
        cudaFuncSetAttribute(k_vsweep_tb<2, 12, false>, a, (int)vt_smem_bytes<2, 12>()) == cudaSuccess &&
        cudaFuncSetAttribute(k_vsweep_tb<4, 16, true>, a, (int)vt_smem_bytes<4, 16>()) == cudaSuccess &&
        cudaFuncSetAttribute(k_vsweep_tb<4, 16, false>, a, (int)vt_smem_bytes<4, 16>()) == cudaSuccess;
    return ok ? 0 : -1;
}

VSweepMaps* create_vsweep_maps(const Grid& g, float* const* u, float* const* v, float* const* w, const float* xu,
                               const float* xv, const float* xw, const uint8_t* flags) {
    VSweepMaps* m = new VSweepMaps();
    const int rows[2] = {VTGeom<16>::ROWS, VTGeom<12>::ROWS};
    bool ok = true;
    for (int h = 0; h < 2 && ok; ++h) {
        ok = tb::encode_3d(&m->f[h], flags, true, g, rows[h]) && tb::encode_3d(&m->xu[h], xu, false, g, rows[h]) &&
             tb::encode_3d(&m->xv[h], xv, false, g, rows[h]) && tb::encode_3d(&m->xw[h], xw, false, g, rows[h]);
        for (int b = 0; b < 2 && ok; ++b)
            ok = tb::encode_3d(&m->su[h][b], u[b], false, g, rows[h]) &&
                 tb::encode_3d(&m->sv[h][b], v[b], false, g, rows[h]) &&
                 tb::encode_3d(&m->sw[h][b], w[b], false, g, rows[h]);
    }
    if (!ok) {
        delete m;
        return nullptr;
    }
    return m;
}

void destroy_vsweep_maps(VSweepMaps* m) { delete m; }

template <int T>
static int launch_vt(const VSweepMaps* m, const Grid& g, int buf, bool from_state, float* uo, float* vo, float* wo,
                     int nhalf, int colour0, int zchunk, double omega, const OmegaSplit& os, int* kerr,
                     cudaStream_t st) {
    constexpr int TY = vt_ty(T);
    using G = VTGeom<TY>;
    constexpr int h = G::MAPS;
    VMaps maps;
    maps.u = from_state ? m->su[h][buf] : m->xu[h];
    maps.v = from_state ? m->sv[h][buf] : m->xv[h];
    maps.w = from_state ? m->sw[h][buf] : m->xw[h];
    maps.f = m->f[h];
    const dim3 grid((unsigned)sweep_windows(g.nx + 1, 2 * TX, T), (unsigned)sweep_windows(g.ny + 1, G::ROWS, T),
                    (unsigned)((g.nz + 1 + zchunk - 1) / zchunk));
    const dim3 block(TX, TY);
    const size_t smem = vt_smem_bytes<T, TY>();
    if (nhalf == T)
        k_vsweep_tb<T, TY, true><<<grid, block, smem, st>>>(maps, g, uo, vo, wo, nhalf, colour0, zchunk, os, omega,
                                                            kerr);
    else
        k_vsweep_tb<T, TY, false><<<grid, block, smem, st>>>(maps, g, uo, vo, wo, nhalf, colour0, zchunk, os, omega,
                                                             kerr);
    return (int)cudaGetLastError();
}

int launch_vsweep_tb(const VSweepMaps* m, const Grid& g, int buf, bool from_state, float* uo, float* vo, float* wo,
                     int T, int nhalf, int colour0, int zchunk, double omega, const OmegaSplit& os, int* kerr,
                     cudaStream_t st) {
    if (!vsweep_depth_supported(T) || nhalf < 1 || nhalf > T || zchunk < 1) return -1;
    if (T == 2) return launch_vt<2>(m, g, buf, from_state, uo, vo, wo, nhalf, colour0, zchunk, omega, os, kerr, st);
    return launch_vt<4>(m, g, buf, from_state, uo, vo, wo, nhalf, colour0, zchunk, omega, os, kerr, st);
}

}  // namespace smk

// ---- testing: the exact arithmetic's host instances, compared with the double product and the
// IEEE quotient by the CPU tests ----------------------------------------------------------------

extern "C" int smk_test_exact_arith(const float* x, const int* d, int n, double omega, float* scaled,
                                    float* quotient) {
    if (!x || n < 0) return 1;
    const smk::OmegaSplit os = smk::omega_split(omega);
    for (int i = 0; i < n; ++i) {
        if (scaled) scaled[i] = smk::omega_scale(x[i], os, omega);
        if (quotient && d) {
            const int k = d[i] < 1 ? 1 : (d[i] > 6 ? 6 : d[i]);
            quotient[i] = smk::div_small(x[i], (float)k, 1.0f / (float)k);
        }
    }
    return 0;
}

extern "C" int smk_test_exact_cell(const float* x, const int* d, int n, double omega, float* pt) {
    if (!x || !d || !pt || n < 0) return 1;
    const smk::OmegaSplit os = smk::omega_split(omega);
    for (int i = 0; i < n; ++i) {
        const int k = d[i] < 1 ? 1 : (d[i] > 6 ? 6 : d[i]);
        const float df = (float)k, r = 1.0f / (float)k;
        bool rare = false;
        float v = smk::div_scale_fast(x[i], df, r, os, rare);
        if (rare) v = smk::div_scale_full(x[i], df, r, os.mo_hi, os.mo_lo, os.eo, os.sign, os.emin, os.emax, omega);
        pt[i] = v;
    }
    return 0;
}
