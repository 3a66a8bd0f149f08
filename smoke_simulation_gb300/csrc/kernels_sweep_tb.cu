// Temporally blocked red-black SOR sweeps on the cell pressure (the projection's hot loop).
//
// One launch applies `nhalf` <= T half-sweeps (colour passes) to P in a single pass over HBM:
// read P_in, b and the flag byte once, write P_out once -- 13 bytes per cell for T/2 sweeps,
// where one colour pass per launch moves ~9-11 bytes per pass.
//
// Decomposition.  A CTA of 32 x TY threads owns an x-y tile of 64 x 2TY cells (a T-cell halo
// on each side; the interior is (64-2T) x (2TY-2T)) and a z-range [za, zb) of output planes.
// It marches z as a wavefront: at iteration q it takes plane q, computes the residual of plane
// q-1 at time 0 (tolerance-check launches) and brings plane q-1-t from time t-1 to time t for
// t = 1..T, so plane q-1-T leaves the pipeline finished.  A colour-t cell reads only
// opposite-colour neighbours, whose time t-1 values are exactly what the neighbouring planes
// hold at that moment, so one copy of each plane suffices.  Halo cells are recomputed
// redundantly; cells within T - t of the interior are exact after half-sweep t.  A window side
// that reaches the grid's edge needs no halo where that saves windows (sweep_window), and a
// z-chunk near plane 0 starts there where that saves a pass of the unrolled loop (qbeg).
//
// Loads.  Planes arrive through TMA: thread 0 issues cp.async.bulk.tensor copies of the
// tile's P, b and flag boxes for plane q+S into an S-stage shared-memory ring (S = (T+4)/2,
// half the register ring, so stage and phase are fixed per unrolled iteration) while plane q is
// being computed; an mbarrier per stage counts the bytes.  Boxes outside the grid (halo, first
// and last planes) are zero-filled by the TMA unit, which is what the solver needs there (P = 0,
// not projectable).  Waits are bounded: on timeout the kernel records an error, waits (bounded)
// for its own copies still in flight and returns.
//
// Per thread: a 2 x PY patch (columns x0, x0+1 = A, B; PY = 2 or 4 rows) with x0, y0 even, so
// a cell's colour is the parity of z alone and the cells updated per stage are column A of the
// even rows and B of the odd rows, or the reverse, uniformly over the CTA.  The z-rings of P, b
// and flags live in registers; the loop over z is unrolled by the ring length so every slot is
// a fixed register.  x-neighbours come from the patch or a warp shuffle (a tile row of 32
// threads is one warp), y-neighbours from the patch or a shared-memory copy of each in-flight
// plane, published once per iteration (double-buffered: one barrier per iteration).  All
// stages of an iteration update the same colour pattern, so a stage needs one value per
// neighbour row (the last-row value of the thread above in one column, the row-0 value of the
// thread below in the other): only those two are published per plane, each as a float plane so
// a warp's read is 32 consecutive floats (one shared-memory wavefront); the residual plane of
// check launches publishes all four.
//
// Every update is  r = fma(-acc, P_c, b_c + (((P_x- + P_x+) + (P_y- + P_y+)) + (P_z- + P_z+)));
// P_c = fma(omega/acc, r, P_c), the oracle's order, so every launch shape gives the same bits
// as one colour pass per launch.  (-acc, omega/acc) come from a 128-entry table indexed by the
// flag byte (six neighbour bits + "projectable"), kept in shared memory once per lane so that
// lookups never conflict.
//
// Forms (one tile body, sweep_tile): k_sweep_tb<T, PY, FULL, CHK> (one grid, tensor maps as
// kernel parameters), k_group_sweep_tb<6, FULL, CHK> (the tiles of every grid of a batch in one
// launch, each grid's tensor maps in global memory), k_sweep_tb_ycl<6> (runs of 2, 4 or all of
// the CTAs of an x-z column as thread-block clusters that exchange boundary rows through
// distributed shared memory instead of recomputing a y-halo between them).  Launches of all T
// colour passes run the FULL instantiations (no per-stage tests), with the tolerance-check code
// compiled in (CHK = 1) or out (CHK = 0); partial launches test both at run time.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "common.cuh"
#include "kernels.h"
#include "tb_common.cuh"

namespace smk {

namespace {

using namespace tb;
constexpr int TB_TX = tb::TX;  // threads per tile row (one warp) = 64 cells

// Tile geometry for a patch of PY rows per thread: TY tile rows of threads (warps) give
// ROWS = PY * TY cell rows.  PY = 2: 16 warps, 32 rows; PY = 4: 8 warps, 32 rows (the ring of a
// 4-row patch needs ~225 registers per thread).
template <int PY>
struct TBGeom {
    static_assert(PY == 2 || PY == 4, "patch rows");
    static constexpr int TY = PY == 2 ? 16 : 8;
    static constexpr int ROWS = PY * TY;
    static constexpr int STAGE_P = ROWS * BOX_F * 4;  // bytes (a multiple of 128)
    static constexpr int STAGE_F = ROWS * BOX_U8;     // bytes (a multiple of 128)
    static constexpr int STAGE_BYTES = 2 * STAGE_P + STAGE_F;
    static constexpr int PROW = (TY + 2) * TB_TX;     // floats per published plane (zero row above/below)
    static constexpr int THREADS = TB_TX * TY;
};

struct WAcc8 { float w[8]; };

constexpr int GROUP_TB_DEPTH = 6;  // colour passes per launch of the grouped blocked solve

struct TBMaps {
    CUtensorMap pin;  // P_in
    CUtensorMap b;
    CUtensorMap f;
};

// Issue the three boxes of plane z into stage `st` (thread 0 only).
template <int PY>
__device__ __forceinline__ void issue_plane(const TBMaps& m, unsigned char* stage, uint32_t bar,
                                            int xf, int xb, int y, int z) {
    using G = TBGeom<PY>;
    mbar_expect_tx(bar, (uint32_t)G::STAGE_BYTES);
    tma_load_3d(smem_u32(stage), &m.pin, xf, y, z, bar);
    tma_load_3d(smem_u32(stage + G::STAGE_P), &m.b, xf, y, z, bar);
    tma_load_3d(smem_u32(stage + 2 * G::STAGE_P), &m.f, xb, y, z, bar);
}

// One cell update in the oracle's operation order; `c` = {-acc, omega/acc} from the flag
// table, `proj` = the cell is projectable (else it keeps its value, 0).
__device__ __forceinline__ float relax(float pc, float bc, float2 c, bool proj, float xm, float xp,
                                       float ym, float yp, float zm, float zp) {
    const float sum = ((xm + xp) + (ym + yp)) + (zm + zp);
    const float r = fmaf(c.x, pc, bc + sum);
    const float pn = fmaf(c.y, r, pc);
    return proj ? pn : pc;
}

__device__ __forceinline__ unsigned resid_bits(float pc, float bc, float2 c, bool proj, float xm,
                                               float xp, float ym, float yp, float zm, float zp) {
    const float sum = ((xm + xp) + (ym + yp)) + (zm + zp);
    const float r = fmaf(c.x, pc, bc + sum);
    return proj ? __float_as_uint(fabsf(r)) : 0u;
}

// flag byte of cell k (0..3 = A, B of the word's first row, A, B of its second row) of a packed
// flag word -> table index: bits 0-5 the six fluid-neighbour bits, bit 6 "projectable"
__device__ __forceinline__ unsigned fidx(unsigned f, int k) { return (f >> (8 * k + 1)) & 0x7fu; }

// Make the tensor map at `map` (global memory, written before the launch) current for the
// TMA unit's tensor-map reads from this CTA.
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
                 : "memory");
}

// Cluster barrier: every thread of every CTA of the cluster arrives (release) and waits
// (acquire); it also orders this CTA's shared-memory accesses like __syncthreads.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of this CTA's shared-memory word `local` in the shared memory of cluster CTA `rank`.
__device__ __forceinline__ uint32_t cluster_map(uint32_t local, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}

__device__ __forceinline__ void st_cluster(uint32_t addr, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

// The faces next to cell (x, y, z) that the gradient subtract moves, from the cell's flag byte f
// (body_gradient_subtract's rule: a face moves when its two cells are fluid and it lies in the
// range [1, nx) x [1, ny) x [1, nz) with its other two coordinates in [1, n - 2]), as bits:
// 0 the lower x face (index i), 1 the upper x face (i + 1), 2 lower y (i), 3 upper y (i + X),
// 4 lower z (i), 5 upper z (i + XY).  x >= 0.
__device__ __forceinline__ unsigned fused_face_mask(const Grid& g, unsigned f, int x, int y, int z) {
    if (!(f & F_SELF)) return 0u;
    const bool inx = x >= 1 && x <= g.nx - 2, iny = y >= 1 && y <= g.ny - 2, inz = z >= 1 && z <= g.nz - 2;
    unsigned m = 0u;
    if ((f & F_XM) && x >= 1 && x <= g.nx - 1 && iny && inz) m |= 1u;
    if ((f & F_XP) && x + 1 <= g.nx - 1 && iny && inz) m |= 2u;
    if ((f & F_YM) && y >= 1 && y <= g.ny - 1 && inx && inz) m |= 4u;
    if ((f & F_YP) && y + 1 <= g.ny - 1 && inx && inz) m |= 8u;
    if ((f & F_ZM) && z >= 1 && z <= g.nz - 1 && inx && iny) m |= 16u;
    if ((f & F_ZP) && z + 1 <= g.nz - 1 && inx && iny) m |= 32u;
    return m;
}

// One tile (bx, by, bz) of a blocked launch: the CTA's whole job.  `group` is absolute.
// GLOBAL_MAPS: the tensor maps are in global memory (grouped launches), not kernel parameters.
// YCLUSTER: runs of `ycl_n` CTAs along y (blockIdx.y / ycl_n = the run, blockIdx.y % ycl_n = the
// CTA's rank in it) form thread-block clusters; a run covers ycl_n * ROWS consecutive rows of
// which the first and last `ycl_hy` are halo (0 when one run spans the whole y extent, else T).
// Instead of recomputing a T-row halo between the CTAs of a run, every CTA writes its boundary
// rows' published values into its neighbours' shared memory (the padding rows of their
// published planes), and the per-iteration barrier is a cluster barrier.
// FULL: the launch applies all T colour passes (nhalf == T), so the stages need no test; CHK: 0
// or 1 = the launch is (not) a tolerance-check launch, fixed at compile time; -1 = `check` decides.
// FUSE (full non-check launches of the plain form): when fz says this launch ends the solve, the
// gradient subtract is applied inside it.  Pass T changes one colour only, so every face has
// exactly one cell of that colour next to it; the thread owning that cell moves the face with
// the operands of the cell's last update (its new value and its six neighbours, which pass T
// leaves at their final values), one iteration after the pass, the face loads issued before
// the iteration's wait so that their latency overlaps it.  The face values are those of
// body_gradient_subtract on the final pressure, bit for bit.
template <int T, int PY, bool GLOBAL_MAPS = false, bool YCLUSTER = false, bool FULL = false, int CHK = -1,
          bool FUSE = false>
__device__ __forceinline__ void sweep_tile(const TBMaps& maps, const Grid& g, float* __restrict__ Pout,
                                           int nhalf, int colour0, int zchunk, const WAcc8& wa,
                                           StepStatus* status, int check, int group, float tol,
                                           int* __restrict__ pcur, int out_idx, int* __restrict__ kerr,
                                           int bx, int by, int bz, unsigned ntiles, int ycl_n = 1,
                                           int ycl_hy = 0, SweepFuse fz = SweepFuse{}) {
    static_assert(!FUSE || (FULL && CHK == 0 && !YCLUSTER && !GLOBAL_MAPS), "fused subtract: plain full launches");
    const bool chk = CHK < 0 ? check != 0 : CHK == 1;
    using G = TBGeom<PY>;
    constexpr int TY = G::TY, ROWS = G::ROWS, PROW = G::PROW, STAGE_BYTES = G::STAGE_BYTES,
                  STAGE_P = G::STAGE_P;
    constexpr int L = PY - 1;                // last row of the patch
    constexpr int R = T + 4;                 // register ring length (even, >= T + 3)
    constexpr int TB_S = R / 2;              // TMA stages (planes in flight)
    const int yrank = YCLUSTER ? by % ycl_n : 0;  // rank in the cluster (clusters run along y)
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // TMA destinations must be 128-byte aligned: align the dynamic base explicitly (the launch
    // requests 128 spare bytes)
    unsigned char* stages = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // [S][STAGE_BYTES]
    // published planes, per buffer (2): the residual plane as 4 column planes (row 0 A, row 0 B,
    // last row A, last row B), then for stages 1..T a row-0 and a last-row plane; each
    // [TY+2][32] floats
    // the fused form has no check launch, so no residual planes: stage s publishes planes
    // PR - 2 + 2s (row 0) and PR - 1 + 2s (last row)
    constexpr int PR = FUSE ? 0 : 4;
    constexpr int NPUB = PR + 2 * T;
    // copies of the coefficient table: one per lane (the fused form: one per half-warp lane, to
    // make room for its staged faces; two lanes then share a copy)
    constexpr int CL = FUSE ? 16 : TB_TX;
    float* pub = reinterpret_cast<float*>(stages + TB_S * STAGE_BYTES);
    // the (-acc, omega/acc) table, one copy per lane: entry e of lane l at [e][l], so a warp's
    // lookup touches each bank pair once whatever the 32 flag bytes are (one shared copy made
    // a lookup near scattered solids take ~3.5 wavefronts instead of 2)
    float2* coef_all = reinterpret_cast<float2*>(pub + 2 * NPUB * PROW);
    // FUSE: the faces a thread moves, staged by cp.async two planes ahead, in two slots
    // ([plane & 1][row * 6 + face][thread])
    float* fbuf = reinterpret_cast<float*>(coef_all + 128 * CL);
    __shared__ __align__(8) uint64_t mbar[TB_S];
    __shared__ float2 coef_one[128];  // the table once, replicated into coef_all
    __shared__ int tma_bad;           // YCLUSTER: a TMA stage of this CTA never completed

    const bool first_tile = (bx | by | bz) == 0;
    // the solve ended at an earlier check (check_decide at the end of a check launch)
    if (status != nullptr && *(volatile int*)&status->done) return;
    const bool fuse = FUSE && fz.mode == 1;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TB_TX + tx;
    const bool leader = tid == 0;
    if (fuse && first_tile && leader) *fz.sub_done = 1;
    if (tid < 128) {  // one read of omega/acc per entry (global memory in the grouped form)
        const int acc = __popc(tid & 0x3f);
        coef_one[tid] = make_float2(-(float)acc, (tid & 0x40) ? wa.w[acc] : 0.0f);
    }
    __syncthreads();
    for (int i = tid; i < 128 * CL; i += G::THREADS) coef_all[i] = coef_one[i / CL];
    const float2* coef = coef_all + tx % CL;  // this lane's copy: entry e at coef[e * CL]
    // zero the padding rows of every published plane (never written afterwards, except by the
    // cluster neighbours in the YCLUSTER form)
    if (YCLUSTER && tid == 0) tma_bad = 0;
    for (int i = tid; i < 2 * NPUB * 2 * TB_TX; i += G::THREADS) {
        const int lane = i % TB_TX, edge = (i / TB_TX) % 2, set = i / (2 * TB_TX);
        pub[set * PROW + (edge ? (TY + 1) * TB_TX : 0) + lane] = 0.0f;
    }
    if (pcur != nullptr && first_tile && leader) *pcur = out_idx;

    // owned columns [xlo, xhi) and rows [ylo, yhi) of the grid; X0, Y0 (even) = the window's
    // first column and row (sweep_window)
    int X0, xlo, xhi, Yw, ylo = 0, yhi = 0;
    sweep_window(g.nx, 2 * TB_TX, T, bx, X0, xlo, xhi);
    if (!YCLUSTER) sweep_window(g.ny, ROWS, T, by, Yw, ylo, yhi);
    const int Y0 = YCLUSTER ? (by / ycl_n) * (ycl_n * ROWS - 2 * ycl_hy) - ycl_hy + yrank * ROWS : Yw;
    const int xf = X0 - (X0 & 3);             // 16-byte aligned float box start
    const int xb = X0 - (X0 & 15);            // 16-byte aligned flag box start
    const int of = X0 - xf + 2 * tx;          // this thread's column in the float box
    const int ob = X0 - xb + 2 * tx;          // ... in the flag box
    const int x0 = X0 + 2 * tx;
    const int y0 = Y0 + PY * ty;
    const int za = bz * zchunk;
    const int zb = min(za + zchunk, g.nz);
    const bool inx = x0 >= xlo && x0 < xhi;
    bool in[PY];  // row r of the patch is a row this tile owns, inside the grid
#pragma unroll
    for (int r = 0; r < PY; ++r)
        in[r] = inx &&
                (YCLUSTER ? (yrank * ROWS + PY * ty + r >= ycl_hy && yrank * ROWS + PY * ty + r < ycl_n * ROWS - ycl_hy)
                          : (y0 + r >= ylo && y0 + r < yhi)) &&
                y0 + r >= 0 && y0 + r < g.ny;
    const int off0 = x0 + g.X * y0;

    // planes below 0 are never projectable: a chunk near z = 0 may start at plane 0 (the ring's
    // zero-initialised slots stand for the planes below, as the zero-filled loads do), which it
    // does where that saves a pass of the unrolled loop
    // a fused launch runs one iteration more: the subtract of a plane comes one iteration after it
    // leaves the pipeline
    const int qend = zb + T + (fuse ? 1 : 0);
    const int qbeg = (za - T < 0 && (qend + R) / R < (qend - (za - T) + R) / R) ? 0 : za - T;
    const int nouter = (qend - qbeg + R) / R;
    const int qfinal = qbeg + nouter * R - 1;  // last iteration executed

    if (leader) {
        if (GLOBAL_MAPS) {
            tensormap_acquire(&maps.pin);
            tensormap_acquire(&maps.b);
            tensormap_acquire(&maps.f);
        }
        for (int s = 0; s < TB_S; ++s) mbar_init(smem_u32(&mbar[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int s = 0; s < TB_S; ++s)
            issue_plane<PY>(maps, stages + s * STAGE_BYTES, smem_u32(&mbar[s]), xf, xb, Y0, qbeg + s);
    }

    float2 pp[PY][R], bb[PY][R];  // P and b per patch row, slot = plane mod R
    unsigned ff[PY / 2][R];       // flags: bytes A, B of rows 2h and 2h+1
#pragma unroll
    for (int j = 0; j < R; ++j) {
#pragma unroll
        for (int r = 0; r < PY; ++r) pp[r][j] = bb[r][j] = make_float2(0.f, 0.f);
#pragma unroll
        for (int h = 0; h < PY / 2; ++h) ff[h][j] = 0u;
    }

    unsigned rmax = 0u;
    const int p_par = (qbeg + colour0) & 1;  // stage colour parity of the first iteration
    int par = 0;                             // publish-buffer parity
    const int me0 = (ty + 1) * TB_TX + tx;   // my slot in a padded published row set
    // YCLUSTER: the neighbours' copies of my boundary rows go to the padding rows of their
    // published planes (row TY+1 of the CTA above, row 0 of the CTA below)
    const bool push_up = YCLUSTER && ty == 0 && yrank > 0;
    const bool push_dn = YCLUSTER && ty == TY - 1 && yrank + 1 < ycl_n;
    uint32_t up_base = 0, dn_base = 0;
    if (YCLUSTER) {
        up_base = cluster_map(smem_u32(pub + (TY + 1) * TB_TX + tx), (uint32_t)(yrank > 0 ? yrank - 1 : 0));
        dn_base = cluster_map(smem_u32(pub + tx), (uint32_t)(yrank + 1 < ycl_n ? yrank + 1 : yrank));
        cluster_sync_all();  // every CTA's padding is zero before any neighbour writes into it
    } else {
        __syncthreads();  // barriers, table and padding visible
    }

    for (int base = qbeg; base <= qend; base += R) {
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int q = base + k;
            const int st = k % TB_S;
            const uint32_t phase = (uint32_t)((k / TB_S) & 1);
            // ---- FUSE: plane zs = q-2-T left the pipeline last iteration; its faces move below.
            // The y-neighbours pass T read at the patch's edges (row y0-1 in row 0's column, row
            // y0+PY in the last row's) come from last iteration's published planes, read before
            // this iteration's barrier (nobody writes that buffer again before it)
            const int zs = q - 2 - T;
            const bool sub = fuse && zs >= za && zs < zb;
            const bool sAp = ((k + R - 1 + p_par) & 1) == 0;  // last iteration's stage pattern
            float sv_above = 0.0f, sv_below = 0.0f;
            if (FUSE && sub) {
                const float* pq = pub + (par ^ 1) * NPUB * PROW;
                sv_above = pq[(PR - 1 + 2 * T) * PROW + me0 - TB_TX];
                sv_below = pq[(PR - 2 + 2 * T) * PROW + me0 + TB_TX];
            }
            // ---- plane q: wait for its TMA stage, take this thread's patch into slot k
            const bool ok = mbar_wait(smem_u32(&mbar[st]), phase);
            {
                const unsigned char* S_ = stages + st * STAGE_BYTES;
                const float* sp = reinterpret_cast<const float*>(S_);
                const float* sb = reinterpret_cast<const float*>(S_ + STAGE_P);
                const unsigned char* sf = S_ + 2 * STAGE_P;
#pragma unroll
                for (int r = 0; r < PY; ++r) {
                    const int rr = (PY * ty + r) * BOX_F + of;
                    pp[r][k] = *reinterpret_cast<const float2*>(sp + rr);
                    bb[r][k] = *reinterpret_cast<const float2*>(sb + rr);
                }
#pragma unroll
                for (int h = 0; h < PY / 2; ++h) {
                    const unsigned f0 =
                        *reinterpret_cast<const unsigned short*>(sf + (PY * ty + 2 * h) * BOX_U8 + ob);
                    const unsigned f1 =
                        *reinterpret_cast<const unsigned short*>(sf + (PY * ty + 2 * h + 1) * BOX_U8 + ob);
                    ff[h][k] = f0 | (f1 << 16);
                }
            }
            // ---- publish planes q-1-s (slot (k-1-s) mod R) for the y-neighbours; the residual
            // plane (s = 0) only in check launches.  This iteration's stages all update column A
            // of the even rows and B of the odd rows when sA, else the opposite (PY is even, so
            // the pattern is the same for every thread): a stage reads the last row's other
            // column of the thread above and row 0's other column of the thread below.
            const bool sA = ((k + p_par) & 1) == 0;
            float* pb = pub + par * NPUB * PROW;
            const uint32_t pofs = (uint32_t)(par * NPUB * PROW) * 4u;  // byte offset of this buffer
            if (chk) {
                const int j = (k - 1 + 2 * R) % R;
                pb[0 * PROW + me0] = pp[0][j].x;
                pb[1 * PROW + me0] = pp[0][j].y;
                pb[2 * PROW + me0] = pp[L][j].x;
                pb[3 * PROW + me0] = pp[L][j].y;
                if (push_up) {
                    st_cluster(up_base + pofs + 0u * PROW * 4u, pp[0][j].x);
                    st_cluster(up_base + pofs + 1u * PROW * 4u, pp[0][j].y);
                }
                if (push_dn) {
                    st_cluster(dn_base + pofs + 2u * PROW * 4u, pp[L][j].x);
                    st_cluster(dn_base + pofs + 3u * PROW * 4u, pp[L][j].y);
                }
            }
            // v0: row 0's value, read from above; vl: the last row's, read from below (the column
            // is chosen by branching once per iteration, not by a select per value)
            auto publish = [&](int s, float v0, float vl) {
                pb[(PR - 2 + 2 * s) * PROW + me0] = v0;
                pb[(PR - 1 + 2 * s) * PROW + me0] = vl;
                if (push_up) st_cluster(up_base + pofs + (uint32_t)(PR - 2 + 2 * s) * PROW * 4u, v0);
                if (push_dn) st_cluster(dn_base + pofs + (uint32_t)(PR - 1 + 2 * s) * PROW * 4u, vl);
            };
            if (sA) {
#pragma unroll
                for (int s = 1; s <= T; ++s) {
                    const int j = (k - 1 - s + 2 * R) % R;
                    publish(s, pp[0][j].y, pp[L][j].x);
                }
            } else {
#pragma unroll
                for (int s = 1; s <= T; ++s) {
                    const int j = (k - 1 - s + 2 * R) % R;
                    publish(s, pp[0][j].x, pp[L][j].y);
                }
            }
            if (YCLUSTER) {
                // every CTA of the cluster runs the same number of cluster barriers, so a CTA
                // whose TMA stage never completed records it and carries on (its results are
                // void; the error is reported) instead of leaving its neighbours waiting
                if (!ok) tma_bad = 1;
                cluster_sync_all();
            } else if (__syncthreads_or(!ok)) {
                // a TMA stage never completed: record it, drain what is in flight, stop
                if (leader) {
                    atomicExch(kerr, 1);
                    const int last = min(q + TB_S - 1, qfinal);
                    for (int pq = q; pq <= last; ++pq) {
                        const int d = pq - qbeg;
                        mbar_wait(smem_u32(&mbar[d % TB_S]), (uint32_t)((d / TB_S) & 1));
                    }
                }
                if (FUSE && fuse) cp_async_wait_all();
                __syncthreads();
                return;
            }
            // every thread has read stage st: refill it with plane q + S
            if (leader && q + TB_S <= qfinal)
                issue_plane<PY>(maps, stages + st * STAGE_BYTES, smem_u32(&mbar[st]), xf, xb, Y0, q + TB_S);

            // ---- FUSE: move the faces of plane zs, then stage the faces of plane q-T (two
            // iterations ahead; its last pass comes next iteration, with the opposite pattern).
            // Plane zs's last-colour cells hold their final values (slot js), their neighbours in
            // planes zs-1, zs, zs+1 the values pass T read (other colour: final, and exact one
            // cell beyond the owned region); the x-neighbours come from the patch or the next
            // lane, the y-neighbours at the patch's edge from pass T's reads (sv_above, sv_below)
            if (FUSE && fuse) {
                if (sub) {
                    cp_async_wait_one();  // plane zs's copies (two groups back) have landed
                    const int js = (k - 2 - T + 2 * R) % R, jm = (k - 3 - T + 2 * R) % R,
                              jp = (k - 1 - T + 2 * R) % R;
                    const float* fs = fbuf + (zs & 1) * (6 * PY * G::THREADS) + tid;
#pragma unroll
                    for (int r = 0; r < PY; ++r) {
                        const int cb = (r & 1) ^ (sAp ? 0 : 1);
                        // the x-neighbour in the next lane: B of the lane to the left (column A), A
                        // of the lane to the right (column B); every lane takes part
                        const float nx = cb ? __shfl_down_sync(0xffffffffu, pp[r][js].x, 1)
                                            : __shfl_up_sync(0xffffffffu, pp[r][js].y, 1);
                        const unsigned f = (ff[r / 2][js] >> (8 * (2 * (r & 1) + cb))) & 0xffu;
                        const unsigned m = in[r] ? fused_face_mask(g, f, x0 + cb, y0 + r, zs) : 0u;
                        if (m == 0u) continue;
                        const int ru = r > 0 ? r - 1 : 0, rd = r < L ? r + 1 : L;
                        const float pn = cb ? pp[r][js].y : pp[r][js].x;
                        const float xm = cb ? pp[r][js].x : nx;
                        const float xp = cb ? nx : pp[r][js].y;
                        const float ym = r == 0 ? sv_above : (cb ? pp[ru][js].y : pp[ru][js].x);
                        const float yp = r == L ? sv_below : (cb ? pp[rd][js].y : pp[rd][js].x);
                        const float zm = cb ? pp[r][jm].y : pp[r][jm].x;
                        const float zp = cb ? pp[r][jp].y : pp[r][jp].x;
                        const int i = off0 + cb + r * g.X + g.XY * zs;
                        const float* fr = fs + r * 6 * G::THREADS;
                        if (m & 1u) fz.u[i] = fr[0] - (pn - xm);
                        if (m & 2u) fz.u[i + 1] = fr[G::THREADS] - (xp - pn);
                        if (m & 4u) fz.v[i] = fr[2 * G::THREADS] - (pn - ym);
                        if (m & 8u) fz.v[i + g.X] = fr[3 * G::THREADS] - (yp - pn);
                        if (m & 16u) fz.w[i] = fr[4 * G::THREADS] - (pn - zm);
                        if (m & 32u) fz.w[i + g.XY] = fr[5 * G::THREADS] - (zp - pn);
                    }
                }
                const int zl = q - T;
                if (zl >= za && zl < zb) {
                    const int jl = (k - T + 2 * R) % R;
                    const bool sAn = !((((k + p_par) & 1) == 0));  // next iteration's stage pattern
                    const uint32_t d0 = smem_u32(fbuf + (zl & 1) * (6 * PY * G::THREADS) + tid);
#pragma unroll
                    for (int r = 0; r < PY; ++r) {
                        const int cb = (r & 1) ^ (sAn ? 0 : 1);
                        const unsigned f = (ff[r / 2][jl] >> (8 * (2 * (r & 1) + cb))) & 0xffu;
                        const unsigned m = in[r] ? fused_face_mask(g, f, x0 + cb, y0 + r, zl) : 0u;
                        const int i = off0 + cb + r * g.X + g.XY * zl;
                        const uint32_t d = d0 + 4u * (uint32_t)(r * 6 * G::THREADS);
                        if (m & 1u) cp_async4(d, fz.u + i);
                        if (m & 2u) cp_async4(d + 4u * G::THREADS, fz.u + i + 1);
                        if (m & 4u) cp_async4(d + 8u * G::THREADS, fz.v + i);
                        if (m & 8u) cp_async4(d + 12u * G::THREADS, fz.v + i + g.X);
                        if (m & 16u) cp_async4(d + 16u * G::THREADS, fz.w + i);
                        if (m & 32u) cp_async4(d + 20u * G::THREADS, fz.w + i + g.XY);
                    }
                }
                cp_async_commit();  // one group per iteration, empty or not
            }

            // ---- stage 0: residual of plane q-1 at time 0
            if (chk) {
                const int j = (k - 1 + R) % R, ju = k, jd = (k - 2 + R) % R;
                float lB[PY], rA[PY];
#pragma unroll
                for (int r = 0; r < PY; ++r) {
                    lB[r] = __shfl_up_sync(0xffffffffu, pp[r][j].y, 1);
                    rA[r] = __shfl_down_sync(0xffffffffu, pp[r][j].x, 1);
                }
                const int zp = q - 1;
                if (zp >= za && zp < zb) {
                    // row y0-1 (thread above, last row) and row y0+PY (thread below, row 0)
                    const float2 up = make_float2(pb[2 * PROW + me0 - TB_TX], pb[3 * PROW + me0 - TB_TX]);
                    const float2 dn = make_float2(pb[me0 + TB_TX], pb[PROW + me0 + TB_TX]);
#pragma unroll
                    for (int r = 0; r < PY; ++r) {
                        if (!in[r]) continue;
                        const float2 ym = r == 0 ? up : pp[r - 1][j];
                        const float2 yp = r == L ? dn : pp[r + 1][j];
                        const unsigned f = ff[r / 2][j];
                        const unsigned ia = fidx(f, 2 * (r & 1)), ib = fidx(f, 2 * (r & 1) + 1);
                        rmax = max(rmax, resid_bits(pp[r][j].x, bb[r][j].x, coef[ia * CL], ia & 0x40u, lB[r],
                                                    pp[r][j].y, ym.x, yp.x, pp[r][jd].x, pp[r][ju].x));
                        rmax = max(rmax, resid_bits(pp[r][j].y, bb[r][j].y, coef[ib * CL], ib & 0x40u, pp[r][j].x,
                                                    rA[r], ym.y, yp.y, pp[r][jd].y, pp[r][ju].y));
                    }
                }
            }

            // ---- stages 1..T: plane q-1-t (slot k-1-t) from time t-1 to t (pattern sA above)
#pragma unroll
            for (int t = 1; t <= T; ++t) {
                if (FULL || t <= nhalf) {  // FULL: nhalf == T, one basic block per stage run
                    const int j = (k - 1 - t + 2 * R) % R;
                    const int ju = (k - t + 2 * R) % R;
                    const int jd = (k - 2 - t + 2 * R) % R;
                    const float* r0 = pb + (PR - 2 + 2 * t) * PROW;  // row-0 values (the thread below's)
                    const float* rl = pb + (PR - 1 + 2 * t) * PROW;  // last-row values (the thread above's)
                    const float above = rl[me0 - TB_TX];       // row y0-1, the column row 0 updates
                    const float below = r0[me0 + TB_TX];       // row y0+PY, the column row L updates
                    float nv[PY];
                    if (sA) {
#pragma unroll
                        for (int r = 0; r < PY; ++r) {
                            const unsigned f = ff[r / 2][j];
                            if ((r & 1) == 0) {  // column A
                                const float lB = __shfl_up_sync(0xffffffffu, pp[r][j].y, 1);
                                const float ym = r == 0 ? above : pp[r - 1][j].x;
                                const float yp = pp[r + 1][j].x;
                                const unsigned ia = fidx(f, 0);
                                nv[r] = relax(pp[r][j].x, bb[r][j].x, coef[ia * CL], ia & 0x40u, lB, pp[r][j].y,
                                              ym, yp, pp[r][jd].x, pp[r][ju].x);
                            } else {              // column B
                                const float rA = __shfl_down_sync(0xffffffffu, pp[r][j].x, 1);
                                const float ym = pp[r - 1][j].y;
                                const float yp = r == L ? below : pp[r + 1 < PY ? r + 1 : r][j].y;
                                const unsigned ib = fidx(f, 3);
                                nv[r] = relax(pp[r][j].y, bb[r][j].y, coef[ib * CL], ib & 0x40u, pp[r][j].x, rA,
                                              ym, yp, pp[r][jd].y, pp[r][ju].y);
                            }
                        }
#pragma unroll
                        for (int r = 0; r < PY; ++r) {
                            if ((r & 1) == 0) pp[r][j].x = nv[r];
                            else pp[r][j].y = nv[r];
                        }
                    } else {
#pragma unroll
                        for (int r = 0; r < PY; ++r) {
                            const unsigned f = ff[r / 2][j];
                            if ((r & 1) == 0) {  // column B
                                const float rA = __shfl_down_sync(0xffffffffu, pp[r][j].x, 1);
                                const float ym = r == 0 ? above : pp[r - 1][j].y;
                                const float yp = pp[r + 1][j].y;
                                const unsigned ib = fidx(f, 1);
                                nv[r] = relax(pp[r][j].y, bb[r][j].y, coef[ib * CL], ib & 0x40u, pp[r][j].x, rA,
                                              ym, yp, pp[r][jd].y, pp[r][ju].y);
                            } else {              // column A
                                const float lB = __shfl_up_sync(0xffffffffu, pp[r][j].y, 1);
                                const float ym = pp[r - 1][j].x;
                                const float yp = r == L ? below : pp[r + 1 < PY ? r + 1 : r][j].x;
                                const unsigned ia = fidx(f, 2);
                                nv[r] = relax(pp[r][j].x, bb[r][j].x, coef[ia * CL], ia & 0x40u, lB, pp[r][j].y,
                                              ym, yp, pp[r][jd].x, pp[r][ju].x);
                            }
                        }
#pragma unroll
                        for (int r = 0; r < PY; ++r) {
                            if ((r & 1) == 0) pp[r][j].y = nv[r];
                            else pp[r][j].x = nv[r];
                        }
                    }
                }
            }

            // ---- plane q-1-T is finished (slot k-1-T)
            const int zo = q - 1 - T;
            if (zo >= za && zo < zb) {
                const int j = (k - 1 - T + 2 * R) % R;
#pragma unroll
                for (int r = 0; r < PY; ++r)
                    if (in[r]) *reinterpret_cast<float2*>(Pout + off0 + r * g.X + g.XY * zo) = pp[r][j];
            }
            par ^= 1;
        }
    }

    if (YCLUSTER && tma_bad) {
        // a stage failed: report it and wait (bounded) for this CTA's copies still in flight
        if (leader) {
            atomicExch(kerr, 1);
            for (int pq = qfinal - TB_S + 1; pq <= qfinal; ++pq) {
                const int d = pq - qbeg;
                mbar_wait(smem_u32(&mbar[d % TB_S]), (uint32_t)((d / TB_S) & 1));
            }
        }
    }
    if (FUSE && fuse) cp_async_wait_all();  // no staged copy outlives the CTA
    if (chk) {
        // the residual of this launch's input; if it is within tolerance the solve ends on that
        // input and this launch's passes are dropped
        block_max_to(rmax, &status->rmax_bits[group]);
        if (tid == 0) check_decide(status, group, tol, ntiles, pcur, 1 - out_idx);
    }
    if (YCLUSTER) cluster_sync_all();  // no CTA leaves while a neighbour may still address it
}

template <int T, int PY, bool FULL, int CHK>
__global__ void __launch_bounds__(TBGeom<PY>::THREADS, 1)
k_sweep_tb(const __grid_constant__ TBMaps maps, Grid g, float* __restrict__ Pout, int nhalf,
           int colour0, int zchunk, const __grid_constant__ WAcc8 wa, StepStatus* status, int check, int group,
           float tol, int* __restrict__ pcur, int out_idx, int* __restrict__ kerr,
           const int* __restrict__ group_base) {
    // inside a graph's device-side group loop the group index is relative to the loop counter
    if (group_base != nullptr) group += *group_base;
    sweep_tile<T, PY, false, false, FULL, CHK>(maps, g, Pout, nhalf, colour0, zchunk, wa, status, check, group,
                                               tol, pcur, out_idx, kerr, (int)blockIdx.x, (int)blockIdx.y,
                                               (int)blockIdx.z, gridDim.x * gridDim.y * gridDim.z);
}

// A full non-check launch that may end the solve: the gradient subtract fused (sweep_tile FUSE).
template <int T, int PY>
__global__ void __launch_bounds__(TBGeom<PY>::THREADS, 1)
k_sweep_tb_fused(const __grid_constant__ TBMaps maps, Grid g, float* __restrict__ Pout, int colour0, int zchunk,
                 const __grid_constant__ WAcc8 wa, StepStatus* status, int group, float tol, int* __restrict__ pcur,
                 int out_idx, int* __restrict__ kerr, const int* __restrict__ group_base, SweepFuse fz) {
    if (group_base != nullptr) group += *group_base;
    sweep_tile<T, PY, false, false, true, 0, true>(maps, g, Pout, T, colour0, zchunk, wa, status, 0, group, tol, pcur,
                                                   out_idx, kerr, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z,
                                                   gridDim.x * gridDim.y * gridDim.z, 1, 0, fz);
}

// The y-cluster form (2-row patches): runs of ycl_n CTAs along y form clusters, with a halo of
// ycl_hy rows at each end of a run.
template <int T>
__global__ void __launch_bounds__(TBGeom<2>::THREADS, 1)
k_sweep_tb_ycl(const __grid_constant__ TBMaps maps, Grid g, float* __restrict__ Pout, int nhalf, int colour0,
               int zchunk, const __grid_constant__ WAcc8 wa, StepStatus* status, int check, int group, float tol,
               int* __restrict__ pcur, int out_idx, int* __restrict__ kerr, const int* __restrict__ group_base,
               int ycl_n, int ycl_hy) {
    if (group_base != nullptr) group += *group_base;
    sweep_tile<T, 2, false, true>(maps, g, Pout, nhalf, colour0, zchunk, wa, status, check, group, tol, pcur,
                                  out_idx, kerr, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z,
                                  gridDim.x * gridDim.y * gridDim.z, ycl_n, ycl_hy);
}

// ---- grouped form: one blocked launch over the tiles of every grid of a batch ---------------

// One grid of a grouped blocked launch.  The tensor maps live in global memory (64-byte
// aligned records), one set per input buffer: maps[0] reads P, maps[1] reads P2.
struct GroupTBGrid {
    TBMaps maps[2];
    Grid g;
    float* P;
    float* P2;
    StepStatus* status;
    int* pcur;
    int* kerr;
    WAcc8 wa;
    float tol;
    int tiles_x, tiles_y, zchunks;
};

// CTA b of the launch takes tile b of the flat index space (the tiles of one grid are
// contiguous; `starts` holds n + 1 prefix sums).  in_a: read P and write P2, else the reverse.
template <int T, bool FULL, int CHK>
__global__ void __launch_bounds__(TBGeom<2>::THREADS, 1)
k_group_sweep_tb(const GroupTBGrid* __restrict__ grids, const int* __restrict__ starts, int n, int in_a,
                 int nhalf, int colour0, int zchunk, int check, int group, const int* __restrict__ group_base) {
    const int t = (int)blockIdx.x;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (starts[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const GroupTBGrid& d = grids[lo];
    const int local = t - starts[lo];
    const int tx = d.tiles_x, per = tx * d.tiles_y;
    const int bz = local / per, r = local - bz * per, by = r / tx, bx = r - by * tx;
    if (group_base != nullptr) group += *group_base;
    // the record's scalars in registers; the tensor maps and omega/acc stay in global memory
    const Grid g = d.g;
    float* const Pout = in_a ? d.P2 : d.P;
    StepStatus* const status = d.status;
    int* const pcur = d.pcur;
    int* const kerr = d.kerr;
    const float tol = d.tol;
    sweep_tile<T, 2, true, false, FULL, CHK>(d.maps[in_a ? 0 : 1], g, Pout, nhalf, colour0, zchunk, d.wa, status,
                                             check, group, tol, pcur, in_a ? 1 : 0, kerr, bx, by, bz,
                                             (unsigned)(per * d.zchunks));
}

// End of one iteration of a grouped step's device-side loop over tolerance groups: advance
// the group counter; loop again while some grid's solve is not done and full groups remain.
// One block.
__global__ void k_group_tb_loop_next(const GroupTBGrid* __restrict__ grids, int n, int* counter, int step,
                                     int limit, unsigned long long* launches, int launches_per_iter,
                                     cudaGraphConditionalHandle handle) {
    int active = 0;
    for (int j = (int)threadIdx.x; j < n; j += (int)blockDim.x)
        active |= *(volatile const int*)&grids[j].status->done == 0;
    active = __syncthreads_or(active);
    if (threadIdx.x == 0) {
        const int c = *counter + step;
        *counter = c;
        if (launches != nullptr) *launches += (unsigned long long)launches_per_iter;
        cudaGraphSetConditional(handle, (active && c < limit) ? 1u : 0u);
    }
}

// ---- host side --------------------------------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

template <int T, int PY>
constexpr size_t tb_smem_bytes() {
    using G = TBGeom<PY>;
    return 128 + (size_t)((T + 4) / 2) * G::STAGE_BYTES + sizeof(float) * 2 * (4 + 2 * T) * G::PROW +
           sizeof(float2) * 128 * TB_TX;
}

// The fused-subtract form: no residual planes, 16 copies of the coefficient table, and the
// staged faces (two planes of 6 floats per patch row and thread).
template <int T, int PY>
constexpr size_t tb_smem_bytes_fused() {
    using G = TBGeom<PY>;
    return 128 + (size_t)((T + 4) / 2) * G::STAGE_BYTES + sizeof(float) * 2 * (2 * T) * G::PROW +
           sizeof(float2) * 128 * 16 + sizeof(float) * 2 * 6 * PY * G::THREADS;
}

template <int T, int PY>
int configure_tb() {
    const int bytes = (int)tb_smem_bytes<T, PY>();
    static_assert(tb_smem_bytes_fused<T, PY>() <= 227 * 1024, "shared memory of the fused form");
    const cudaFuncAttribute attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const bool ok = cudaFuncSetAttribute(k_sweep_tb<T, PY, false, -1>, attr, bytes) == cudaSuccess &&
                    cudaFuncSetAttribute(k_sweep_tb<T, PY, true, 0>, attr, bytes) == cudaSuccess &&
                    cudaFuncSetAttribute(k_sweep_tb<T, PY, true, 1>, attr, bytes) == cudaSuccess &&
                    cudaFuncSetAttribute(k_sweep_tb_fused<T, PY>, attr, (int)tb_smem_bytes_fused<T, PY>()) ==
                        cudaSuccess;
    return ok ? 0 : -1;
}

template <int T, int PY>
int launch_tb(const TBMaps& maps, const Grid& g, float* Pout, int nhalf, int colour0, int zchunk,
              const float* wacc7, StepStatus* status, int check, int group, float tol, int* pcur,
              int out_idx, int* kerr, const int* group_base, cudaStream_t st, const SweepFuse* fuse) {
    using G = TBGeom<PY>;
    const size_t smem = tb_smem_bytes<T, PY>();
    WAcc8 wa;
    for (int k = 0; k < 7; ++k) wa.w[k] = wacc7[k];
    wa.w[7] = 0.0f;
    dim3 grid((unsigned)sweep_windows(g.nx, 2 * TB_TX, T), (unsigned)sweep_windows(g.ny, G::ROWS, T),
              (unsigned)((g.nz + zchunk - 1) / zchunk));
    // a launch of all T colour passes runs an instantiation without per-stage tests and with the
    // check code present or absent; a partial launch decides both at run time
#define SMK_TB_LAUNCH(FULL, CHK)                                                                             \
    k_sweep_tb<T, PY, FULL, CHK><<<grid, dim3(TB_TX, G::TY), smem, st>>>(maps, g, Pout, nhalf, colour0, zchunk, \
                                                                        wa, status, check, group, tol, pcur,  \
                                                                        out_idx, kerr, group_base)
    if (nhalf == T && check) SMK_TB_LAUNCH(true, 1);
    else if (nhalf == T && fuse != nullptr && fuse->mode == 1)
        k_sweep_tb_fused<T, PY><<<grid, dim3(TB_TX, G::TY), tb_smem_bytes_fused<T, PY>(), st>>>(
            maps, g, Pout, colour0, zchunk, wa, status, group, tol, pcur, out_idx, kerr, group_base, *fuse);
    else if (nhalf == T) SMK_TB_LAUNCH(true, 0);
    else SMK_TB_LAUNCH(false, -1);
#undef SMK_TB_LAUNCH
    return 0;
}

constexpr int YCL_DEPTH = 6;  // the y-cluster form's depth

// Cluster geometry of a y-cluster shape: `n` CTAs per cluster, `hy` halo rows at each end of a
// cluster's run of rows, `grid_y` CTAs along y.  n_req = 0: one cluster spans the y extent
// (ny <= 256, no halo); 2 or 4: clusters of that many CTAs, each run of n * 32 rows overlapping
// the next by 2T halo rows.  False when the shape does not fit the grid.
struct YclGeom {
    int n, hy, grid_y;
};
inline bool ycl_geom(const Grid& g, int n_req, YclGeom* o) {
    constexpr int ROWS = TBGeom<2>::ROWS, T = YCL_DEPTH;
    if (n_req == 0) {
        const int c = (g.ny + ROWS - 1) / ROWS;
        if (c > 8) return false;
        *o = YclGeom{c, 0, c};
        return true;
    }
    if (n_req != 2 && n_req != 4) return false;
    const int run = n_req * ROWS - 2 * T;  // interior rows per cluster
    *o = YclGeom{n_req, T, ((g.ny + run - 1) / run) * n_req};
    return true;
}

cudaLaunchConfig_t ycl_config(const Grid& g, const YclGeom& y, int zchunk, cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)sweep_windows(g.nx, 2 * TB_TX, YCL_DEPTH), (unsigned)y.grid_y,
                       (unsigned)((g.nz + zchunk - 1) / zchunk));
    cfg.blockDim = dim3(TB_TX, TBGeom<2>::TY);
    cfg.dynamicSmemBytes = tb_smem_bytes<YCL_DEPTH, 2>();
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1;
    attr[0].val.clusterDim.y = (unsigned)y.n;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

int launch_tb_ycl(int n_req, const TBMaps& maps, const Grid& g, float* Pout, int nhalf, int colour0, int zchunk,
                  const float* wacc7, StepStatus* status, int check, int group, float tol, int* pcur, int out_idx,
                  int* kerr, const int* group_base, cudaStream_t st) {
    YclGeom y;
    if (!ycl_geom(g, n_req, &y)) return -1;
    WAcc8 wa;
    for (int k = 0; k < 7; ++k) wa.w[k] = wacc7[k];
    wa.w[7] = 0.0f;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = ycl_config(g, y, zchunk, attr);
    cfg.stream = st;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_sweep_tb_ycl<YCL_DEPTH>, maps, g, Pout, nhalf, colour0, zchunk,
                                             wa, status, check, group, tol, pcur, out_idx, kerr, group_base, y.n,
                                             y.hy);
    return e == cudaSuccess ? 0 : -1;
}

// End of one iteration of a graph's device-side loop over tolerance groups: advance the group
// counter and keep looping while the solve is not done and full groups remain.  One thread.
__global__ void k_group_loop_next(const StepStatus* status, int* counter, int step, int limit,
                                  unsigned long long* launches, int launches_per_iter,
                                  cudaGraphConditionalHandle handle) {
    const int c = *counter + step;
    *counter = c;
    *launches += (unsigned long long)launches_per_iter;
    const bool more = *(volatile const int*)&status->done == 0 && c < limit;
    cudaGraphSetConditional(handle, more ? 1u : 0u);
}

}  // namespace

namespace tb {
bool encode_3d(CUtensorMap* m, const void* base, bool is_u8, const Grid& g, int rows) {
    return encode_3d_box(m, base, is_u8, g, is_u8 ? BOX_U8 : BOX_F, rows);
}

bool encode_3d_box(CUtensorMap* m, const void* base, bool is_u8, const Grid& g, int box_w, int rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || base == nullptr || (reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false;
    const size_t es = is_u8 ? 1 : 4;
    if (box_w <= 0 || box_w > 256 || (box_w * es) % 16 != 0) return false;
    cuuint64_t dims[3] = {(cuuint64_t)g.X, (cuuint64_t)(g.ny + 1), (cuuint64_t)(g.nz + 1)};
    cuuint64_t strides[2] = {(cuuint64_t)g.X * es, (cuuint64_t)g.XY * es};
    cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)rows, 1u};
    cuuint32_t estr[3] = {1u, 1u, 1u};
    CUresult r = fn(m, is_u8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                    const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}
}  // namespace tb

bool sweep_tb_fusable(int T, int rows, int nhalf, int check) {
    return (rows == 2 || rows == 4) && sweep_tb_shape_supported(T, rows) && nhalf == T && !check;
}

int sweep_tb_shape_supported(int T, int rows) {
    if (rows & SWEEP_YCLUSTER) {
        const int n = sweep_ycluster_n(rows);
        return T == YCL_DEPTH && (rows & ~(SWEEP_YCLUSTER | (0xf << SWEEP_YCLUSTER_N_SHIFT))) == 2 &&
               (n == 0 || n == 2 || n == 4);
    }
    return (rows == 2 && (T == 2 || T == 4 || T == 6)) || (rows == 4 && T == 4);
}

int sweep_ycluster_usable(const Grid& g, int n_req) {
    YclGeom y;
    if (!ycl_geom(g, n_req, &y)) return 0;
    y.grid_y = y.n;  // one cluster's worth is enough for the query
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = ycl_config(g, y, g.nz, attr);
    cfg.gridDim.x = 1;
    cfg.gridDim.z = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_sweep_tb_ycl<YCL_DEPTH>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int prepare_sweep_kernels() {
    const int gbytes = (int)tb_smem_bytes<GROUP_TB_DEPTH, 2>();
    const cudaFuncAttribute gattr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const int grouped = (cudaFuncSetAttribute(k_group_sweep_tb<GROUP_TB_DEPTH, false, -1>, gattr, gbytes) == cudaSuccess &&
                         cudaFuncSetAttribute(k_group_sweep_tb<GROUP_TB_DEPTH, true, 0>, gattr, gbytes) == cudaSuccess &&
                         cudaFuncSetAttribute(k_group_sweep_tb<GROUP_TB_DEPTH, true, 1>, gattr, gbytes) == cudaSuccess)
                            ? 0 : -1;
    const int ycl = cudaFuncSetAttribute(k_sweep_tb_ycl<YCL_DEPTH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tb_smem_bytes<YCL_DEPTH, 2>()) == cudaSuccess ? 0 : -1;
    return configure_tb<2, 2>() | configure_tb<4, 2>() | configure_tb<6, 2>() | configure_tb<4, 4>() | grouped | ycl;
}

// Tensor maps for the sweep's TMA loads: P_a, P_b, b (float) and flags (u8), for the box
// heights of the 2-row ([0]) and 4-row ([1]) patch kernels.
struct SweepMaps {
    CUtensorMap pa[2], pb[2], b[2], f[2];
};

SweepMaps* create_sweep_maps(const Grid& g, const float* Pa, const float* Pb, const float* b,
                             const uint8_t* flags) {
    SweepMaps* m = new SweepMaps();
    const int rows[2] = {TBGeom<2>::ROWS, TBGeom<4>::ROWS};
    for (int v = 0; v < 2; ++v) {
        if (!encode_3d(&m->pa[v], Pa, false, g, rows[v]) || !encode_3d(&m->pb[v], Pb, false, g, rows[v]) ||
            !encode_3d(&m->b[v], b, false, g, rows[v]) || !encode_3d(&m->f[v], flags, true, g, rows[v])) {
            delete m;
            return nullptr;
        }
    }
    return m;
}

void destroy_sweep_maps(SweepMaps* m) { delete m; }

int launch_sweep_tb(const SweepMaps* m, const Grid& g, bool in_is_a, float* Pout, int T, int rows,
                    int nhalf, int colour0, int zchunk, const float* wacc7, StepStatus* status,
                    int check, int group, float tol, int* pcur, int out_idx, int* kerr,
                    const int* group_base, cudaStream_t st, const SweepFuse* fuse) {
    if (!sweep_tb_shape_supported(T, rows)) return -1;
    if (fuse != nullptr && (fuse->mode == 0 || !sweep_tb_fusable(T, rows, nhalf, check))) fuse = nullptr;
    const int v = rows == 4 ? 1 : 0;
    TBMaps maps;
    maps.pin = in_is_a ? m->pa[v] : m->pb[v];
    maps.b = m->b[v];
    maps.f = m->f[v];
#define SMK_TB_ARGS maps, g, Pout, nhalf, colour0, zchunk, wacc7, status, check, group, tol, pcur, out_idx, kerr, group_base, st
    if (rows & SWEEP_YCLUSTER) return launch_tb_ycl(sweep_ycluster_n(rows), SMK_TB_ARGS);
#undef SMK_TB_ARGS
#define SMK_TB_ARGS maps, g, Pout, nhalf, colour0, zchunk, wacc7, status, check, group, tol, pcur, out_idx, kerr, group_base, st, fuse
    if (rows == 4) return launch_tb<4, 4>(SMK_TB_ARGS);
    switch (T) {
        case 2: return launch_tb<2, 2>(SMK_TB_ARGS);
        case 4: return launch_tb<4, 2>(SMK_TB_ARGS);
        default: return launch_tb<6, 2>(SMK_TB_ARGS);
    }
#undef SMK_TB_ARGS
}

size_t group_tb_record_bytes() { return sizeof(GroupTBGrid); }

int group_tb_fill(void* rec, const SweepMaps* m, const Grid& g, float* P, float* P2, StepStatus* status, int* pcur,
                  int* kerr, const float* wacc7, float tol, int zchunk) {
    constexpr int T = GROUP_TB_DEPTH;
    GroupTBGrid d;
    memset(&d, 0, sizeof(d));
    d.maps[0].pin = m->pa[0];
    d.maps[1].pin = m->pb[0];
    d.maps[0].b = d.maps[1].b = m->b[0];
    d.maps[0].f = d.maps[1].f = m->f[0];
    d.g = g;
    d.P = P;
    d.P2 = P2;
    d.status = status;
    d.pcur = pcur;
    d.kerr = kerr;
    for (int k = 0; k < 7; ++k) d.wa.w[k] = wacc7[k];
    d.wa.w[7] = 0.0f;
    d.tol = tol;
    d.tiles_x = sweep_windows(g.nx, 2 * TB_TX, T);
    d.tiles_y = sweep_windows(g.ny, TBGeom<2>::ROWS, T);
    d.zchunks = (g.nz + zchunk - 1) / zchunk;
    memcpy(rec, &d, sizeof(d));
    return d.tiles_x * d.tiles_y * d.zchunks;
}

int launch_group_sweep_tb(const void* grids, const int* starts, int n, int total_tiles, bool in_a, int nhalf,
                          int colour0, int zchunk, int check, int group, const int* group_base, cudaStream_t st) {
    if (total_tiles <= 0) return 0;
    // as launch_tb: full launches without per-stage tests, check code present only where needed
#define SMK_GTB_LAUNCH(FULL, CHK)                                                                             \
    k_group_sweep_tb<GROUP_TB_DEPTH, FULL, CHK><<<(unsigned)total_tiles, dim3(TB_TX, TBGeom<2>::TY),          \
                                                 tb_smem_bytes<GROUP_TB_DEPTH, 2>(), st>>>(                  \
        static_cast<const GroupTBGrid*>(grids), starts, n, in_a ? 1 : 0, nhalf, colour0, zchunk, check, group, \
        group_base)
    if (nhalf == GROUP_TB_DEPTH && check) SMK_GTB_LAUNCH(true, 1);
    else if (nhalf == GROUP_TB_DEPTH) SMK_GTB_LAUNCH(true, 0);
    else SMK_GTB_LAUNCH(false, -1);
#undef SMK_GTB_LAUNCH
    return (int)cudaGetLastError();
}

void launch_group_tb_loop_next(const void* grids, int n, int* counter, int step, int limit,
                               unsigned long long* launches, int launches_per_iter,
                               cudaGraphConditionalHandle handle, cudaStream_t st) {
    k_group_tb_loop_next<<<1, 256, 0, st>>>(static_cast<const GroupTBGrid*>(grids), n, counter, step, limit,
                                            launches, launches_per_iter, handle);
}

void launch_group_loop_next(const StepStatus* status, int* counter, int step, int limit,
                            unsigned long long* launches, int launches_per_iter,
                            cudaGraphConditionalHandle handle, cudaStream_t st) {
    k_group_loop_next<<<1, 1, 0, st>>>(status, counter, step, limit, launches, launches_per_iter, handle);
}

}  // namespace smk
