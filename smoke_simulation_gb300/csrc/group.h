// Grouped step of a batch: one persistent launch per stage over every grid of the batch.
//
// The host writes one GroupGrid record per grid (its buffers for this step's ping-pong parity,
// its parameters, its emitters) plus, per stage, the prefix sums of the grids' tile counts.  A
// grouped kernel walks the flat tile index space of its stage with a grid-stride loop; the
// tiles of one grid are contiguous, so a CTA finds the grid of its next tile by advancing
// through the prefix sums.  A tile is one 64 x 4 thread block of the single-grid launch of the
// same stage (block index = position inside the grid's range), so a tile evaluates exactly the
// cells the single-grid kernel's block would, with the same stage body.  The red-black sweeps
// and the residual use flattened tiles instead: 256 consecutive same-colour (or interior) cells
// of one z plane, so that grids of 32 cells per side do not leave three quarters of a 64-wide
// block idle.
#pragma once
#include <stdint.h>

#include "common.cuh"

namespace smk {

enum GroupStage : int {
    GS_OBJECTS = 0,  // box emitters, then sphere sources (per cell, in that order)
    GS_FORCE,        // integrate + clamp
    GS_RHS,          // b = -div u*, pressure start
    GS_SWEEP,        // one colour pass (flattened tiles)
    GS_RESID,        // residual of a tolerance check (flattened tiles, interior)
    GS_PROJECT,      // gradient subtract (FP32) or FP32 projection + BF16 rounding
    GS_DIV,          // max |div u| (flattened tiles, interior); 0 tiles when not reported
    GS_ADV_VEL,      // velocity advection
    GS_ADV_RHO,      // density advection
    GS_COUNT
};

constexpr int GROUP_TILE = 256;  // threads per tile (64 x 4)

// Storage kinds (the SMK_STORAGE_* values).
enum : int { GK_F32 = 0, GK_BF16 = 1, GK_BF16_VEL = 2 };

struct GroupGrid {
    Grid g;
    int kind;        // storage: GK_*
    int report_div;  // measure max |div u| after the projection
    // this step's buffers: `now` is the step's input state, `past` receives the advection
    void* rho0;
    void* rho1;  // both density buffers (emitters write both, as fillSmoke does)
    void* rho_now;
    void* rho_past;
    void* u_now;
    void* v_now;
    void* w_now;
    void* u_past;
    void* v_past;
    void* w_past;
    float* pu;  // projected velocity advection reads (FP32): the state itself, or the FP32
    float* pv;  // copy written by the projection in the BF16 storage forms
    float* pw;
    float* P;
    float* b;
    const float* P2;  // second pressure buffer: a warm start reads it when *pcur == 1
    int* pcur;
    float* Ph;        // pressure history of the extrapolated warm start (NULL: none)
    float extrap;     // its factor this step (0: start from the last pressure)
    const uint8_t* flags;
    StepStatus* status;
    int status_words;  // words of *status the step zeroes (header + residual groups)
    int* kerr;         // set when a bounded grid-barrier wait gave up
    float dt, gravity, alpha, lim_sq, lim;
    int clamp_mode;
    float wacc[8];  // omega / acc for acc = 0..6
    float tol;
    int check_every;
    int max_sweeps;
    int warm;
    int box0, nbox, sph0, nsph;  // ranges in the batch's box and sphere arrays
    int bx0, by0, bz0, bx1, by1, bz1;  // region of the clipped boxes (empty when x0 >= x1)
    int sx0, sy0, sz0, sx1, sy1, sz1;  // region of the spheres (interior, one cell margin)
    int ox0, oy0, oz0, ox1, oy1, oz1;  // union of both: the objects stage's tiles
    int wave;  // solve wave: waves run one after another, each to completion
    int vec4;  // rows on vector boundaries (vec4_layout): forcing, rhs and the subtract / BF16 projection take the 4-wide bodies
};

// Grid barrier of the cooperative projection kernel (reset before every launch).
struct GroupSync {
    unsigned long long count;  // arrivals so far
    int abort;                 // a wait gave up: every CTA leaves at its next barrier
    int left;                  // CTAs that left the kernel because a barrier gave up
};

// Phases of the cooperative projection kernel.
enum : int { GP_RHS = 1, GP_SOLVE = 2, GP_FINISH = 4, GP_ALL = 7 };

struct GroupArgs {
    const GroupGrid* grids;
    const int* starts;  // GS_COUNT rows of n + 1 tile prefix sums
    const BoxObj* boxes;
    const SphereObj* spheres;
    GroupSync* sync;
    int n;
    int zslab;        // z planes per sweep / residual / divergence tile (a thread walks them)
    int nwaves;       // solve waves (every grid's `wave` is below this)
    int sweeps_only;  // tuning: only the sweep passes (fixed count, no checks), on scratch buffers
    int phases;       // GP_* bits: rhs + pressure start, colour-pass solve, subtract + divergence
    unsigned long long wait_ns;  // a barrier wait gives up after this long (%globaltimer)
    int skip_barrier;            // testing: CTA 0 does not arrive at this barrier (1-based; 0 = none)
};

// The blocked form of the grouped solve (host side): instead of the cooperative kernel's colour
// passes, launches of the temporally blocked sweep kernel over every grid's tiles, each
// launch depth 6, a tolerance check in the first launch of each group (all grids share the
// group size and the sweep cap), the full groups as a device-side WHILE loop when captured.
struct GroupTBLaunch {
    const void* grids;   // device records (group_tb_record_bytes() each)
    const int* starts;   // device: n + 1 tile prefix sums
    int n;
    int total;           // tiles of one launch
    int zchunk;
    int check_every;     // sweeps per tolerance group
    int max_sweeps;
    int* counter;        // device: the loop's group counter
    cudaStream_t body;   // stream used to capture the loop body
    unsigned long long* launches;  // device (may be NULL): kernels run inside the loop
    int issued;          // set by launch_group_step: kernels the host issued for the solve
};

__host__ __device__ inline int group_div_up(int a, int b) { return (a + b - 1) / b; }

// Tiles of a 64 x 4 block launch over an rx x ry x rz range.
__host__ __device__ inline int group_block_tiles(int rx, int ry, int rz) {
    if (rx <= 0 || ry <= 0 || rz <= 0) return 0;
    return group_div_up(rx, 64) * group_div_up(ry, 4) * rz;
}

// Flattened tiles per z plane: same-colour cells (sweep) or all interior cells (residual/div).
__host__ __device__ inline int group_sweep_tpp(const Grid& g) {
    const int L = g.nx - 2, rows = g.ny - 2;
    return (L <= 0 || rows <= 0) ? 0 : group_div_up(((L + 1) / 2) * rows, GROUP_TILE);
}
__host__ __device__ inline int group_interior_tpp(const Grid& g) {
    const int L = g.nx - 2, rows = g.ny - 2;
    return (L <= 0 || rows <= 0) ? 0 : group_div_up(L * rows, GROUP_TILE);
}

// Extent of a block-tiled stage: the range its single-grid launch covers.
__host__ __device__ inline void group_extent(int stage, const GroupGrid& d, int& rx, int& ry, int& rz) {
    const Grid& g = d.g;
    rx = ry = rz = 0;
    switch (stage) {
        case GS_OBJECTS: rx = d.ox1 - d.ox0; ry = d.oy1 - d.oy0; rz = d.oz1 - d.oz0; break;
        case GS_FORCE: rx = g.nx; ry = g.ny - 1; rz = g.nz; break;
        case GS_RHS: rx = g.nx; ry = g.ny; rz = g.nz; break;
        case GS_PROJECT:
            if (d.kind == GK_F32) { rx = g.nx - 1; ry = g.ny - 1; rz = g.nz - 1; }
            else { rx = g.nx + 1; ry = g.ny + 1; rz = g.nz + 1; }
            break;
        case GS_ADV_VEL: rx = g.nx - 1; ry = g.ny - 1; rz = g.nz - 1; break;
        case GS_ADV_RHO: rx = g.nx - 2; ry = g.ny - 2; rz = g.nz - 2; break;
        default: break;
    }
}

// Advection tiles walk GROUP_ADV_ZC consecutive planes (as the single-grid advection kernels).
constexpr int GROUP_ADV_ZC = 4;

// 4-wide tiles (grids with vec4): 16 groups of 4 consecutive x by 16 rows of one plane, over
// gx groups (from x = 0), ry rows and rz planes.
constexpr int GX4_GX = 16, GX4_GY = 16;
__host__ __device__ inline int group_x4_tiles(int gx, int ry, int rz) {
    if (gx <= 0 || ry <= 0 || rz <= 0) return 0;
    return group_div_up(gx, GX4_GX) * group_div_up(ry, GX4_GY) * rz;
}
// Range of a 4-wide stage: groups of x, rows (from y0) and planes (from z0).
__host__ __device__ inline bool group_x4_extent(int stage, const GroupGrid& d, int& gx, int& ry, int& rz, int& y0,
                                                int& z0) {
    if (!d.vec4) return false;
    const Grid& g = d.g;
    gx = group_div_up(g.nx, 4);
    switch (stage) {
        case GS_FORCE: ry = g.ny - 1; rz = g.nz; y0 = 1; z0 = 0; return true;
        case GS_RHS: ry = g.ny; rz = g.nz; y0 = 0; z0 = 0; return true;
        case GS_PROJECT:
            if (d.kind == GK_F32) { ry = g.ny - 1; rz = g.nz - 1; y0 = 1; z0 = 1; }  // gradient subtract
            else { gx = group_div_up(g.nx + 1, 4); ry = g.ny + 1; rz = g.nz + 1; y0 = 0; z0 = 0; }  // BF16 projection
            return true;
        default: return false;
    }
}

// Tiles of a stage for one grid; the flattened stages cut the interior planes into slabs of
// `zslab` planes.
__host__ __device__ inline int group_tiles(int stage, const GroupGrid& d, int zslab) {
    const Grid& g = d.g;
    const int slabs = g.nz >= 3 ? group_div_up(g.nz - 2, zslab) : 0;
    int gx, ry4, rz4, y0, z0;
    if (group_x4_extent(stage, d, gx, ry4, rz4, y0, z0)) return group_x4_tiles(gx, ry4, rz4);
    switch (stage) {
        case GS_SWEEP: return group_sweep_tpp(g) * slabs;
        case GS_RESID: return group_interior_tpp(g) * slabs;
        case GS_DIV: return d.report_div ? group_interior_tpp(g) * slabs : 0;
        case GS_ADV_VEL:
        case GS_ADV_RHO: {
            int rx, ry, rz;
            group_extent(stage, d, rx, ry, rz);
            return group_block_tiles(rx, ry, group_div_up(rz, GROUP_ADV_ZC));
        }
        default: {
            int rx, ry, rz;
            group_extent(stage, d, rx, ry, rz);
            return group_block_tiles(rx, ry, rz);
        }
    }
}

// Tuned schedule of the grouped projection (host side).
struct GroupSchedule {
    int ctas_per_sm;        // cooperative CTAs per SM
    int zslab;              // planes per flattened tile
    long long wave_bytes;   // pressure + rhs + flags bytes per solve wave (0: one wave)
    int blocked_zchunk;     // > 0: blocked solve (GroupTBLaunch) with z-chunks of this many planes
};

// Launch configuration of one grouped step (host side).
struct GroupLaunch {
    int total[GS_COUNT];  // tiles per stage over the batch
    int ctas[GS_COUNT];   // CTAs of each grid-stride launch
    int coop_ctas;        // CTAs of the cooperative projection kernel
};

// Host launchers (kernels_group.cu).  Return 0 or a cudaError_t value.
int group_occupancy(int* coop_per_sm, int* stage_per_sm, int* sms);
int launch_group_step(const GroupArgs& a, const GroupLaunch& L, cudaStream_t st,
                      GroupTBLaunch* tb = nullptr);
int launch_group_tb_sweeps(const GroupTBLaunch& tb, int launches, cudaStream_t st);
int launch_group_sweeps_only(const GroupArgs& a, const GroupLaunch& L, cudaStream_t st);

}  // namespace smk
