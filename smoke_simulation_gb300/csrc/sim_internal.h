// The simulation handle behind smk_sim* (host side).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/smoke_gb300.h"
#include "common.cuh"

namespace smk { struct SweepMaps; struct VSweepMaps; struct AdvectMaps; }

// Records `msg` as smk_last_error's text and returns `code` (sim.cpp).
int smk_fail(int code, const std::string& msg);

#define SMK_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            return smk_fail(e_ == cudaErrorMemoryAllocation ? SMK_ERR_OOM : SMK_ERR_CUDA, \
                            std::string(#call) + ": " + cudaGetErrorString(e_));         \
        }                                                                                \
    } while (0)

// Makes `dev` the current device for the scope.
struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) {
            changed = cudaSetDevice(dev) == cudaSuccess;
        }
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
};

struct smk_sim {
    enum Kind { OBJ_OBSTACLE = 0, OBJ_SPHERE = 1, OBJ_BOX = 2 };
    struct Object {
        int kind;
        smk::SphereObj sphere;
        smk::ObstacleObj obstacle;
        smk::BoxObj box;
    };

    smk::Grid g{};
    smk_params p{};
    int device = 0;

    // Ping-pong fields (the reference's dev_smoke/u/v/w[2], smokeSimulation.cu:20-23), the
    // pressure-scheme P and b, the mask (dev_s, :24) and its derived neighbour flags.
    float* rho[2] = {nullptr, nullptr};
    float* u[2] = {nullptr, nullptr};
    float* v[2] = {nullptr, nullptr};
    float* w[2] = {nullptr, nullptr};
    // With BF16 storage (bf16 == true) rho/u/v/w point to __nv_bfloat16 arrays, and proj[]
    // holds the FP32 projected velocity advection consumes (scratch between steps).
    bool bf16 = false;      // u, v, w stored in BF16 (both BF16 storage forms)
    bool rho_bf16 = false;  // density stored in BF16 (SMK_STORAGE_BF16)
    float* proj[3] = {nullptr, nullptr, nullptr};
    float* P = nullptr;
    float* P2 = nullptr;  // second pressure buffer (temporally blocked sweeps ping-pong)
    float* b = nullptr;
    int* pcur = nullptr;  // device: which pressure buffer the last executed sweep wrote
    int* kerr = nullptr;  // device: a bounded wait in a kernel gave up (sticky until read)
    int* kerr_host = nullptr;  // page-locked: *kerr as copied at the end of an smk_simulate step
    int* gcount = nullptr;  // device: tolerance groups done by a graph's device-side group loop
    unsigned long long* loop_launches = nullptr;  // device: kernels launched by those loops
    smk::RefineStatus* refine = nullptr;          // device: FP64-checked refinement rounds
    void* render_scratch = nullptr;               // device: the renderer's light buffer per plane
    size_t render_scratch_bytes = 0;
    smk::SweepMaps* maps = nullptr;  // TMA tensor maps of P, P2, b, flags
    smk::AdvectMaps* amaps = nullptr;  // TMA tensor maps of the velocity advection's inputs
    smk::VSweepMaps* vmaps = nullptr;  // TMA tensor maps of u, v, w (both buffers), P, P2, b, flags
    uint8_t* s = nullptr;
    uint8_t* flags = nullptr;
    smk::StepStatus* status = nullptr;
    smk::StepStatus* tune_status = nullptr;  // status of the autotuner's timing launches
    int status_groups = 0;

    int index_now = 1;  // indexNow (:707)
    std::vector<Object> objects;
    bool mask_dirty = true;
    bool obstacles_dirty = false;

    // sweep kernel: 0 = one colour pass per launch; T > 0 = temporally blocked, T passes per
    // launch over z-chunks of sweep_zchunk planes (chosen by smk_set_sweep_kernel / autotune)
    int sweep_depth = 4;
    int sweep_zchunk = 47;
    int sweep_rows = 2;  // cell rows of a thread's patch in the blocked kernel (2 or 4)
    // reference scheme: 0 = one colour pass per launch (k_project_velocity); T = 2 or 4 = the
    // temporally blocked velocity sweep, T passes per launch over z-chunks of vsweep_zchunk planes
    // (the pressure buffers P, P2, b hold the intermediate face arrays); smk_autotune chooses
    int vsweep_depth = 0;
    int vsweep_zchunk = 0;  // 0: chosen from the grid
    // the blocked velocity sweep used P, P2, b as scratch: a PRESSURE step must restart its
    // pressure from zero (cleared in step(), outside any captured graph)
    bool pressure_clobbered = false;
    // steps since the pressure history started (creation, smk_write_state, a pressure reset):
    // decides between omega and omega_warm (pressure_omega)
    long long hist_steps = 0;
    double pressure_omega() const {
        return (p.warm_start && p.omega_warm > 0.0 && hist_steps >= p.omega_warm_after) ? p.omega_warm : p.omega;
    }
    // smk_params.warm_extrapolate: Ph holds the pressure the previous step's solve started from
    // (the solution of the step before it), saved by every rhs pass from step ph_from on; a solve
    // extrapolates once two solves of the history exist and Ph was saved by the previous step
    float* Ph = nullptr;
    int ph_from = 0;
    int enable_pressure_history();
    bool keeps_history() const {
        return p.projection == SMK_PROJECT_PRESSURE && p.warm_start && p.warm_extrapolate > 0.0f && Ph != nullptr;
    }
    float extrapolation() const {
        return (keeps_history() && hist_steps >= 2 && steps > ph_from) ? p.warm_extrapolate : 0.0f;
    }

    bool timing = false;
    cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    long long launches = 0;
    int steps = 0;

    // what the last step ran (for smk_get_stats)
    int last_projection = 0;
    float last_tol = 0.0f;
    int last_max_sweeps = 0;
    int last_check_every = 1;
    int last_groups = 0;
    int last_refine = 0;

    size_t elems() const { return (size_t)g.XY * (size_t)(g.nz + 1); }
    int alloc();
    void release();
    int upload_mask(const uint8_t* host);
    // CUDA graph replay of steady-state steps, one graph per ping-pong parity
    struct GraphSlot {
        cudaGraphExec_t exec = nullptr;
        std::string sig;
        long long launches = 0;
        int groups = 0;
    };
    bool use_graphs = true;
    // in a captured step, the tolerance groups of the blocked solve run as a device-side WHILE
    // loop (graph conditional node) instead of launches for every group up to the cap
    bool graph_loops = true;
    bool vec_stages = true;  // 4-wide forcing / rhs / subtract kernels where the layout allows
    bool fuse_subtract = false;  // the gradient subtract inside the solve's last sweep launch
    GraphSlot graphs[2];
    cudaStream_t cap_stream = nullptr;
    cudaStream_t body_stream = nullptr;  // captures the loop body
    // smk_simulate into page-locked host memory: the step issues its advection in z-slabs and
    // copies each slab's density planes to rb_host on rb_stream as soon as the slab is advected,
    // so that the copies overlap the rest of the advection (joined before the step ends); rb_host
    // is set only for the duration of that step.  rb_slabs < 0: one slab per 16 MiB of density,
    // 1 to 8 (a slab costs a copy and two launches: measured at 256^3, 4 slabs 1.88 ms per call,
    // 8 slabs 1.89, 16 slabs 2.03, the copy after the step 2.08; at 128^3, 2 slabs 0.376 ms,
    // 8 slabs 0.52, after the step 0.383)
    float* rb_host = nullptr;
    int rb_slabs = -1;
    int readback_slabs() const {
        if (rb_slabs >= 0) return rb_slabs;
        const long long n = (long long)g.nx * g.ny * g.nz * 4 / (16LL << 20);
        return (int)(n < 1 ? 1 : n > 8 ? 8 : n);
    }
    cudaStream_t rb_stream = nullptr;
    cudaEvent_t rb_fork = nullptr, rb_join = nullptr;

    int step(float dt, cudaStream_t st);
    int enqueue(float dt, cudaStream_t st);
    std::string graph_signature(float dt) const;
    // The one-off part of a step after a mask or obstacle change (fillObstacle, neighbour
    // flags), as enqueue issues it; used before a grouped step.  Returns the kernels launched.
    int prepare_mask(cudaStream_t st);
};

// After a synchronisation point of the simulation's work: report (and clear) a bounded device
// wait that gave up (sim.cpp).
int check_kernel_error(smk_sim* sim);

// ---- grouped steps over many simulations (batch.cpp) -----------------------------------------
namespace smk { struct GroupSchedule; }
struct GroupRunner;
GroupRunner* group_runner_create();
// The simulation can be a member of a grouped step (its parameters are ones the grouped
// kernels run).
bool group_runner_eligible(smk_sim* sim);
void group_runner_destroy(GroupRunner* r);
// One grouped step of `n` simulations (dts[i] each) on `st` with direct launches; the
// per-step tables come from a ring of device buffers recycled once their step completed.
// Members must use the PRESSURE projection.  *kernels (may be NULL) receives the launches.
int group_runner_step(GroupRunner* r, smk_sim* const* sims, const float* dts, int n,
                      const smk::GroupSchedule& sched, cudaStream_t st, int* kernels);
