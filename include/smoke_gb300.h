/*
 * smoke_gb300.h -- C ABI of libsmoke_gb300, a GB300-native (sm_103a) implementation of the
 * semi-Lagrangian smoke step of RasmusAlmryd/smoke-simulation on a staggered MAC grid.
 *
 * The reference exposes one implicit simulation through ten C++ free functions
 * (project/smokeSimulation.cuh:4-17).  This ABI keeps the same operations but with an explicit
 * handle, status codes instead of exit(-1), and stream-ordered steps.  The reference's own
 * C++ signatures are also exported by the library (include/smokeSimulation_gb300.cuh).
 *
 * Conventions
 *   - Every function returns SMK_OK (0) or an SMK_ERR_* code; smk_last_error() gives detail.
 *   - Host arrays use the reference's layout (smokeSimulation.cu:127-147): cells
 *     nx*ny*nz floats, faces (nx+1)*(ny+1)*(nz+1) floats per component, x fastest.
 *   - Mask bytes: nonzero = fluid, 0 = solid (the reference's dev_s, :24, :200-207, :306-309).
 *   - `stream` arguments are cudaStream_t passed as void* (NULL = the legacy default stream).
 *   - A handle is not thread-safe; distinct handles are independent.
 */
#ifndef SMOKE_GB300_H
#define SMOKE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SMK_OK 0
#define SMK_ERR_INVALID 1     /* bad argument (null pointer, size, id) */
#define SMK_ERR_CUDA 2        /* a CUDA runtime call failed */
#define SMK_ERR_OOM 3         /* device memory allocation failed */
#define SMK_ERR_STATE 4       /* call not valid in the current state */
#define SMK_ERR_TIMEOUT 5     /* a bounded device wait gave up */

/* Projection schemes. */
#define SMK_PROJECT_REFERENCE 0 /* in-place velocity red-black SOR, bit-exact with the reference */
#define SMK_PROJECT_PRESSURE 1  /* pressure red-black SOR on P, then one pass subtracting grad P */
#define SMK_SOLVER_RBSOR 0
#define SMK_SOLVER_JACOBI 1

/* Velocity clamp modes. */
#define SMK_CLAMP_REFERENCE 0 /* if |u|^2*dt > c^2 scale by c^2/(|u|^2*dt) (smokeSimulation.cu:343-349) */
#define SMK_CLAMP_MAGNITUDE 1 /* |u| <= c */
#define SMK_CLAMP_NONE 2

/* Storage precision of the advected fields (u, v, w, density). */
#define SMK_STORAGE_F32 0
#define SMK_STORAGE_BF16 1     /* density and u, v, w in BF16 (FP32 arithmetic, FP32 pressure) */
#define SMK_STORAGE_BF16_VEL 2 /* u, v, w in BF16, density in FP32 */

typedef struct smk_sim smk_sim;

typedef struct smk_params {
    float gravity;      /* reference: -9.82 (smokeSimulation.cu:28) */
    float buoyancy;     /* reference: 2.0   (:29) */
    float clamp_const;  /* reference: MAX_VELOCITY_PER_STEP 3.0 (:39) */
    int clamp_mode;     /* SMK_CLAMP_* */
    int projection;     /* SMK_PROJECT_* */
    int max_sweeps;     /* red+black sweeps; reference: num_iterations 30 (:797) */
    double omega;       /* over-relaxation; reference: OVER_RELAXATION 1.9 (:38) */
    float tol;          /* PRESSURE only: stop on max|residual| <= tol (0: fixed sweeps) */
    int check_every;    /* PRESSURE only: residual check cadence in sweeps */
    int warm_start;     /* PRESSURE only: keep the pressure across steps */
    int report_div;     /* measure max|div u| after the projection every step */
    int storage;        /* SMK_STORAGE_* (F32 only for PROJECT_REFERENCE) */
    int refine;         /* PRESSURE with tol > 0: FP64-checked refinement rounds after the
                           solve (0: none).  Each round measures max|div u| of the projected
                           velocity with FP64 accumulation; while a cell exceeds tol it solves
                           for a correction (refine_sweeps FP32 sweeps on the FP64 divergence,
                           rounded) and applies it to the velocity and the pressure. */
    int refine_sweeps;  /* sweeps of each correction solve */
    int obstacle_velocity; /* 1: the obstacles' velocity (stored but unused by the reference,
                              smokeSimulation.cu:299-301) drives the fluid: after forcing, every
                              face touching a cell of the last obstacle (the one that decides the
                              mask) takes that obstacle's velocity, a moving boundary the
                              projection then respects.  0 (default): the reference's behaviour. */
    int solver;         /* PRESSURE only: SMK_SOLVER_RBSOR (default) red-black SOR, or
                           SMK_SOLVER_JACOBI weighted Jacobi: every cell from the previous
                           iterate, P += (omega/acc) * residual, one iteration per "sweep" (use
                           omega <= 1); the refinement rounds' correction solves stay red-black. */
    double omega_warm;  /* PRESSURE with warm_start: the over-relaxation of the solves from the
                           (omega_warm_after + 1)-th step after the pressure history started (at
                           creation, smk_write_state, or a switch from the REFERENCE scheme); the
                           earlier steps use omega.  0 (default): omega throughout.  A warm-started
                           solve corrects the last step's pressure, an error of shorter wavelength
                           than a cold start's, which a smaller over-relaxation damps in fewer
                           sweeps (256^3 workload at tol 1e-4: 22.6 instead of 35.3 sweeps per step
                           with 1.75 after 2 steps).  Every batch form and serving mode follows
                           it per grid. */
    int omega_warm_after; /* see omega_warm; default 2 */
    float warm_extrapolate; /* PRESSURE with warm_start: a solve starts from the last pressure
                             extrapolated along the last change, P + a (P - P_before), once two
                             solves of the history exist (a = this value, 0..1; 0, the default:
                             the last pressure).  Keeps one more pressure array.  256^3 workload
                             at tol 1e-4: 20.4 instead of 23.1 sweeps per step over the first 20
                             steps with a = 0.5; a = 0.75 and 1 let the solve error grow and are
                             not stable.  Every batch form and serving mode follows it per
                             grid. */
} smk_params;

typedef struct smk_stats {
    int sweeps;         /* sweeps performed by the last step's projection */
    int converged;      /* tolerance reached (PRESSURE with tol > 0) */
    float resid_max;    /* max |residual| at the last residual check */
    float div_max;      /* max |div u| after projection (report_div), else -1 */
    int step_index;     /* steps taken since creation */
    int refine_rounds;  /* correction rounds applied by the last step (refine > 0) */
    float div64_max;    /* max |div u| of the last FP64 measurement (refine > 0), else -1 */
    int subtract_fused; /* 1: the last step's gradient subtract ran inside its last sweep launch
                           (PRESSURE, FP32, blocked sweeps), 0: as a pass of its own */
} smk_stats;

/* Host copy of the full state in the reference's layout (both ping-pong buffers). */
typedef struct smk_host_state {
    float* rho[2];
    float* u[2];
    float* v[2];
    float* w[2];
    uint8_t* s;
    int index_now;      /* the reference's indexNow (smokeSimulation.cu:707); 1 after init */
} smk_host_state;

/* The reference's constants (smokeSimulation.cu:28-39, :797), PROJECT_REFERENCE, F32. */
void smk_default_params(smk_params* p);

/* Status text for a code, and the last error message of the calling thread. */
const char* smk_error_string(int code);
const char* smk_last_error(void);

/* Allocate a simulation of nx*ny*nz cells on the current device.  The state matches the
 * reference's initializeVolume (smokeSimulation.cu:124-238): density zero, velocities zero,
 * mask fluid except the y = 0 floor.  Replaces initializeVolume's allocation part. */
int smk_create(int nx, int ny, int nz, const smk_params* params, smk_sim** out);
/* Free everything (replaces deleteVolume, :240-248). */
int smk_destroy(smk_sim* sim);

int smk_set_params(smk_sim* sim, const smk_params* params);
int smk_get_params(const smk_sim* sim, smk_params* params);
int smk_get_dims(const smk_sim* sim, int* nx, int* ny, int* nz);

/* Upload density into buffer [0] (initializeVolume's H2D copy, :138). */
int smk_set_density(smk_sim* sim, const float* host_rho);
/* Replace the solid mask (nx*ny*nz bytes, nonzero = fluid). Registered obstacles still
 * overwrite interior cells every step, as fillObstacle does (:289-313). */
int smk_set_solid_mask(smk_sim* sim, const uint8_t* host_s);

/* Object registry (addObstacle :88-95, addSmokeSource :97-104, updateObjectPos :106-109).
 * Ids are sequential across kinds, as in the reference.  No cap on the object count. */
int smk_add_obstacle(smk_sim* sim, float x, float y, float z, float vx, float vy, float vz, float r,
                     int* id);
int smk_add_smoke_source(smk_sim* sim, float x, float y, float z, float r, int* id);
/* Box emitter over cells [x0,x1)x[y0,y1)x[z0,z1): density into both buffers each step (the
 * reference's documented emulation of a box source); when set_vy, v-faces below and above each
 * box cell are set to vy before forcing. */
int smk_add_box_emitter(smk_sim* sim, int x0, int y0, int z0, int x1, int y1, int z1,
                        float density, float vy, int set_vy, int* id);
int smk_update_object_pos(smk_sim* sim, int id, float x, float y, float z);
int smk_clear_objects(smk_sim* sim);

/* One step, stream-ordered (no host synchronisation): the stage sequence of simulate()
 * (:774-811) without its D2H copy. */
int smk_step(smk_sim* sim, float dt, void* stream);
/* simulate(float*, dt) (:774-819): one step, then a blocking copy of the new density into
 * host_out (nx*ny*nz floats).  When host_out is page-locked (cudaHostAlloc, cudaHostRegister)
 * and the density is stored in FP32, the copy overlaps the step's advection: the advection runs
 * in z-slabs and each slab's density planes go to host_out while the next slab computes
 * (smk_set_readback_slabs).  Otherwise the copy follows the step. */
int smk_simulate(smk_sim* sim, float* host_out, float dt);
/* Slabs of smk_simulate's overlapped readback: 1..64, 0 = the copy after the step, -1 (the
 * default) = one slab per 16 MiB of density, 1 to 8 (4 at 256^3).  The result is the same for
 * every count.  smk_get_readback_slabs gives the count this simulation uses. */
int smk_set_readback_slabs(smk_sim* sim, int slabs);
int smk_get_readback_slabs(const smk_sim* sim, int* slabs);
/* Copy the current density (the buffer the last step wrote) to host or device memory,
 * stream-ordered; call smk_sync (or synchronise the stream) before reading a host copy. */
int smk_read_density(smk_sim* sim, float* dst, int dst_on_device, void* stream);
int smk_sync(smk_sim* sim, void* stream);

/* Full state in the reference layout (checkpoint / resume, parity checks).  Blocking.  The
 * state is the reference's (fields, mask, ping-pong index); writing one also restarts the
 * PRESSURE projection's warm-start history, so the next step starts from zero pressure as the
 * first step of a new simulation does. */
int smk_read_state(smk_sim* sim, const smk_host_state* st);
int smk_write_state(smk_sim* sim, const smk_host_state* st);
/* The projected velocities of the last step (buffer "now" after projection) are not kept
 * separately; smk_read_state returns both buffers as the reference holds them. */

/* Statistics of the last step (blocking). */
int smk_get_stats(smk_sim* sim, smk_stats* out);

/* Per-stage device times of the last step, measured with CUDA events on the step's stream
 * when timing is enabled.  Stages: 0 objects+emitters, 1 forcing, 2 projection,
 * 3 advection, 4 whole step, 5 the sweep phase inside the projection (red-black passes and
 * residual checks; PRESSURE only, else 0).  Blocking. */
int smk_set_timing(smk_sim* sim, int enable);
int smk_get_stage_times(smk_sim* sim, float* ms, int count);
/* Number of kernel launches the library issued since creation. */
long long smk_launch_count(const smk_sim* sim);

/* Pressure sweep kernel (PRESSURE projection).  depth 0: one colour pass per launch.
 * depth 2, 4 or 6: temporally blocked, `depth` colour passes per pass over HBM, the grid
 * cut into z-chunks of `zchunk` planes (>= 1).  Results are bit-identical for every choice;
 * only speed differs.  No counterpart in the reference (its projection is fixed,
 * smokeSimulation.cu:795-801). */
int smk_set_sweep_kernel(smk_sim* sim, int depth, int zchunk);
int smk_get_sweep_kernel(const smk_sim* sim, int* depth, int* zchunk);
/* The same with the blocked kernel's patch height: `rows` cell rows per thread (2 with depth 2,
 * 4 or 6; 4 with depth 4: a 64 x 32 tile of 8 warps instead of 16), or 2 | SMK_SWEEP_YCLUSTER
 * with depth 6 (ny <= 256): the CTAs of one x-z column form a thread-block cluster spanning y
 * and exchange their boundary rows through distributed shared memory instead of recomputing a
 * halo; 2 | SMK_SWEEP_YCLUSTER | SMK_SWEEP_YCLUSTER_N(n), n = 2 or 4, with depth 6 (any ny):
 * clusters of n CTAs along y exchange boundary rows the same way, with a halo only at the ends
 * of each cluster's rows.  smk_set_sweep_kernel is rows = 2. */
#define SMK_SWEEP_YCLUSTER 0x100
#define SMK_SWEEP_YCLUSTER_N(n) ((n) << 9)
int smk_set_sweep_shape(smk_sim* sim, int depth, int rows, int zchunk);
int smk_get_sweep_shape(const smk_sim* sim, int* depth, int* rows, int* zchunk);
/* Projection kernel of the REFERENCE scheme (the reference's in-place velocity red-black SOR,
 * smokeSimulation.cu:356-394 run max_sweeps times, :795-801).  depth 0 (default): one colour pass
 * per launch, as the reference launches it; depth 2 or 4: temporally blocked, `depth` colour
 * passes per pass over HBM on z-chunks of `zchunk` planes (0: chosen from the grid), with the
 * simulation's pressure buffers as scratch (a later PRESSURE step then restarts its pressure from
 * zero); smk_autotune picks the fastest.  Results are bit-identical for every choice.  FP32
 * storage only.  No counterpart in the reference's API. */
int smk_set_velocity_sweep(smk_sim* sim, int depth, int zchunk);
int smk_get_velocity_sweep(const smk_sim* sim, int* depth, int* zchunk);
/* Replay steady-state steps as a captured CUDA graph (default on).  A graph is re-captured
 * when dt, the parameters, the objects or the sweep kernel change; steps after a mask or
 * obstacle change run directly.  Results are identical either way. */
int smk_set_graphs(smk_sim* sim, int enable);
/* In a captured step, run the tolerance groups of the blocked solve as a device-side WHILE loop
 * (a graph conditional node: no launches after the solve has converged; default on) or as the
 * unrolled launches up to max_sweeps (later ones exit at entry).  Results are identical. */
int smk_set_graph_loops(smk_sim* sim, int enable);
/* Run the forcing, rhs and gradient-subtract / BF16-projection stages with four consecutive x
 * per thread (vector loads and stores; default on, used where the arrays' rows start on vector
 * boundaries, as every simulation's own arrays do) or one cell per thread.  Results are
 * identical; batches follow each member's setting.  No counterpart in the reference. */
int smk_set_vector_stages(smk_sim* sim, int enable);
/* PRESSURE scheme, FP32 state, blocked sweeps: apply the gradient subtract inside the sweep
 * launch that ends the solve (the launch that applies the last colour pass moves every face by
 * the final pressure gradient) instead of as a pass of its own after the solve.  Where only the
 * device knows which tolerance group ends the solve, each group's last launch is issued as a
 * pair, of which exactly one does the work.  Bit-identical to the separate pass; default off:
 * at 256^3 the fused launch measures 465 us against 117 us for the plain launch plus 81 us for
 * the separate pass (smk_stats.subtract_fused reports which way a step went).  Reference: the
 * face updates inside every colour pass of divergence(), smokeSimulation.cu:384-391. */
int smk_set_fused_subtract(smk_sim* sim, int enable);
/* Time the blocked sweep kernel's shapes (depth, patch rows) and z-chunk sizes on this simulation's buffers and
 * keep the fastest (cached per grid shape and device for the process).  With the REFERENCE
 * projection it times the velocity sweep instead (one colour pass per launch, or the blocked
 * kernel with depth 2 or 4 over its z-chunks; smk_set_velocity_sweep) and reports the time per
 * iteration.  Synchronises; does not change the simulation's results.  Outputs may be NULL;
 * us_per_sweep is -1 on a cache hit.  No counterpart in the reference. */
int smk_autotune(smk_sim* sim, int* depth, int* zchunk, float* us_per_sweep);

/* Batches: many independent grids of any sizes stepped together.  Members keep their own state
 * and results (identical to stepping them alone); the batch does not own them.  Two forms:
 *   GROUPED   one persistent launch per stage over every member (emitters, forcing, the whole
 *             projection as one cooperative kernel, velocity advection, density advection:
 *             five launches per batch step whatever the number of grids), replayed as a
 *             captured CUDA graph; needs the PRESSURE projection in every member;
 *   BRANCHES  one CUDA graph whose concurrent branches are the members' own single-grid steps.
 * AUTO (the default) takes GROUPED when every member allows it.  Graphs are re-captured when a
 * member's dt, parameters, objects, sweep kernel or ping-pong parity changes; a step in which a
 * member has a pending mask change or stage timing runs as BRANCHES without a graph.  No
 * counterpart in the reference (one implicit grid, smokeSimulation.cu:16-24). */
#define SMK_BATCH_AUTO 0
#define SMK_BATCH_GROUPED 1
#define SMK_BATCH_BRANCHES 2
typedef struct smk_batch smk_batch;
int smk_batch_create(int count, smk_sim* const* sims, smk_batch** out);
/* dts: one dt per member, or NULL to use dt_all for every member.  Stream-ordered. */
int smk_batch_step(smk_batch* batch, const float* dts, float dt_all, void* stream);
int smk_batch_destroy(smk_batch* batch);
int smk_batch_set_mode(smk_batch* batch, int mode);
/* Replay batch steps as captured graphs (default on); off: direct launches. */
int smk_batch_set_graphs(smk_batch* batch, int enable);
/* The form the last step ran (SMK_BATCH_GROUPED or SMK_BATCH_BRANCHES; 0 before the first
 * step) and the kernels the batch has launched so far (either pointer may be NULL). */
int smk_batch_get_info(const smk_batch* batch, int* last_mode, long long* launches);
/* Time the grouped projection's schedules (the cooperative colour-pass kernel: CTAs per SM, z
 * planes per tile, solve-wave budget; the blocked solve: z-chunk) on the members' scratch
 * pressure buffers and keep the fastest.  Synchronises; does not change any member's results.
 * Outputs may be NULL (ctas_per_sm is 0 when the blocked solve wins). */
int smk_batch_autotune(smk_batch* batch, int* ctas_per_sm, float* us_per_sweep);
/* The grouped projection's schedule: cooperative CTAs per SM (0: all resident), z planes per
 * sweep tile, and the solve-wave budget in bytes of pressure + rhs + flags (0: one wave; else
 * members are packed into waves solved one after another so a wave's passes stay in L2).
 * Results do not depend on it. */
int smk_batch_get_schedule(const smk_batch* batch, int* ctas_per_sm, int* zslab, long long* wave_bytes);
int smk_batch_set_schedule(smk_batch* batch, int ctas_per_sm, int zslab, long long wave_bytes);
/* The grouped form's blocked solve: zchunk > 0 replaces the cooperative kernel's colour passes
 * by launches of the temporally blocked sweep kernel over every member's tiles (3 sweeps per
 * launch, z-chunks of `zchunk` planes, the tolerance groups as a device-side loop in the
 * captured step), when every member has a tolerance rule with the same group size and sweep
 * cap; 0 = colour passes.  smk_batch_set_schedule resets it to 0.  Results do not depend on
 * it. */
int smk_batch_set_blocked(smk_batch* batch, int zchunk);
int smk_batch_get_blocked(const smk_batch* batch, int* zchunk);

/* Serving: many simulation requests kept resident on one GPU with continuous admission.  No
 * counterpart in the reference (one simulation stepped from the render loop, main.cpp:889-896).
 * smk_server_tick retires requests whose last step completed (their density goes to
 * out_density), admits queued requests in arrival order while the device-memory budget and
 * the slot limit allow, and issues the next step of every active request (work of different
 * requests overlaps: concurrent streams, or one grouped step, see smk_server_set_mode).
 * Per-step latency = device time of a request's step, measured with events.  Each request is
 * an independent simulation: its results are the same alone and in the mix. */
#define SMK_REQ_QUEUED 0
#define SMK_REQ_ACTIVE 1
#define SMK_REQ_DONE 2
#define SMK_REQ_FAILED 3
#define SMK_REQ_CANCELLED 4
typedef struct smk_server smk_server;
typedef struct smk_request_desc {
    int nx, ny, nz;            /* grid cells */
    int steps;                 /* steps to run */
    float dt;
    const smk_params* params;  /* NULL: smk_default_params */
    const uint8_t* mask;       /* host, nx*ny*nz bytes (1 = fluid); NULL: reference initial mask */
    const float* spheres;      /* sphere sources, 4 floats each (x, y, z, r) */
    int n_spheres;
    const float* boxes;        /* box emitters, 9 floats each (x0,y0,z0,x1,y1,z1,density,vy,set_vy) */
    int n_boxes;
    const float* obstacles;    /* obstacles, 7 floats each (x,y,z,vx,vy,vz,r) */
    int n_obstacles;
    float* out_density;        /* nx*ny*nz floats written at completion (may be NULL): host memory
                                  (page-locked by the server while the request lives, so the copy
                                  is asynchronous), or device memory when out_on_device */
    int out_on_device;         /* out_density is device memory: the handoff is a stream-ordered
                                  device-to-device copy, no host involvement */
} smk_request_desc;
typedef struct smk_server_stats {
    long long steps_completed;
    int requests_completed;
    int active, queued;
    double cell_updates;
    size_t bytes_in_use;
    float p50_step_ms, p99_step_ms, max_step_ms;
    /* queueing delay of the admitted requests: host time from smk_server_submit to admission */
    float p50_queue_ms, p99_queue_ms, max_queue_ms;
    int peak_active, peak_queued;  /* most requests resident / waiting at once */
    size_t peak_bytes;             /* most budgeted device memory in use at once */
} smk_server_stats;
int smk_server_create(size_t budget_bytes, int max_active, smk_server** out);
/* Serving form, before the first request runs: STREAMS (default) steps every request with its
 * own single-grid kernels on its own stream; GROUPED issues one grouped step (the batch's
 * GROUPED kernels) over all active requests per tick.  Results are the same in both. */
#define SMK_SERVE_STREAMS 0
#define SMK_SERVE_GROUPED 1
int smk_server_set_mode(smk_server* server, int mode);
/* smk_set_graph_loops for the requests admitted from now on (default off: with many request
 * graphs in flight at once, the loop's per-iteration cost exceeds the launches it saves). */
int smk_server_set_graph_loops(smk_server* server, int enable);
/* GROUPED form: the blocked solve, with z-chunks of `zchunk` planes, for the ticks whose requests
 * share a tolerance group size and sweep cap (smk_batch_set_blocked; default 137; 0 = cooperative
 * colour passes for every tick). */
int smk_server_set_blocked(smk_server* server, int zchunk);
int smk_server_submit(smk_server* server, const smk_request_desc* request, int* id);
int smk_server_tick(smk_server* server, int* n_active, int* n_queued);
int smk_server_request_status(smk_server* server, int id, int* state, int* steps_done, int* error);
/* Cancel a request: a queued one is dropped now; an active one gets no further steps and is
 * released (no density copy) by the tick after its issued steps have completed.  Cancelling a
 * finished request does nothing. */
int smk_server_cancel(smk_server* server, int id);

int smk_server_get_stats(smk_server* server, smk_server_stats* out);
int smk_server_destroy(smk_server* server);
const char* smk_server_last_error(void);

/* Pressure projection of a caller-owned velocity field that allocates no device memory.
 * No counterpart in the reference.  It is for callers that cannot call cudaMalloc when they need
 * the projection: an application that has handed the device's memory to its own pool allocator
 * or runs under a fixed memory budget, or a plugin called from a per-frame or per-request
 * callback where cudaMalloc's implicit device-wide synchronisation would stall other work.
 * u, v, w: device arrays in the reference's face layout ((nx+1)(ny+1)(nz+1) floats, x fastest),
 * projected in place; mask: device array of nx*ny*nz bytes, nonzero = fluid.  Runs the PRESSURE
 * scheme's red-black SOR from a zero pressure (params->projection must be SMK_PROJECT_PRESSURE,
 * solver SMK_SOLVER_RBSOR, refine 0; warm_start is ignored) with params->max_sweeps, omega
 * (0 < omega < 2), tol and check_every; the result equals, bit for bit, the projection that
 * smk_step's PRESSURE scheme applies to the same field and mask from a zero pressure.  Scratch comes from one fixed device array inside the
 * library (about 19 MB, held by every GPU that loads the library until exit): grids with
 * (nx+1)(ny+1)(nz+1) > 2,097,152 or nz > 65535 are rejected with SMK_ERR_INVALID.  All calls
 * share that array and find the previous call's contents in it (each call rewrites what it
 * reads): calls that overlap on the GPU race; order them on one stream.  The first call on a
 * device, with that device current, looks up the array's address (cudaGetSymbolAddress; again
 * after the device's context was replaced, e.g. by cudaDeviceReset): make it before any stream
 * capture.  stats may be NULL (stream-ordered call); when given, the call synchronises `stream`
 * and fills sweeps/converged/resid/div, and `stream` must not be under capture. */
int smk_project_noalloc(float* u, float* v, float* w, const uint8_t* mask, int nx, int ny, int nz,
                        const smk_params* params, smk_stats* stats, void* stream);
/* The size limit above, and the message of the last failed smk_project_noalloc call. */
long long smk_project_noalloc_max_elems(void);
const char* smk_project_noalloc_last_error(void);

/* Headless volume renderer: the reference's half-angle slice compositing with a light buffer
 * (project/texVolume.frag:27-52, light.frag:16-23, the two-pass drawing and blend equations of
 * main.cpp:369-419, 474-476, 660-661, 676-687, proxy planes of boundingBox.cpp:135-181,
 * 228-345) restated as CUDA kernels writing device images; no graphics API is used.  Proxy
 * plane i (of `planes`, perpendicular to the half vector between the view and light directions)
 * is drawn into the eye buffer (density x light-buffer colour, blended front-to-back when camera
 * and light face the same way, else back-to-front) and then into the light buffer (colour x
 * (1 - density)).  Both buffers hold half-precision RGBA as the reference's RGBA16F framebuffers
 * do.  Defaults are the reference application's (camera, light, 512^2 light buffer, 100 planes,
 * 45-degree perspectives with near 5 / far 2000, box at the origin with unit cells). */
typedef struct smk_render_params {
    int width, height;        /* eye image (the reference: the window) */
    int light_res;            /* light buffer side (lightMapResolution 512) */
    int planes;               /* proxy planes (proxy_step_count 100) */
    float camera_pos[3];      /* (1, 20, 100) */
    float camera_dir[3];      /* toward the box centre */
    float up[3];              /* (0, 1, 0) */
    float fovy_deg, znear, zfar;                   /* 45, 5, 2000 */
    float light_pos[3];                            /* (120, 80, 0) */
    float light_fovy_deg, light_znear, light_zfar; /* 45, 5, 2000 (aspect 1) */
    float light_color[3];     /* (0.9882, 0.9333, 0.7549) */
    float box_pos[3];         /* box centre (0, 0, 0) */
    float cell_size;          /* world units per cell (1) */
    float bg_color[3];        /* 20/255 grey */
} smk_render_params;
void smk_default_render_params(smk_render_params* rp);
/* Render the simulation's current density.  eye_rgba: device, width*height*4 floats (the eye
 * buffer, rows bottom-up as in OpenGL); composite_rgb: device, width*height*3 floats (the eye
 * buffer blended over bg_color as the reference's final pass does) or NULL.  Stream-ordered;
 * scratch (the light buffer after every plane) is kept with the simulation. */
int smk_render(smk_sim* sim, const smk_render_params* rp, float* eye_rgba, float* composite_rgb,
               void* stream);

/* Proxy-slice geometry on the device: the reference's proxy-plane polygons
 * (boundingBox.cpp:135-181, 228-345) for callers that draw them with a graphics API.  Plane i of
 * `planes` is perpendicular to normalize(-view_dir) at (i + 0.5) / planes between the box's
 * extreme projections; outputs (device): vertices planes*7*3 floats (plane i: counts[i] polygon
 * points sorted by pseudo-angle, then the centroid, rest 0), counts planes ints, triangles
 * planes*6*3 ints (fan around the centroid, indices into the vertex array; -1 rows unused). */
int smk_proxy_planes(const float view_origin[3], const float view_dir[3], const float box_pos[3],
                     const float dims[3], int planes, float* vertices, int* counts, int* triangles, void* stream);

/* Testing: the next `count` smk_create calls fail with SMK_ERR_OOM as a device allocation
 * failure would, without touching the device (host-side fault injection). */
int smk_inject_alloc_failures(int count);
/* Testing: the next cooperative grouped-projection launch made outside a graph capture (batch
 * GROUPED form with graphs off) has its CTA 0 skip its arrival at grid barrier `barrier`
 * (1-based; 0 cancels a pending injection), and its barrier waits give up after wait_ms
 * (1..10000) instead of 2 s: every wait on that barrier runs out, every CTA leaves the kernel, and
 * the members' next synchronisation reports SMK_ERR_TIMEOUT.  No device fault is involved; the
 * context stays usable.  smk_barrier_timeout_report synchronises the device and gives, for that
 * launch, how many CTAs left because a barrier gave up and how many it had. */
int smk_inject_barrier_timeout(int barrier, int wait_ms);
int smk_barrier_timeout_report(int* ctas_left, int* ctas);
/* Testing (host only, no device): the exact arithmetic of the blocked REFERENCE-scheme sweep on
 * n values: scaled[i] = float(double(x[i]) * omega) and quotient[i] = x[i] / d[i] (d in 1..6) as
 * the kernel computes them without the FP64 pipe (either output may be NULL). */
int smk_test_exact_arith(const float* x, const int* d, int n, double omega, float* scaled, float* quotient);
/* Testing: the blocked velocity sweep's per-cell p_t = float(double(x / d) * omega), d = 1..6,
 * through its branch-free common path and its out-of-line path for rare operands (host
 * instance). */
int smk_test_exact_cell(const float* x, const int* d, int n, double omega, float* pt);

#ifdef __cplusplus
}
#endif

#endif /* SMOKE_GB300_H */
