// Host-side launchers of the step's kernels (implemented in the .cu files).
#pragma once
#include <initializer_list>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace smk {

// Stage a4: emitters and obstacles.
// Storage-typed launchers are instantiated for float (FP32 form) and __nv_bfloat16 (BF16
// storage form); arithmetic is FP32 in both.
template <typename T, typename Tv>
void launch_emit_boxes(const Grid& g, T* rho0, T* rho1, Tv* v_now, const BoxObj* boxes, int nb,
                       cudaStream_t st);
template <typename T>
void launch_fill_smoke(const Grid& g, T* rho0, T* rho1, const SphereObj* sp, int ns, cudaStream_t st);
// Union bounding box (one cell of margin) of spheres, clipped to the interior [1, n-2]:
// [a0, a1) per axis; false when empty.
bool sphere_bounds(const Grid& g, const SphereObj* sp, int ns, int a0[3], int a1[3]);
void launch_fill_obstacles(const Grid& g, uint8_t* s, const ObstacleObj* ob, int no, cudaStream_t st);
// Neighbour flags from the mask; zeroes the pressure where a cell is not projectable.
void launch_build_flags(const Grid& g, const uint8_t* s, uint8_t* flags, cudaStream_t st);

// Moving-obstacle boundary (smk_params.obstacle_velocity): faces touching a cell of `last`
// take its velocity.
template <typename Tv>
void launch_obstacle_velocity(const Grid& g, Tv* u, Tv* v, Tv* w, const ObstacleObj& last, cudaStream_t st);

// Stage b: integrate (forcing) + velocityConfinement (clamp), fused.
template <typename Tv, typename T>
void launch_forcing(const Grid& g, Tv* u, Tv* v, Tv* w, const T* rho,
                    const uint8_t* flags, float dt, float gravity, float buoyancy, float clamp_const,
                    int clamp_mode, cudaStream_t st, bool vec = true);

// Stage d (reference scheme): one colour pass of the in-place velocity red-black SOR.
void launch_project_velocity(const Grid& g, float* u, float* v, float* w, const uint8_t* flags,
                             int colour, double omega, cudaStream_t st);

// Stage c/d (pressure scheme).
template <typename T>
// Ph (may be NULL): the pressure history of smk_params.warm_extrapolate (body_rhs), alpha its
// extrapolation factor for this step (0: start from the last pressure, still saving it).
void launch_rhs(const Grid& g, const T* u, const T* v, const T* w, const uint8_t* flags,
                float* b, float* P, const float* P2, const int* pcur, int warm, cudaStream_t st, bool vec = true,
                float* Ph = nullptr, float alpha = 0.0f);
// One weighted Jacobi iteration Pin -> Pout (see k_jacobi); *pcur = out_idx when it runs.
void launch_jacobi(const Grid& g, const float* Pin, float* Pout, const float* b, const uint8_t* flags,
                   const float* wacc7, const StepStatus* status, int* pcur, int out_idx, cudaStream_t st);
void launch_sweep(const Grid& g, float* P, const float* b, const uint8_t* flags, int colour,
                  const float* wacc7, const StepStatus* status, cudaStream_t st);
void launch_resid_check(const Grid& g, const float* P, const float* b, const uint8_t* flags,
                        StepStatus* status, int group, float tol, cudaStream_t st);
// skip (device, may be NULL): when *skip is set at run time the launch does nothing (a blocked
// launch already applied the subtract, SweepFuse).
void launch_gradient_subtract(const Grid& g, float* u, float* v, float* w, const float* P0,
                              const float* P1, const int* pcur, const uint8_t* flags,
                              cudaStream_t st, bool vec = true, const int* skip = nullptr);
// Temporally blocked sweeps: nhalf <= T colour passes in one pass over HBM, P_in -> P_out;
// `check` launches also record the residual of the input state for tolerance group `group`.
// The pressure buffers are read through TMA tensor maps built once per simulation.
// The 4-wide stage kernels (vector loads and stores of four consecutive x) need rows that start
// on vector boundaries: a row pitch that is a multiple of 4 elements, 16-byte aligned float
// arrays, 8-byte aligned bf16 arrays and 4-byte aligned byte arrays.  Callers with other layouts
// get the per-cell kernels.
inline bool vec4_layout(const Grid& g, std::initializer_list<const void*> floats, const void* bytes,
                        std::initializer_list<const void*> halves = {}) {
    if (g.X % 4 != 0 || g.XY % 4 != 0) return false;
    for (const void* p : floats)
        if (p != nullptr && (reinterpret_cast<uintptr_t>(p) & 15u) != 0) return false;
    for (const void* p : halves)
        if (p != nullptr && (reinterpret_cast<uintptr_t>(p) & 7u) != 0) return false;
    return (reinterpret_cast<uintptr_t>(bytes) & 3u) == 0;
}
// vec4_layout for arrays of storage type T (float or bf16).
template <typename T>
inline bool vec4_layout_of(const Grid& g, std::initializer_list<const T*> ts,
                           std::initializer_list<const void*> floats, const void* bytes) {
    for (const T* p : ts) {
        const uintptr_t m = sizeof(T) == 4 ? 15u : 7u;
        if (p != nullptr && (reinterpret_cast<uintptr_t>(p) & m) != 0) return false;
    }
    return vec4_layout(g, floats, bytes);
}

// Supported shapes: `rows` = cell rows of a thread's patch (2: T = 2, 4, 6; 4: T = 4), or
// 2 | SWEEP_YCLUSTER | (n << SWEEP_YCLUSTER_N_SHIFT) with T = 6: 2-row patches whose CTAs form
// thread-block clusters along y exchanging boundary rows through distributed shared memory;
// n = 0: one cluster spans the y extent (ny <= 256), n = 2 or 4: clusters of n CTAs with a
// halo only at the ends of each cluster's rows.
constexpr int SWEEP_YCLUSTER = 0x100;
constexpr int SWEEP_YCLUSTER_N_SHIFT = 9;
inline int sweep_ycluster_n(int rows) { return (rows >> SWEEP_YCLUSTER_N_SHIFT) & 0xf; }
int sweep_tb_shape_supported(int T, int rows);
// Clusters of the y-cluster form with n_req CTAs each (0: one spanning y) that can be resident
// at once for grid g (0: not usable).
int sweep_ycluster_usable(const Grid& g, int n_req);
// Set the kernels' shared-memory attributes once (outside any stream capture).
int prepare_sweep_kernels();
struct SweepMaps;
SweepMaps* create_sweep_maps(const Grid& g, const float* Pa, const float* Pb, const float* b,
                             const uint8_t* flags);
void destroy_sweep_maps(SweepMaps* m);
// The gradient subtract fused into the last launch of a solve: u, v, w (FP32, the grid's
// layout) move by the final pressure's gradient inside the launch that applies the last colour
// pass, and *sub_done is set so that the separate subtract (launch_gradient_subtract with
// skip = sub_done) does nothing.  mode 1: the launch ends the solve unless the tolerance rule
// ended it earlier (fixed sweep count, or the last launch under the sweep cap; the host knows).
// Under the tolerance rule the solve ends on the input of a check launch, which only its end
// decides, so the launch that ends it is known to nobody in time and the subtract stays a pass.
struct SweepFuse {
    float* u;
    float* v;
    float* w;
    int* sub_done;
    int mode;
};
// Whether launch_sweep_tb can fuse the subtract into a launch of this shape (full launches of
// the plain 2-row and 4-row kernels, not check launches).
bool sweep_tb_fusable(int T, int rows, int nhalf, int check);

// group_base (device, may be NULL): the launch's group index is group + *group_base (a graph's
// device-side group loop).  fuse (may be NULL, or mode 0): see SweepFuse; ignored where
// sweep_tb_fusable is false.
int launch_sweep_tb(const SweepMaps* m, const Grid& g, bool in_is_a, float* Pout, int T, int rows,
                    int nhalf, int colour0, int zchunk, const float* wacc7, StepStatus* status,
                    int check, int group, float tol, int* pcur, int out_idx, int* kerr,
                    const int* group_base, cudaStream_t st, const SweepFuse* fuse = nullptr);
// Grouped blocked solve over many grids (depth 6, 2-row patches): one record per grid (its
// tensor maps, buffers and tolerance), tiles of all grids in one launch.
size_t group_tb_record_bytes();
// Fill one record (rec: group_tb_record_bytes(), 64-byte aligned in the device copy); returns
// the grid's tile count for `zchunk`-plane chunks.
int group_tb_fill(void* rec, const SweepMaps* m, const Grid& g, float* P, float* P2, StepStatus* status, int* pcur,
                  int* kerr, const float* wacc7, float tol, int zchunk);
int launch_group_sweep_tb(const void* grids, const int* starts, int n, int total_tiles, bool in_a, int nhalf,
                          int colour0, int zchunk, int check, int group, const int* group_base, cudaStream_t st);
// Last node of a grouped solve's device-side loop body: counter += step; loop again while some
// grid's solve is not done and counter < limit; *launches += launches_per_iter (launches may be
// NULL).
void launch_group_tb_loop_next(const void* grids, int n, int* counter, int step, int limit,
                               unsigned long long* launches, int launches_per_iter,
                               cudaGraphConditionalHandle handle, cudaStream_t st);
// Last node of a device-side group loop's body: counter += step; loop again while the solve is
// not done and counter < limit; *launches += launches_per_iter.
void launch_group_loop_next(const StepStatus* status, int* counter, int step, int limit,
                            unsigned long long* launches, int launches_per_iter,
                            cudaGraphConditionalHandle handle, cudaStream_t st);
// Reference scheme, temporally blocked (kernels_vsweep_tb.cu): T colour passes of the in-place
// velocity red-black SOR per pass over HBM, bit-exact with launch_project_velocity.
// OmegaSplit: omega's sign, 53-bit significand (hi 21 / lo 32 bits) and exponent, and the range
// of biased float exponents for which float(double(q) * omega) is evaluated with integer
// arithmetic (exact_scale.cuh).
struct OmegaSplit {
    uint32_t mo_hi, mo_lo;
    int eo;
    uint32_t sign;
    int emin, emax;
};
OmegaSplit omega_split(double omega);
struct VSweepMaps;
int vsweep_depth_supported(int T);  // T = 2 or 4
int prepare_vsweep_kernels();
// Tensor maps of the state's face arrays (both ping-pong buffers), the scratch face arrays and
// the flags; all buffers must exist.  NULL on failure.
VSweepMaps* create_vsweep_maps(const Grid& g, float* const* u, float* const* v, float* const* w, const float* xu,
                               const float* xv, const float* xw, const uint8_t* flags);
void destroy_vsweep_maps(VSweepMaps* m);
// One launch: nhalf <= T colour passes starting at colour0 on the state buffer `buf`
// (from_state) or on the scratch arrays, written to (uo, vo, wo); z-chunks of zchunk planes.
int launch_vsweep_tb(const VSweepMaps* m, const Grid& g, int buf, bool from_state, float* uo, float* vo, float* wo,
                     int T, int nhalf, int colour0, int zchunk, double omega, const OmegaSplit& os, int* kerr,
                     cudaStream_t st);
void launch_div_max(const Grid& g, const float* u, const float* v, const float* w,
                    const uint8_t* flags, StepStatus* status, cudaStream_t st);
// FP64-checked refinement rounds after the projection (u, v, w: the FP32 projected velocity;
// us, vs, ws: the BF16 state to re-round, or NULL).  Adds the launches to *launches.
template <typename Tv>
void launch_refine(const Grid& g, float* u, float* v, float* w, Tv* us, Tv* vs, Tv* ws, float* b, float* P0,
                   float* P1, const int* pcur, const uint8_t* flags, const float* wacc7, int rounds,
                   int sweeps, double tol, RefineStatus* rs, long long* launches, cudaStream_t st);

// Stage a: advection.  The velocity advection reads its FP32 input planes through TMA tensor
// maps: create_advect_maps encodes n <= 2 input sets (u[k], v[k], w[k]) once the buffers exist
// (NULL on failure); a launch names the set its u0, v0, w0 are.
struct AdvectMaps;
AdvectMaps* create_advect_maps(const Grid& g, const float* const* u, const float* const* v, const float* const* w,
                               int n);
void destroy_advect_maps(AdvectMaps* m);
// The velocity advection walks the face planes 1 .. nz - 1 in chunks of
// advect_velocity_chunk_planes() planes (chunk c: planes 1 + c * that .. ); a launch advects the
// chunks [c0, c1) (c1 < 0: through the last).  The density advection's launch covers cells
// z = 1 + zz for zz in [z0, z1) (z1 < 0: through nz - 2); cell z reads the advected faces of
// planes z and z + 1.
template <typename To>
int launch_advect_velocity_tile(const AdvectMaps* m, int set, const Grid& g, const float* u0, const float* v0,
                                const float* w0, To* u1, To* v1, To* w1, const uint8_t* flags, float dt, int* kerr,
                                cudaStream_t st, int c0 = 0, int c1 = -1);
int advect_velocity_chunk_planes();
int advect_velocity_chunks(const Grid& g);
template <typename T, typename Tv>
void launch_advect_density(const Grid& g, const T* r0, T* r1, const Tv* u1, const Tv* v1, const Tv* w1,
                           const uint8_t* flags, float dt, cudaStream_t st, int z0 = 0, int z1 = -1);
// BF16 storage form: the projection written in FP32 over every face, and rounded into the state.
void launch_project_bf16(const Grid& g, __nv_bfloat16* u, __nv_bfloat16* v, __nv_bfloat16* w,
                         const float* P0, const float* P1, const int* pcur, const uint8_t* flags,
                         float* pu, float* pv, float* pw, cudaStream_t st, bool vec = true);
void launch_convert(const __nv_bfloat16* src, float* dst, size_t n, cudaStream_t st);
void launch_convert(const float* src, __nv_bfloat16* dst, size_t n, cudaStream_t st);

}  // namespace smk
