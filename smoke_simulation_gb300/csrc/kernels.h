// Host-side launchers of the step's kernels (implemented in the .cu files).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace smk {

// Stage a4: emitters and obstacles.
void launch_emit_boxes(const Grid& g, float* rho0, float* rho1, float* v_now, const BoxObj* boxes,
                       int nb, cudaStream_t st);
void launch_fill_smoke(const Grid& g, float* rho0, float* rho1, const SphereObj* sp, int ns,
                       cudaStream_t st);
void launch_fill_obstacles(const Grid& g, uint8_t* s, const ObstacleObj* ob, int no, cudaStream_t st);
// Neighbour flags from the mask; zeroes the pressure where a cell is not projectable.
void launch_build_flags(const Grid& g, const uint8_t* s, uint8_t* flags, float* P, cudaStream_t st);

// Stage b: integrate (forcing) + velocityConfinement (clamp), fused.
void launch_forcing(const Grid& g, float* u, float* v, float* w, const float* rho,
                    const uint8_t* flags, float dt, float gravity, float buoyancy, float clamp_const,
                    int clamp_mode, cudaStream_t st);

// Stage d (reference scheme): one colour pass of the in-place velocity red-black SOR.
void launch_project_velocity(const Grid& g, float* u, float* v, float* w, const uint8_t* flags,
                             int colour, double omega, cudaStream_t st);

// Stage c/d (pressure scheme).
void launch_rhs(const Grid& g, const float* u, const float* v, const float* w, const uint8_t* flags,
                float* b, float* P, const float* P2, const int* pcur, int warm, cudaStream_t st);
void launch_sweep(const Grid& g, float* P, const float* b, const uint8_t* flags, int colour,
                  const float* wacc7, const StepStatus* status, cudaStream_t st);
void launch_resid_check(const Grid& g, const float* P, const float* b, const uint8_t* flags,
                        StepStatus* status, int group, float tol, cudaStream_t st);
void launch_gradient_subtract(const Grid& g, float* u, float* v, float* w, const float* P0,
                              const float* P1, const int* pcur, const uint8_t* flags,
                              cudaStream_t st);
// Temporally blocked sweeps: nhalf <= T colour passes in one pass over HBM, P_in -> P_out;
// `check` launches also record the residual of the input state for tolerance group `group`.
// The pressure buffers are read through TMA tensor maps built once per simulation.
int sweep_tb_depth_supported(int T);
// Set the kernels' shared-memory attributes once (outside any stream capture).
int prepare_sweep_kernels();
struct SweepMaps;
SweepMaps* create_sweep_maps(const Grid& g, const float* Pa, const float* Pb, const float* b,
                             const uint8_t* flags);
void destroy_sweep_maps(SweepMaps* m);
int launch_sweep_tb(const SweepMaps* m, const Grid& g, bool in_is_a, float* Pout, int T, int nhalf,
                    int colour0, int zchunk, const float* wacc7, StepStatus* status, int check,
                    int group, float tol, int* pcur, int out_idx, int* kerr, cudaStream_t st);
void launch_div_max(const Grid& g, const float* u, const float* v, const float* w,
                    const uint8_t* flags, StepStatus* status, cudaStream_t st);

// Stage a: advection.
void launch_advect_velocity(const Grid& g, const float* u0, const float* v0, const float* w0,
                            float* u1, float* v1, float* w1, const uint8_t* flags, float dt,
                            cudaStream_t st);
void launch_advect_density(const Grid& g, const float* r0, float* r1, const float* u1,
                           const float* v1, const float* w1, const uint8_t* flags, float dt,
                           cudaStream_t st);

}  // namespace smk
