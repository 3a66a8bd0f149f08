// TEST INFRASTRUCTURE ONLY (oracle).  Host stand-in for the few CUDA runtime names that the
// reference's simulation translation unit (project/smokeSimulation.cu) uses, so that the
// reference's own step compiles with g++ and runs on the CPU.  Device memory is host memory
// (calloc, so the buffers the reference leaves uninitialised start at zero), and a kernel
// launch runs the grid's blocks in parallel with OpenMP and each block's threads one after
// another.  Every kernel of the reference writes disjoint locations within one launch (the
// projection is red-black coloured), so the result does not depend on the thread count.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define __global__
#define __device__
#define __host__

struct uint3 { unsigned int x, y, z; };
struct float3 { float x, y, z; };
struct uchar3 { unsigned char x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;

// Solver constants the recipe turns into variables (defaults = the reference's literals).
extern double ref_over_relaxation;
extern float ref_max_velocity;
extern int ref_num_iterations;

enum cudaError_t { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
};
struct cudaDeviceProp {
    int maxThreadsPerBlock;
    int maxThreadsDim[3];
    int maxGridSize[3];
    size_t sharedMemPerBlock;
};

// Allocations are rounded up to 256 bytes, the granularity cudaMalloc gives on a GPU.  The
// reference sizes its object buffers for 3 objects (smokeSimulation.cu:56, :221-229) but
// copies every registered object into them (:729, :760); on a GPU a 4th sphere still lands
// inside the 256-byte allocation, and the same holds here.
template <typename T>
inline cudaError_t cudaMalloc(T** p, size_t n) {
    size_t rounded = (n + 255) / 256 * 256;
    *p = (T*)calloc(rounded ? rounded : 256, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void* p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    if (n) memcpy(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void* d, int v, size_t n) { memset(d, v, n); return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "error"; }
inline cudaError_t cudaGetDeviceCount(int* n) { *n = 1; return cudaSuccess; }
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) {
    p->maxThreadsPerBlock = 1024;
    p->maxThreadsDim[0] = p->maxThreadsDim[1] = 1024; p->maxThreadsDim[2] = 64;
    p->maxGridSize[0] = 2147483647; p->maxGridSize[1] = p->maxGridSize[2] = 65535;
    p->sharedMemPerBlock = 49152;
    return cudaSuccess;
}

// `kernel<<<grid, block>>>(args...)` is rewritten by the recipe into this call.
template <typename K, typename... A>
inline void host_launch(dim3 grid, dim3 block, K kernel, A... args) {
    const long long nb = (long long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(static)
    for (long long bi = 0; bi < nb; ++bi) {
        blockIdx.x = (unsigned)(bi % grid.x);
        blockIdx.y = (unsigned)((bi / grid.x) % grid.y);
        blockIdx.z = (unsigned)(bi / ((long long)grid.x * grid.y));
        blockDim = block;
        for (unsigned tz = 0; tz < block.z; ++tz)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = tz;
                    kernel(args...);
                }
    }
}
