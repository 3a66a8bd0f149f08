// Shared device definitions for libsmoke_gb300.
//
// HBM layout.  Every field of one simulation -- density (cells), u, v, w (faces), pressure and
// right-hand side (cells), the solid mask and the neighbour-flag byte (cells) -- uses ONE
// index function  i = x + X*y + XY*z  with X = round_up(nx+1, 16) (64-byte float rows and
// 16-byte flag rows, as TMA tensor maps require) and
// XY = X*(ny+1).  Faces use x <= nx, y <= ny, z <= nz; cells use x < nx, y < ny, z < nz and
// leave the last row/plane unused.  One index therefore addresses a cell and its three
// "lower" faces (u at x, v at y, w at z), exactly like the reference's shared staggered index
// (project/smokeSimulation.cu:146-147, :337), while rows stay aligned for vector access.
//
// The whole library is compiled with -fmad=false so that every float expression rounds
// exactly as written (no contraction); fused multiply-adds appear only as explicit fmaf().
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace smk {

struct Grid {
    int nx, ny, nz;
    int X;   // row pitch in elements
    int XY;  // plane pitch in elements
    __host__ __device__ __forceinline__ int idx(int x, int y, int z) const { return x + X * y + XY * z; }
};

// Neighbour-flag byte per cell, derived from the mask whenever it changes.
enum : uint8_t {
    F_SELF = 1u << 0,  // s(x,y,z)
    F_XM = 1u << 1,    // s(x-1,y,z)
    F_XP = 1u << 2,    // s(x+1,y,z)
    F_YM = 1u << 3,    // s(x,y-1,z)
    F_YP = 1u << 4,    // s(x,y+1,z)
    F_ZM = 1u << 5,    // s(x,y,z-1)
    F_ZP = 1u << 6,    // s(x,y,z+1)
    F_PROJ = 1u << 7,  // updated by the projection: interior, fluid, >= 1 fluid neighbour
    F_NBRS = 0x7E,
};

// Device-side per-step status written by the solver kernels.
struct StepStatus {
    unsigned div_bits;   // max |div u| after projection, as float bits (non-negative)
    int done;            // tolerance reached: later sweep groups are skipped
    int done_group;      // the solve ended at the start of this check group (its residual <= tol)
    unsigned arrivals;   // blocks of the running check launch that have added their residual;
                         // the last one decides and resets it (check_decide)
    unsigned rmax_bits[1];  // max |residual| per check group (flexible; sized at allocation)
};

// The tolerance rule, decided at the end of the launch that records the residual of check
// group `group`: every block calls it once after its block_max_to into rmax_bits[group] (thread
// 0 of the block, which made that atomic); the last of `nblocks` to arrive reads the group's
// residual and, when it is <= tol, ends the solve there (done, done_group) and, for a launch
// that swept from one pressure buffer into the other, points *pcur back at the launch's input
// (in_idx >= 0), so that the passes it applied are dropped.  Returns whether it ended the solve.
__device__ __forceinline__ bool check_decide(StepStatus* status, int group, float tol, unsigned nblocks,
                                             int* pcur, int in_idx) {
    __threadfence();
    const unsigned prev = atomicAdd(&status->arrivals, 1u);
    if (prev + 1u != nblocks) return false;
    __threadfence();
    const float r = __uint_as_float(*(volatile unsigned*)&status->rmax_bits[group]);
    status->arrivals = 0u;
    if (!(r <= tol)) return false;
    status->done = 1;
    status->done_group = group;
    if (pcur != nullptr && in_idx >= 0) *pcur = in_idx;
    return true;
}

// Device-side state of the projection's FP64-checked refinement rounds.
struct RefineStatus {
    unsigned long long div_bits;  // max |div u| of the last measurement (FP64, as IEEE bits)
    int need;                     // the last measurement found a cell above tolerance
    int rounds;                   // correction rounds applied in this step
    int stop;                     // a measurement was within tolerance: later rounds do nothing
    int pad;
};

// Object records (the reference's packing, smokeSimulation.cu:719-725, :750-758).
struct SphereObj { float x, y, z, r; };
struct ObstacleObj { float x, y, z, vx, vy, vz, r; };
struct BoxObj { int x0, y0, z0, x1, y1, z1; float density, vy; int set_vy; };

__device__ __forceinline__ void atomic_max_bits(unsigned* p, float nonneg) {
    atomicMax(p, __float_as_uint(nonneg));
}

// Max-reduce `v` (bit patterns of non-negative floats: the IEEE order, NaN largest) over the
// block, then one atomicMax per block, skipped when the stored value is already larger.  One
// atomic per warp on a single address serialises at L2 and costs ~1 ms on a 256^3 grid.
// Every thread of the block must call it; it ends with a block barrier, so a persistent loop
// may call it again without racing on the shared scratch.
__device__ __forceinline__ void block_max_to(unsigned v, unsigned* dst) {
    __shared__ unsigned red[32];
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5, nwarps = (nthreads + 31) >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < nwarps ? red[lane] : 0u;
        for (int o = 16; o > 0; o >>= 1) w = max(w, __shfl_xor_sync(0xffffffffu, w, o));
        if (lane == 0 && w > *(volatile unsigned*)dst) atomicMax(dst, w);
    }
    __syncthreads();
}

// ---- storage types ----------------------------------------------------------------------------
// Fields are stored as float (FP32 form) or bf16 (BF16 storage form); arithmetic is FP32 in
// both.  ldv/stv are the only places a stored value is converted.
__device__ __forceinline__ float ldv(const float* __restrict__ p, int i) { return p[i]; }
__device__ __forceinline__ float ldv(const __nv_bfloat16* __restrict__ p, int i) { return __bfloat162float(p[i]); }
__device__ __forceinline__ void stv(float* __restrict__ p, int i, float v) { p[i] = v; }
__device__ __forceinline__ void stv(__nv_bfloat16* __restrict__ p, int i, float v) { p[i] = __float2bfloat16_rn(v); }

// Four consecutive stored values (index a multiple of 4 in a row with 16-byte aligned float or
// 8-byte aligned bf16 rows): one vector load, the raw bits kept so that a store can leave the
// lanes that did not change bit for bit as they were.  A bf16 value widens to float exactly by
// its bits (the conversion ldv makes).
struct Raw4f { float4 v; };
struct Raw4h { uint2 r; };
__device__ __forceinline__ Raw4f ld4raw(const float* p) { return Raw4f{*reinterpret_cast<const float4*>(p)}; }
__device__ __forceinline__ Raw4h ld4raw(const __nv_bfloat16* p) { return Raw4h{*reinterpret_cast<const uint2*>(p)}; }
__device__ __forceinline__ float4 to4(const Raw4f& a) { return a.v; }
__device__ __forceinline__ float4 to4(const Raw4h& a) {
    return make_float4(__uint_as_float(a.r.x << 16), __uint_as_float(a.r.x & 0xffff0000u),
                       __uint_as_float(a.r.y << 16), __uint_as_float(a.r.y & 0xffff0000u));
}
// Store the four values; lane c keeps its raw bits unless bit c of `changed` is set (a float lane
// that did not change holds its loaded value, so storing it is the same).
__device__ __forceinline__ void st4(float* p, const Raw4f&, float4 v, unsigned) {
    *reinterpret_cast<float4*>(p) = v;
}
__device__ __forceinline__ unsigned bf16_bits(float v) {
    return (unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(v));
}
__device__ __forceinline__ void st4(__nv_bfloat16* p, const Raw4h& a, float4 v, unsigned changed) {
    const unsigned h0 = (changed & 1u) ? bf16_bits(v.x) : (a.r.x & 0xffffu);
    const unsigned h1 = (changed & 2u) ? bf16_bits(v.y) : (a.r.x >> 16);
    const unsigned h2 = (changed & 4u) ? bf16_bits(v.z) : (a.r.y & 0xffffu);
    const unsigned h3 = (changed & 8u) ? bf16_bits(v.w) : (a.r.y >> 16);
    *reinterpret_cast<uint2*>(p) = make_uint2(h0 | (h1 << 16), h2 | (h3 << 16));
}
template <typename T> struct Raw4;
template <> struct Raw4<float> { typedef Raw4f type; };
template <> struct Raw4<__nv_bfloat16> { typedef Raw4h type; };

// ---- reference-exact helpers ---------------------------------------------------------------

// avgU/avgV/avgW (smokeSimulation.cu:409-447): 8-point sums in the reference's order, / 8.
template <typename T>
__device__ __forceinline__ float avgU(const T* __restrict__ f, const Grid& g, int i) {
    const int X = g.X, XY = g.XY;
    float s = ldv(f, i - XY) + ldv(f, i + 1 - XY) + ldv(f, i - X - XY) + ldv(f, i + 1 - X - XY) + ldv(f, i) +
              ldv(f, i + 1) + ldv(f, i - X) + ldv(f, i + 1 - X);
    return s / 8.0f;
}
template <typename T>
__device__ __forceinline__ float avgV(const T* __restrict__ f, const Grid& g, int i) {
    const int X = g.X, XY = g.XY;
    float s = ldv(f, i - XY) + ldv(f, i - 1 - XY) + ldv(f, i + X - XY) + ldv(f, i - 1 + X - XY) + ldv(f, i) +
              ldv(f, i - 1) + ldv(f, i + X) + ldv(f, i - 1 + X);
    return s / 8.0f;
}
template <typename T>
__device__ __forceinline__ float avgW(const T* __restrict__ f, const Grid& g, int i) {
    const int X = g.X, XY = g.XY;
    float s = ldv(f, i) + ldv(f, i - 1) + ldv(f, i - X) + ldv(f, i - 1 - X) + ldv(f, i - XY) + ldv(f, i - 1 - XY) +
              ldv(f, i - X - XY) + ldv(f, i - 1 - X - XY);
    return s / 8.0f;
}

// The eight weighted corner terms of sampleSmoke (smokeSimulation.cu:474-482), summed in the
// reference's order.
__device__ __forceinline__ float trilinear_ref(float xw0, float xw1, float yw0, float yw1, float zw0, float zw1,
                                               float a000, float a100, float a010, float a110, float a001,
                                               float a101, float a011, float a111) {
    return xw0 * yw0 * zw0 * a000 + xw1 * yw0 * zw0 * a100 + xw0 * yw1 * zw0 * a010 +
           xw1 * yw1 * zw0 * a110 + xw0 * yw0 * zw1 * a001 + xw1 * yw0 * zw1 * a101 +
           xw0 * yw1 * zw1 * a011 + xw1 * yw1 * zw1 * a111;
}

// sampleSmoke (smokeSimulation.cu:451-484): clamp the position to [1, n-1] with the CELL
// dims, trilinear weights from (c - delta) - i0, eight terms summed in the reference's order.
// HX, HY, HZ: delta = 0.5 on that axis (1) or 0 (0); every call site has n >= 2 on every axis
// (it samples only from cells with an interior neighbour).  After the clamp c lies in [1, n-1],
// so c - delta >= 0.5 and floorf equals truncation, and the reference's fminf(i0, n-1) never
// changes i0.  Its upper corner fminf(i0 + 1, n - 1): with delta = 0.5, c - delta <= n - 1.5,
// so i0 <= n - 2 and the corner is always i0 + 1; with delta = 0 it is i0 + 1 unless i0 = n - 1
// (a position clamped to the last cell), where it repeats i0.  Integer index arithmetic with
// these facts gives every result of the reference's float index arithmetic.
template <int HX, int HY, int HZ, typename T>
__device__ __forceinline__ float sample_ref(const T* __restrict__ f, const Grid& g, float px,
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
    // The upper corner is +1 on each axis except where a delta-0 axis was clamped to the last
    // cell (then it repeats the lower one).  Every +1 neighbour lies inside the arrays (rows
    // hold >= nx+1 elements, planes >= ny+1 rows, the field >= nz+1 planes), so the x+1 values
    // are loaded at a fixed offset and replaced by the x0 values where the corner repeats: the
    // eight loads need four row addresses, not eight index computations.
    const int sy = (HY || y0 < ly) ? g.X : 0;
    const int sz = (HZ || z0 < lz) ? g.XY : 0;
    const T* r00 = f + (x0 + y0 * g.X + z0 * g.XY);
    const T* r10 = r00 + sy;
    const T* r01 = r00 + sz;
    const T* r11 = r01 + sy;
    const float a000 = ldv(r00, 0), a010 = ldv(r10, 0), a001 = ldv(r01, 0), a011 = ldv(r11, 0);
    const float b100 = ldv(r00, 1), b110 = ldv(r10, 1), b101 = ldv(r01, 1), b111 = ldv(r11, 1);
    const bool sx = HX || x0 < lx;
    const float a100 = sx ? b100 : a000, a110 = sx ? b110 : a010, a101 = sx ? b101 : a001,
                a111 = sx ? b111 : a011;
    return trilinear_ref(xw0, xw1, yw0, yw1, zw0, zw1, a000, a100, a010, a110, a001, a101, a011, a111);
}

// Loads issued where they stand (volatile inline PTX): the compiler can neither sink them into
// the conditional block that consumes them nor merge them away, so a warp has a cell's loads in
// flight before it waits on the flag byte that decides whether the cell is updated.
__device__ __forceinline__ float ld_eager(const float* p) {
    float v;
    asm volatile("ld.global.f32 %0, [%1];" : "=f"(v) : "l"(__cvta_generic_to_global(p)));
    return v;
}
__device__ __forceinline__ float ld_eager(const __nv_bfloat16* p) {
    unsigned short h;
    asm volatile("ld.global.u16 %0, [%1];" : "=h"(h) : "l"(__cvta_generic_to_global(p)));
    return __bfloat162float(__ushort_as_bfloat16(h));
}

}  // namespace smk
