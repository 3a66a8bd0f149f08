// smk_project_noalloc: the pressure projection for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the time they need a projection: code running inside
// a CUDA graph being captured, a host that has handed the whole device memory pool to another
// allocator (a framework caching allocator, a fixed-budget serving arena), or a hook invoked
// from a context where a blocking, device-synchronising allocation is not allowed.  This entry
// point projects a caller-owned velocity field in place and takes its scratch -- the pressure,
// the right-hand side, the neighbour flags and the solver status -- from one file-scope device
// array of fixed size instead of allocating.
//
// Limits and sharing:
//   - at most NOALLOC_MAX_ELEMS = 2,097,152 face-grid elements, (nx+1)(ny+1)(nz+1) (e.g. a
//     127^3 grid); larger grids are rejected with SMK_ERR_INVALID;
//   - the scratch array (about 19 MB) is held by every GPU that loads the library, until exit;
//   - every call shares it: calls whose work overlaps on the GPU (different streams, or the same
//     array from several host threads without ordering) race and corrupt each other.  Callers
//     must order their calls on one stream or synchronise between them;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress; make that first call before any stream capture.
// The entry point calls no cudaMalloc/cudaFree (nor any allocating library routine): only kernel
// launches, cudaMemsetAsync on the scratch, and -- when statistics are requested -- a
// synchronisation and small device-to-host copies.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/smoke_gb300.h"
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr long long NOALLOC_MAX_ELEMS = 1LL << 21;
constexpr int NOALLOC_GROUPS = 4096;
constexpr long long OFF_P = 0;
constexpr long long OFF_B = OFF_P + 4 * NOALLOC_MAX_ELEMS;
constexpr long long OFF_F = OFF_B + 4 * NOALLOC_MAX_ELEMS;
constexpr long long OFF_STATUS = OFF_F + NOALLOC_MAX_ELEMS;
constexpr long long STATUS_BYTES = (long long)sizeof(smk::StepStatus) + 4LL * NOALLOC_GROUPS;
constexpr long long SCRATCH_BYTES = OFF_STATUS + STATUS_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
void* g_scratch_dev[MAX_DEVICES] = {nullptr};
thread_local std::string g_err;

// Neighbour flags from a caller's tight mask (nx*ny*nz bytes, x fastest) into the face-pitched
// grid the solver kernels use; the pressure is zeroed off the projectable set.
__global__ void k_flags_from_tight_mask(smk::Grid g, const uint8_t* __restrict__ s,
                                        uint8_t* __restrict__ flags, float* __restrict__ P) {
    const int x = blockIdx.x * 64 + threadIdx.x;
    const int y = blockIdx.y * 4 + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    const long long sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
    const long long c = x + sy * y + sz * z;
    unsigned f = s[c] ? smk::F_SELF : 0u;
    if (x > 0 && s[c - sx]) f |= smk::F_XM;
    if (x < g.nx - 1 && s[c + sx]) f |= smk::F_XP;
    if (y > 0 && s[c - sy]) f |= smk::F_YM;
    if (y < g.ny - 1 && s[c + sy]) f |= smk::F_YP;
    if (z > 0 && s[c - sz]) f |= smk::F_ZM;
    if (z < g.nz - 1 && s[c + sz]) f |= smk::F_ZP;
    const bool interior =
        x >= 1 && y >= 1 && z >= 1 && x <= g.nx - 2 && y <= g.ny - 2 && z <= g.nz - 2;
    if (interior && (f & smk::F_SELF) && (f & smk::F_NBRS)) f |= smk::F_PROJ;
    const int i = g.idx(x, y, z);
    flags[i] = (uint8_t)f;
    if (!(f & smk::F_PROJ)) P[i] = 0.0f;
}

int fail(int code, const std::string& m) {
    g_err = m;
    return code;
}

// Device address of the scratch array on the current device (looked up once per device).
int scratch_for_current_device(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SMK_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return fail(SMK_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_scratch_dev[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return fail(SMK_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_dev[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_dev[dev]);
    return SMK_OK;
}

#define NA_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) return fail(SMK_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" {

const char* smk_project_noalloc_last_error(void) { return g_err.c_str(); }

long long smk_project_noalloc_max_elems(void) { return NOALLOC_MAX_ELEMS; }

int smk_project_noalloc(float* u, float* v, float* w, const uint8_t* mask, int nx, int ny, int nz,
                        const smk_params* params, smk_stats* stats, void* stream) {
    if (!u || !v || !w || !mask || !params) return fail(SMK_ERR_INVALID, "null argument");
    if (nx < 1 || ny < 1 || nz < 1) return fail(SMK_ERR_INVALID, "grid dimensions must be >= 1");
    const long long elems = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    if (elems > NOALLOC_MAX_ELEMS)
        return fail(SMK_ERR_INVALID,
                    "grid too large for the no-allocation projection: (nx+1)(ny+1)(nz+1) = " +
                        std::to_string(elems) + " exceeds the fixed scratch of " +
                        std::to_string(NOALLOC_MAX_ELEMS) + " elements");
    const smk_params& p = *params;
    const bool use_tol = p.tol > 0.0f;
    if (p.max_sweeps < 0) return fail(SMK_ERR_INVALID, "max_sweeps must be >= 0");
    if (use_tol && p.check_every <= 0) return fail(SMK_ERR_INVALID, "check_every must be positive when tol > 0");
    const int G = use_tol ? p.check_every : (p.max_sweeps > 0 ? p.max_sweeps : 1);
    const int ngroups = (p.max_sweeps + G - 1) / G;
    if (ngroups > NOALLOC_GROUPS) return fail(SMK_ERR_INVALID, "too many residual checks per call");

    unsigned char* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    float* P = reinterpret_cast<float*>(scratch + OFF_P);
    float* b = reinterpret_cast<float*>(scratch + OFF_B);
    uint8_t* flags = scratch + OFF_F;
    smk::StepStatus* status = reinterpret_cast<smk::StepStatus*>(scratch + OFF_STATUS);
    cudaStream_t st = (cudaStream_t)stream;

    // The caller's faces use the reference layout (stride nx+1): solve on that pitch.
    smk::Grid g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.X = nx + 1;
    g.XY = (nx + 1) * (ny + 1);

    // what must start at zero: the solver status (the previous call's contents stay otherwise)
    NA_CUDA(cudaMemsetAsync(status, 0, (size_t)STATUS_BYTES, st));
    dim3 blk(64, 4), grd((unsigned)((nx + 63) / 64), (unsigned)((ny + 3) / 4), (unsigned)nz);
    k_flags_from_tight_mask<<<grd, blk, 0, st>>>(g, mask, flags, P);
    float wacc[7];
    wacc[0] = 0.0f;
    for (int a = 1; a <= 6; ++a) wacc[a] = (float)p.omega / (float)a;
    smk::launch_rhs(g, u, v, w, flags, b, P, nullptr, nullptr, 0, st);
    int sweep = 0, group = 0;
    while (sweep < p.max_sweeps) {
        if (use_tol) smk::launch_resid_check(g, P, b, flags, status, group, p.tol, st);
        const int end = sweep + G < p.max_sweeps ? sweep + G : p.max_sweeps;
        for (; sweep < end; ++sweep) {
            smk::launch_sweep(g, P, b, flags, 0, wacc, use_tol ? status : nullptr, st);
            smk::launch_sweep(g, P, b, flags, 1, wacc, use_tol ? status : nullptr, st);
        }
        ++group;
    }
    smk::launch_gradient_subtract(g, u, v, w, P, nullptr, nullptr, flags, st);
    smk::launch_div_max(g, u, v, w, flags, status, st);
    NA_CUDA(cudaGetLastError());

    if (stats) {
        NA_CUDA(cudaStreamSynchronize(st));
        smk::StepStatus hs;
        NA_CUDA(cudaMemcpy(&hs, status, sizeof(smk::StepStatus) - sizeof(unsigned), cudaMemcpyDeviceToHost));
        memset(stats, 0, sizeof(*stats));
        memcpy(&stats->div_max, &hs.div_bits, 4);
        stats->sweeps = p.max_sweeps;
        if (use_tol && ngroups > 0) {
            const int last = hs.done ? hs.done_group - 1 : ngroups - 1;
            unsigned bits = 0;
            NA_CUDA(cudaMemcpy(&bits, reinterpret_cast<const unsigned char*>(status) +
                                          offsetof(smk::StepStatus, rmax_bits) + 4 * (size_t)last,
                               4, cudaMemcpyDeviceToHost));
            memcpy(&stats->resid_max, &bits, 4);
            if (hs.done) stats->sweeps = hs.done_group * G;
            stats->converged = (hs.done || stats->resid_max <= p.tol) ? 1 : 0;
        }
    }
    return SMK_OK;
}

}  // extern "C"
