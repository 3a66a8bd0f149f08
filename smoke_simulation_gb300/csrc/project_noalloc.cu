// smk_project_noalloc: the pressure projection for callers that cannot allocate device memory.
//
// Some callers of a projection cannot call cudaMalloc when they need one: a host application
// that has handed the device's memory to its own pool allocator (a framework's caching
// allocator, a serving arena with a fixed budget) and so has nothing left for a library to
// take, or a plugin called from a per-frame or per-request callback, where cudaMalloc's implicit
// device-wide synchronisation would stall the other work on the GPU.  This entry point projects
// a caller-owned velocity field in place and takes its scratch -- the pressure, the right-hand
// side, the neighbour flags and the solver status -- from one file-scope device array of fixed
// size instead of allocating.
//
// Limits and sharing:
//   - at most NOALLOC_MAX_ELEMS = 2,097,152 face-grid elements, (nx+1)(ny+1)(nz+1) (e.g. a
//     127^3 grid), and nz <= 65535; larger grids are rejected with SMK_ERR_INVALID;
//   - the scratch array (about 19 MB) is held by every GPU that loads the library, until exit;
//   - every call shares it and finds it holding the previous call's contents: the call zeroes
//     the solver status and rewrites the flags, the right-hand side and the pressure of its
//     own grid before reading them;
//   - calls whose work overlaps on the GPU (different streams, or several host threads without
//     ordering) race on the array and corrupt each other.  Callers must order their calls on one
//     stream or synchronise between them;
//   - the first call on a device (and the first after that device's primary context was
//     replaced, e.g. by cudaDeviceReset) looks up the array's device address with
//     cudaGetSymbolAddress, with that device current; make that first call before any stream
//     capture.
// The entry point calls no cudaMalloc/cudaFree (nor any allocating library routine): only kernel
// launches, cudaMemsetAsync on the scratch, and -- when statistics are requested -- a
// synchronisation and small device-to-host copies.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
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
// per device: the scratch array's device address and the context it was looked up in
struct ScratchAddr {
    void* ptr = nullptr;
    CUcontext ctx = nullptr;
};
ScratchAddr g_scratch_dev[MAX_DEVICES];
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

// The current context (driver entry point fetched through the runtime, so the library needs
// no link against libcuda).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
CUcontext current_context() {
    static CtxGetCurrentFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrentFn>(p);
    }
    CUcontext c = nullptr;
    if (fn == nullptr || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

// Device address of the scratch array on the current device: looked up once per device and
// again when the device's context changed since (a cudaDeviceReset replaces it, and with it
// the array's address).
int scratch_for_current_device(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SMK_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return fail(SMK_ERR_INVALID, "device index out of range");
    // null when this thread has not used the device yet: the lookup below makes the device's
    // primary context current, and the context is read again after it
    const CUcontext ctx = current_context();
    std::lock_guard<std::mutex> lock(g_mutex);
    ScratchAddr& a = g_scratch_dev[dev];
    if (a.ptr == nullptr || ctx == nullptr || a.ctx != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return fail(SMK_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        a.ptr = p;
        a.ctx = current_context();
    }
    *out = static_cast<unsigned char*>(a.ptr);
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
    // widened before the additions: nx + 1 must not wrap for nx near INT_MAX
    const long long elems = ((long long)nx + 1) * ((long long)ny + 1) * ((long long)nz + 1);
    if (elems > NOALLOC_MAX_ELEMS)
        return fail(SMK_ERR_INVALID,
                    "grid too large for the no-allocation projection: (nx+1)(ny+1)(nz+1) = " +
                        std::to_string(elems) + " exceeds the fixed scratch of " +
                        std::to_string(NOALLOC_MAX_ELEMS) + " elements");
    if (nz > 65535) return fail(SMK_ERR_INVALID, "nz must be <= 65535 (one launch plane per z)");
    const smk_params& p = *params;
    const bool use_tol = p.tol > 0.0f;
    if (p.projection != SMK_PROJECT_PRESSURE || p.solver != SMK_SOLVER_RBSOR)
        return fail(SMK_ERR_INVALID, "the no-allocation projection runs the PRESSURE scheme's red-black SOR only "
                                     "(projection = SMK_PROJECT_PRESSURE, solver = SMK_SOLVER_RBSOR)");
    if (p.refine != 0) return fail(SMK_ERR_INVALID, "the no-allocation projection has no refinement rounds (refine = 0)");
    if (!std::isfinite(p.omega) || !(p.omega > 0.0) || !(p.omega < 2.0))
        return fail(SMK_ERR_INVALID, "omega must be finite and in (0, 2)");
    if (!std::isfinite(p.tol) || p.tol < 0.0f) return fail(SMK_ERR_INVALID, "tol must be finite and >= 0");
    if (p.max_sweeps < 0 || p.max_sweeps > 1000000) return fail(SMK_ERR_INVALID, "max_sweeps must be 0..1000000");
    if (use_tol && p.check_every <= 0) return fail(SMK_ERR_INVALID, "check_every must be positive when tol > 0");
    const int G = use_tol ? p.check_every : (p.max_sweeps > 0 ? p.max_sweeps : 1);
    const int ngroups = (p.max_sweeps + G - 1) / G;
    if (ngroups > NOALLOC_GROUPS) return fail(SMK_ERR_INVALID, "too many residual checks per call");

    cudaStream_t st = (cudaStream_t)stream;
    if (stats) {
        // statistics need a synchronisation of `stream`, which a stream under capture refuses
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        NA_CUDA(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(SMK_ERR_INVALID, "stats must be NULL while `stream` is being captured");
    }
    unsigned char* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    float* P = reinterpret_cast<float*>(scratch + OFF_P);
    float* b = reinterpret_cast<float*>(scratch + OFF_B);
    uint8_t* flags = scratch + OFF_F;
    smk::StepStatus* status = reinterpret_cast<smk::StepStatus*>(scratch + OFF_STATUS);

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
            const int last = hs.done ? hs.done_group : ngroups - 1;
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
