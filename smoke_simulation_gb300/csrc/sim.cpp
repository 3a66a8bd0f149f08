// libsmoke_gb300: handle management and the step driver behind the C ABI (smoke_gb300.h).
//
// Replaces the reference's module globals and host orchestration
// (project/smokeSimulation.cu:16-248, :707-819) with an explicit handle.  A step issues the
// reference's stage sequence (simulate, :774-811) on one CUDA stream without host
// synchronisation; only smk_simulate (the reference's simulate with its blocking D2H, :814)
// and the explicit read/stat calls synchronise.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/smoke_gb300.h"
#include "kernels.h"
#include "sim_internal.h"

using namespace smk;

namespace {

thread_local std::string g_last_error;

// A stored field as BF16 (the allocation is 2 bytes per element in the BF16 storage form).
inline __nv_bfloat16* bf(float* p) { return reinterpret_cast<__nv_bfloat16*>(p); }

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int check_params(const smk_params* p) {
    if (!p) return fail(SMK_ERR_INVALID, "params is null");
    if (p->projection != SMK_PROJECT_REFERENCE && p->projection != SMK_PROJECT_PRESSURE)
        return fail(SMK_ERR_INVALID, "unknown projection scheme");
    if (p->clamp_mode < 0 || p->clamp_mode > 2) return fail(SMK_ERR_INVALID, "unknown clamp mode");
    if (p->max_sweeps < 0 || p->max_sweeps > 1000000) return fail(SMK_ERR_INVALID, "max_sweeps out of range");
    if (p->projection == SMK_PROJECT_PRESSURE && p->tol > 0 && p->check_every <= 0)
        return fail(SMK_ERR_INVALID, "check_every must be positive when tol > 0");
    if (p->storage != SMK_STORAGE_F32 && p->storage != SMK_STORAGE_BF16 && p->storage != SMK_STORAGE_BF16_VEL)
        return fail(SMK_ERR_INVALID, "unknown storage precision");
    if (p->storage != SMK_STORAGE_F32 && p->projection == SMK_PROJECT_REFERENCE)
        return fail(SMK_ERR_INVALID, "BF16 storage needs the pressure projection");
    if (p->refine < 0 || p->refine > 16) return fail(SMK_ERR_INVALID, "refine must be 0..16");
    if (p->refine > 0 && (p->projection != SMK_PROJECT_PRESSURE || !(p->tol > 0.0f)))
        return fail(SMK_ERR_INVALID, "refinement needs the PRESSURE projection with tol > 0");
    if (p->refine > 0 && (p->refine_sweeps < 1 || p->refine_sweeps > 100000))
        return fail(SMK_ERR_INVALID, "refine_sweeps must be 1..100000");
    if (p->solver != SMK_SOLVER_RBSOR && p->solver != SMK_SOLVER_JACOBI) return fail(SMK_ERR_INVALID, "unknown solver");
    if (!std::isfinite(p->omega_warm) || p->omega_warm < 0.0 || p->omega_warm >= 2.0)
        return fail(SMK_ERR_INVALID, "omega_warm must be 0 (off) or in (0, 2)");
    if (p->omega_warm_after < 0) return fail(SMK_ERR_INVALID, "omega_warm_after must be >= 0");
    if (!std::isfinite(p->warm_extrapolate) || p->warm_extrapolate < 0.0f || p->warm_extrapolate > 1.0f)
        return fail(SMK_ERR_INVALID, "warm_extrapolate must be in 0..1");
    if (p->solver == SMK_SOLVER_JACOBI && p->projection != SMK_PROJECT_PRESSURE)
        return fail(SMK_ERR_INVALID, "the Jacobi solver needs the PRESSURE projection");
    if (p->projection == SMK_PROJECT_PRESSURE && p->tol > 0 &&
        (p->max_sweeps + p->check_every - 1) / p->check_every > 4000)
        return fail(SMK_ERR_INVALID, "too many residual checks per step (max_sweeps/check_every > 4000)");
    return SMK_OK;
}

// z-chunk of the blocked velocity sweep when none was chosen: about four CTAs' worth of planes
// per SM-wave of x-y tiles, at least 2T + 8 planes so the chunk's halo stays a minor part.
int default_vsweep_zchunk(const Grid& g, int T) {
    const int rows = T == 2 ? 24 : 32;
    const int tiles = ((g.nx + 1 + 63 - 2 * T) / (64 - 2 * T)) * ((g.ny + 1 + rows - 1 - 2 * T) / (rows - 2 * T));
    const int planes = g.nz + 1;
    int chunks = (4 * 152 + tiles - 1) / (tiles > 0 ? tiles : 1);
    if (chunks < 1) chunks = 1;
    int zc = (planes + chunks - 1) / chunks;
    if (zc < 2 * T + 8) zc = 2 * T + 8;
    return zc;
}

cudaMemcpy3DParms copy3d(void* dst, size_t dpitch, size_t dy, const void* src, size_t spitch,
                         size_t sy, size_t width_bytes, size_t h, size_t d, cudaMemcpyKind kind) {
    cudaMemcpy3DParms m;
    memset(&m, 0, sizeof(m));
    m.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), spitch, width_bytes, sy);
    m.dstPtr = make_cudaPitchedPtr(dst, dpitch, width_bytes, dy);
    m.extent = make_cudaExtent(width_bytes, h, d);
    m.kind = kind;
    return m;
}

}  // namespace

int smk_fail(int code, const std::string& msg) { return fail(code, msg); }

// Fault injection for tests: the next N smk_create calls fail as a device allocation failure
// would, before touching the device.
static std::atomic<int> g_inject_alloc_failures{0};

// ---- smk_sim --------------------------------------------------------------------------------

int smk_sim::enable_pressure_history() {
    if (!Ph) {
        SMK_CUDA(cudaMalloc((void**)&Ph, elems() * sizeof(float)));
        SMK_CUDA(cudaMemset(Ph, 0, elems() * sizeof(float)));
    }
    ph_from = steps;  // saved from the next step on
    return SMK_OK;
}

int smk_sim::alloc() {
    const size_t n = elems();
    bf16 = p.storage == SMK_STORAGE_BF16 || p.storage == SMK_STORAGE_BF16_VEL;
    rho_bf16 = p.storage == SMK_STORAGE_BF16;
    // advected fields: 4 bytes (FP32) or 2 bytes (BF16 storage) per element; the solver's
    // pressure and right-hand side are FP32 in every form
    float** vfields[] = {&u[0], &u[1], &v[0], &v[1], &w[0], &w[1]};
    for (float** f : vfields) {
        SMK_CUDA(cudaMalloc((void**)f, n * (bf16 ? 2 : 4)));
        SMK_CUDA(cudaMemset(*f, 0, n * (bf16 ? 2 : 4)));
    }
    float** rfields[] = {&rho[0], &rho[1]};
    for (float** f : rfields) {
        SMK_CUDA(cudaMalloc((void**)f, n * (rho_bf16 ? 2 : 4)));
        SMK_CUDA(cudaMemset(*f, 0, n * (rho_bf16 ? 2 : 4)));
    }
    float** fl[] = {&P, &P2, &b};
    for (float** f : fl) {
        SMK_CUDA(cudaMalloc((void**)f, n * sizeof(float)));
        SMK_CUDA(cudaMemset(*f, 0, n * sizeof(float)));
    }
    if (p.warm_extrapolate > 0.0f) {
        const int rc = enable_pressure_history();
        if (rc) return rc;
    }
    if (bf16) {
        // FP32 projected velocity (what advection consumes); scratch for conversions between steps
        float** pr[] = {&proj[0], &proj[1], &proj[2]};
        for (float** f : pr) {
            SMK_CUDA(cudaMalloc((void**)f, n * sizeof(float)));
            SMK_CUDA(cudaMemset(*f, 0, n * sizeof(float)));
        }
    }
    SMK_CUDA(cudaMalloc((void**)&pcur, 4 * sizeof(int)));
    SMK_CUDA(cudaMemset(pcur, 0, 4 * sizeof(int)));
    kerr = pcur + 1;
    SMK_CUDA(cudaHostAlloc((void**)&kerr_host, sizeof(int), cudaHostAllocDefault));
    *kerr_host = 0;
    gcount = pcur + 2;
    SMK_CUDA(cudaMalloc((void**)&loop_launches, sizeof(unsigned long long)));
    SMK_CUDA(cudaMemset(loop_launches, 0, sizeof(unsigned long long)));
    SMK_CUDA(cudaMalloc((void**)&refine, sizeof(RefineStatus)));
    SMK_CUDA(cudaMemset(refine, 0, sizeof(RefineStatus)));
    SMK_CUDA(cudaMalloc((void**)&s, n));
    SMK_CUDA(cudaMalloc((void**)&flags, n));
    SMK_CUDA(cudaMemset(flags, 0, n));
    // the tensor maps capture the buffer addresses: every buffer must exist first
    maps = create_sweep_maps(g, P, P2, b, flags);
    if (!maps) return fail(SMK_ERR_CUDA, "could not encode the TMA tensor maps of the sweep kernel");
    if (!bf16) {
        vmaps = create_vsweep_maps(g, u, v, w, P, P2, b, flags);
        if (!vmaps) return fail(SMK_ERR_CUDA, "could not encode the TMA tensor maps of the velocity sweep kernel");
        const float* au[2] = {u[0], u[1]};
        const float* av[2] = {v[0], v[1]};
        const float* aw[2] = {w[0], w[1]};
        amaps = create_advect_maps(g, au, av, aw, 2);
    } else {
        // the BF16 forms advect from the FP32 copy of the projected faces
        const float* au[1] = {proj[0]};
        const float* av[1] = {proj[1]};
        const float* aw[1] = {proj[2]};
        amaps = create_advect_maps(g, au, av, aw, 1);
    }
    if (!amaps) return fail(SMK_ERR_CUDA, "could not encode the TMA tensor maps of the velocity advection");
    status_groups = 4096;
    SMK_CUDA(cudaMalloc((void**)&status, sizeof(StepStatus) + sizeof(unsigned) * status_groups));
    SMK_CUDA(cudaMemset(status, 0, sizeof(StepStatus) + sizeof(unsigned) * status_groups));
    SMK_CUDA(cudaMalloc((void**)&tune_status, sizeof(StepStatus) + sizeof(unsigned)));
    for (auto& e : ev) SMK_CUDA(cudaEventCreate(&e));
    SMK_CUDA(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    SMK_CUDA(cudaStreamCreateWithFlags(&body_stream, cudaStreamNonBlocking));
    SMK_CUDA(cudaStreamCreateWithFlags(&rb_stream, cudaStreamNonBlocking));
    SMK_CUDA(cudaEventCreateWithFlags(&rb_fork, cudaEventDisableTiming));
    SMK_CUDA(cudaEventCreateWithFlags(&rb_join, cudaEventDisableTiming));
    if (prepare_sweep_kernels() != 0 || prepare_vsweep_kernels() != 0)
        return fail(SMK_ERR_CUDA, "sweep kernel configuration failed");
    // initializeVolume's mask: fluid except the y = 0 floor (smokeSimulation.cu:200-207)
    std::vector<uint8_t> host((size_t)g.nx * g.ny * g.nz, 1);
    for (int z = 0; z < g.nz; ++z)
        for (int x = 0; x < g.nx; ++x) host[(size_t)x + (size_t)z * g.nx * g.ny] = 0;
    return upload_mask(host.data());
}

void smk_sim::release() {
    float* fl[] = {rho[0], rho[1], u[0], u[1], v[0], v[1], w[0], w[1], P, P2, b, proj[0], proj[1], proj[2], Ph};
    for (float* f : fl)
        if (f) cudaFree(f);
    if (pcur) cudaFree(pcur);
    if (kerr_host) cudaFreeHost(kerr_host);
    if (loop_launches) cudaFree(loop_launches);
    if (refine) cudaFree(refine);
    if (render_scratch) cudaFree(render_scratch);
    if (maps) destroy_sweep_maps(maps);
    if (vmaps) destroy_vsweep_maps(vmaps);
    if (amaps) destroy_advect_maps(amaps);
    if (s) cudaFree(s);
    if (flags) cudaFree(flags);
    if (status) cudaFree(status);
    if (tune_status) cudaFree(tune_status);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    for (auto& gs : graphs)
        if (gs.exec) cudaGraphExecDestroy(gs.exec);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (body_stream) cudaStreamDestroy(body_stream);
    if (rb_stream) cudaStreamDestroy(rb_stream);
    if (rb_fork) cudaEventDestroy(rb_fork);
    if (rb_join) cudaEventDestroy(rb_join);
}

int smk_sim::upload_mask(const uint8_t* host) {
    std::vector<uint8_t> norm((size_t)g.nx * g.ny * g.nz);
    for (size_t i = 0; i < norm.size(); ++i) norm[i] = host[i] ? 1 : 0;
    auto m = copy3d(s, g.X, g.ny + 1, norm.data(), g.nx, g.ny, g.nx, g.ny, g.nz, cudaMemcpyHostToDevice);
    SMK_CUDA(cudaMemcpy3D(&m));
    mask_dirty = true;
    return SMK_OK;
}

int smk_sim::enqueue(float dt, cudaStream_t st) {
    const int past = index_now;
    const int now = index_now ^ 1;
    index_now = now;
    const bool timed = timing;
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    SMK_CUDA(cudaStreamIsCapturing(st, &cap_status));
    const bool capturing = cap_status == cudaStreamCaptureStatusActive;
    // stage-timing events; inside a capture they become event-record nodes of the graph
    auto rec = [&](cudaEvent_t e) {
        return cudaEventRecordWithFlags(e, st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    };
    if (timed) SMK_CUDA(rec(ev[0]));

    // a4: objects (drawObjects, smokeSimulation.cu:714-771)
    std::vector<BoxObj> boxes;
    std::vector<SphereObj> spheres;
    std::vector<ObstacleObj> obstacles;
    for (const auto& o : objects) {
        if (o.kind == OBJ_BOX) boxes.push_back(o.box);
        else if (o.kind == OBJ_SPHERE) spheres.push_back(o.sphere);
        else obstacles.push_back(o.obstacle);
    }
    if (!boxes.empty()) {
        if (rho_bf16) launch_emit_boxes(g, bf(rho[0]), bf(rho[1]), bf(v[now]), boxes.data(), (int)boxes.size(), st);
        else if (bf16) launch_emit_boxes(g, rho[0], rho[1], bf(v[now]), boxes.data(), (int)boxes.size(), st);
        else launch_emit_boxes(g, rho[0], rho[1], v[now], boxes.data(), (int)boxes.size(), st);
        ++launches;
    }
    if (!spheres.empty()) {
        if (rho_bf16) launch_fill_smoke(g, bf(rho[0]), bf(rho[1]), spheres.data(), (int)spheres.size(), st);
        else launch_fill_smoke(g, rho[0], rho[1], spheres.data(), (int)spheres.size(), st);
        ++launches;
    }
    if (!obstacles.empty() && (obstacles_dirty || mask_dirty)) {
        launch_fill_obstacles(g, s, obstacles.data(), (int)obstacles.size(), st);
        ++launches;
        mask_dirty = true;
    }
    obstacles_dirty = false;
    if (mask_dirty) {
        launch_build_flags(g, s, flags, st);
        ++launches;
        mask_dirty = false;
    }
    if (timed) SMK_CUDA(rec(ev[1]));

    // b: integrate + velocityConfinement (:789-791)
    if (rho_bf16)
        launch_forcing(g, bf(u[now]), bf(v[now]), bf(w[now]), (const __nv_bfloat16*)bf(rho[now]), flags, dt,
                       p.gravity, p.buoyancy, p.clamp_const, p.clamp_mode, st, vec_stages);
    else if (bf16)
        launch_forcing(g, bf(u[now]), bf(v[now]), bf(w[now]), (const float*)rho[now], flags, dt, p.gravity,
                       p.buoyancy, p.clamp_const, p.clamp_mode, st, vec_stages);
    else
        launch_forcing(g, u[now], v[now], w[now], (const float*)rho[now], flags, dt, p.gravity, p.buoyancy,
                       p.clamp_const, p.clamp_mode, st, vec_stages);
    ++launches;
    if (p.obstacle_velocity && !obstacles.empty()) {
        if (bf16) launch_obstacle_velocity(g, bf(u[now]), bf(v[now]), bf(w[now]), obstacles.back(), st);
        else launch_obstacle_velocity(g, u[now], v[now], w[now], obstacles.back(), st);
        ++launches;
    }
    if (timed) SMK_CUDA(rec(ev[2]));

    // c/d: projection (:795-801)
    const size_t status_bytes = sizeof(StepStatus) + sizeof(unsigned) * status_groups;
    SMK_CUDA(cudaMemsetAsync(status, 0, status_bytes, st));
    last_groups = 0;
    if (p.projection == SMK_PROJECT_REFERENCE) {
        if (vsweep_depth > 0 && vmaps != nullptr && p.max_sweeps > 0) {
            // temporally blocked: launches of up to T colour passes alternating between the state
            // (u, v, w)[now] and the scratch arrays (P, P2, b), an even number of them so that the
            // result ends in the state; the passes are those of the loop below, in the same order
            const int T = vsweep_depth;
            const int H = 2 * p.max_sweeps;
            std::vector<int> plan;
            for (int h = 0; h < H; h += T) plan.push_back(H - h < T ? H - h : T);
            if (plan.size() % 2 == 1) {  // split one launch in two (both keep >= 1 pass)
                if (plan.back() >= 2) {
                    plan.back() -= 1;
                    plan.push_back(1);
                } else {
                    plan[plan.size() - 2] -= 1;
                    plan.push_back(1);
                }
            }
            const OmegaSplit os = omega_split(p.omega);
            const int zc = vsweep_zchunk > 0 ? vsweep_zchunk : default_vsweep_zchunk(g, T);
            int h = 0;
            for (size_t l = 0; l < plan.size(); ++l) {
                const bool from_state = (l % 2) == 0;
                float* uo = from_state ? P : u[now];
                float* vo = from_state ? P2 : v[now];
                float* wo = from_state ? b : w[now];
                if (launch_vsweep_tb(vmaps, g, now, from_state, uo, vo, wo, T, plan[l], h & 1, zc, p.omega, os, kerr,
                                     st) != 0)
                    return fail(SMK_ERR_CUDA, "velocity sweep kernel launch failed");
                h += plan[l];
                ++launches;
            }
            pressure_clobbered = true;
        } else {
            for (int it = 0; it < p.max_sweeps; ++it) {
                launch_project_velocity(g, u[now], v[now], w[now], flags, 0, p.omega, st);
                launch_project_velocity(g, u[now], v[now], w[now], flags, 1, p.omega, st);
                launches += 2;
            }
        }
    } else {
        float wacc[7];
        wacc[0] = 0.0f;
        const double om = pressure_omega();  // omega, or omega_warm once the history is long enough
        for (int a = 1; a <= 6; ++a) wacc[a] = (float)om / (float)a;
        // the extrapolated warm start (smk_params.warm_extrapolate): the rhs pass saves the last
        // pressure into Ph and starts the solve from its extrapolation
        float* ph = keeps_history() ? Ph : nullptr;
        const float alpha = extrapolation();
        if (bf16)
            launch_rhs(g, (const __nv_bfloat16*)bf(u[now]), (const __nv_bfloat16*)bf(v[now]),
                       (const __nv_bfloat16*)bf(w[now]), flags, b, P, P2, pcur, p.warm_start, st, vec_stages, ph,
                       alpha);
        else
            launch_rhs(g, (const float*)u[now], (const float*)v[now], (const float*)w[now], flags, b, P, P2,
                       pcur, p.warm_start, st, vec_stages, ph, alpha);
        ++launches;
        const bool use_tol = p.tol > 0.0f;
        const int G = use_tol ? p.check_every : (p.max_sweeps > 0 ? p.max_sweeps : 1);
        int sweep = 0, group = 0;
        bool subtract_fused = false;  // a blocked launch that certainly runs applied the subtract
        if (timed) SMK_CUDA(rec(ev[5]));
        if (p.solver == SMK_SOLVER_JACOBI) {
            // weighted Jacobi, ping-ponging P <-> P2 (each launch records in *pcur where it wrote);
            // the check of each group reads the buffer holding the current iterate
            int nl = 0;
            while (sweep < p.max_sweeps) {
                if (use_tol) {
                    launch_resid_check(g, (nl & 1) ? P2 : P, b, flags, status, group, p.tol, st);
                    ++launches;
                }
                const int end = sweep + G < p.max_sweeps ? sweep + G : p.max_sweeps;
                for (; sweep < end; ++sweep, ++nl) {
                    const bool from_a = (nl & 1) == 0;
                    launch_jacobi(g, from_a ? P : P2, from_a ? P2 : P, b, flags, wacc, use_tol ? status : nullptr,
                                  pcur, from_a ? 1 : 0, st);
                    ++launches;
                }
                ++group;
            }
        } else if (sweep_depth > 0) {
            // temporally blocked: each launch applies up to sweep_depth colour passes,
            // ping-ponging P <-> P2; group starts are the check launches, and a launch of fewer
            // passes comes first in its group, so that the group ends with a full launch
            int nl = 0;
            // With smk_set_fused_subtract, the gradient subtract is fused into the solve's last
            // launch where the host knows it (FP32 state; no tolerance, or the last launch under
            // the sweep cap, when the tolerance rule has not ended the solve before it)
            int* sub_done = reinterpret_cast<int*>(&status->rmax_bits[status_groups]);
            const bool fusable = fuse_subtract && !bf16 && p.max_sweeps > 0;
            bool fused_known = false;  // a launch that certainly runs ends the solve fused
            // at_cap: the group ends at the sweep cap (unrolled groups only)
            auto issue_group = [&](int grp, int s0, int s1, const int* gbase, cudaStream_t s, bool at_cap) -> int {
                const int h0 = 2 * s0, h1 = 2 * s1;
                const int first = (h1 - h0) % sweep_depth;
                for (int h = h0; h < h1;) {
                    const int nh = (h == h0 && first != 0) ? first : sweep_depth;
                    const bool in_a = (nl & 1) == 0;
                    const bool chk = use_tol && h == h0;
                    const bool last = h + nh == h1;
                    const bool fz_on = fusable && last && (!use_tol || at_cap) &&
                                       sweep_tb_fusable(sweep_depth, sweep_rows, nh, chk);
                    fused_known = fused_known || (fz_on && !use_tol);
                    const SweepFuse fz{u[now], v[now], w[now], sub_done, 1};
                    if (launch_sweep_tb(maps, g, in_a, in_a ? P2 : P, sweep_depth, sweep_rows, nh, h & 1, sweep_zchunk,
                                        wacc, use_tol ? status : nullptr, chk, grp, p.tol, pcur, in_a ? 1 : 0, kerr,
                                        gbase, s, fz_on ? &fz : nullptr) != 0)
                        return fail(SMK_ERR_CUDA, "sweep kernel configuration failed");
                    ++launches;
                    ++nl;
                    h += nh;
                }
                return SMK_OK;
            };
            // In a captured step, the full groups run as a WHILE loop on the device: the body is
            // one group (two when a group has an odd number of launches, so that every
            // iteration starts from the same pressure buffer), the loop stops when the tolerance
            // rule declares the solve done or the full groups are used up.  The launches and
            // their order are those of the unrolled sequence minus the ones that would exit at
            // entry, so results are identical.
            const int nlg = (2 * G + sweep_depth - 1) / sweep_depth;
            const int U = (nlg % 2 == 0) ? 1 : 2;
            // with the subtract fused, the group at the cap stays out of the loop: its last launch
            // is then issued knowing that it ends the solve (if the tolerance rule has not)
            const int full = use_tol ? p.max_sweeps / G - (fusable && p.max_sweeps % G == 0 ? 1 : 0) : 0;
            const int loop_groups = (capturing && graph_loops && use_tol) ? (full / U) * U : 0;
            if (loop_groups > U) {
                SMK_CUDA(cudaMemsetAsync(gcount, 0, sizeof(int), st));
                cudaStreamCaptureStatus cs;
                cudaGraph_t cg = nullptr;
                const cudaGraphNode_t* deps = nullptr;
                size_t ndeps = 0;
                SMK_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
                cudaGraphConditionalHandle handle;
                SMK_CUDA(cudaGraphConditionalHandleCreate(&handle, cg, 1, cudaGraphCondAssignDefault));
                cudaGraphNodeParams np = {};
                np.type = cudaGraphNodeTypeConditional;
                np.conditional.handle = handle;
                np.conditional.type = cudaGraphCondTypeWhile;
                np.conditional.size = 1;
                cudaGraphNode_t node;
                SMK_CUDA(cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &np));
                cudaGraph_t body = np.conditional.phGraph_out[0];
                SMK_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
                SMK_CUDA(cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0,
                                                       cudaStreamCaptureModeThreadLocal));
                const int nl0 = nl;
                const long long l0 = launches;
                int rc = SMK_OK;
                for (int u = 0; u < U && rc == SMK_OK; ++u) rc = issue_group(u, u * G, (u + 1) * G, gcount, body_stream, false);
                const int per_iter = (int)(launches - l0) + 1;
                if (rc == SMK_OK)
                    launch_group_loop_next(status, gcount, U, loop_groups, loop_launches, per_iter, handle, body_stream);
                cudaGraph_t bg = nullptr;
                const cudaError_t ee = cudaStreamEndCapture(body_stream, &bg);
                if (rc != SMK_OK) return rc;
                if (ee != cudaSuccess) return fail(SMK_ERR_CUDA, std::string("group loop capture: ") + cudaGetErrorString(ee));
                // the body's launches are counted on the device, per executed iteration
                launches = l0;
                nl = nl0;  // U * nlg is even: the parity after each iteration is the same
                sweep = loop_groups * G;
                group = loop_groups;
            }
            while (sweep < p.max_sweeps) {
                const int end = sweep + G < p.max_sweeps ? sweep + G : p.max_sweeps;
                const int rc = issue_group(group, sweep, end, nullptr, st, end == p.max_sweeps);
                if (rc != SMK_OK) return rc;
                sweep = end;
                ++group;
            }
            subtract_fused = fused_known;
        } else {
            while (sweep < p.max_sweeps) {
                if (use_tol) {
                    launch_resid_check(g, P, b, flags, status, group, p.tol, st);
                    ++launches;
                }
                int end = sweep + G < p.max_sweeps ? sweep + G : p.max_sweeps;
                for (; sweep < end; ++sweep) {
                    launch_sweep(g, P, b, flags, 0, wacc, use_tol ? status : nullptr, st);
                    launch_sweep(g, P, b, flags, 1, wacc, use_tol ? status : nullptr, st);
                    launches += 2;
                }
                ++group;
            }
        }
        last_groups = group;
        if (timed) SMK_CUDA(rec(ev[6]));
        // the blocked and Jacobi solves record where the pressure is; the colour passes keep it in P
        const bool pcur_set = (sweep_depth > 0 || p.solver == SMK_SOLVER_JACOBI) && p.max_sweeps > 0;
        if (!pcur_set) SMK_CUDA(cudaMemsetAsync(pcur, 0, sizeof(int), st));
        if (bf16) {
            launch_project_bf16(g, bf(u[now]), bf(v[now]), bf(w[now]), P, P2, pcur, flags, proj[0], proj[1],
                                proj[2], st, vec_stages);
            ++launches;
        } else if (!subtract_fused) {
            // skipped at run time when a blocked launch applied it (SweepFuse)
            launch_gradient_subtract(g, u[now], v[now], w[now], P, P2, pcur, flags, st, vec_stages,
                                     reinterpret_cast<const int*>(&status->rmax_bits[status_groups]));
            ++launches;
        }
        if (p.refine > 0) {
            if (bf16)
                launch_refine(g, proj[0], proj[1], proj[2], bf(u[now]), bf(v[now]), bf(w[now]), b, P, P2, pcur,
                              flags, wacc, p.refine, p.refine_sweeps, (double)p.tol, refine, &launches, st);
            else
                launch_refine(g, u[now], v[now], w[now], (float*)nullptr, (float*)nullptr, (float*)nullptr, b, P,
                              P2, pcur, flags, wacc, p.refine, p.refine_sweeps, (double)p.tol, refine,
                              &launches, st);
        }
    }
    // the projected velocity advection consumes: the state itself (FP32) or its FP32 copy
    const float* pu = bf16 ? proj[0] : u[now];
    const float* pv = bf16 ? proj[1] : v[now];
    const float* pw = bf16 ? proj[2] : w[now];
    if (p.report_div) {
        launch_div_max(g, pu, pv, pw, flags, status, st);
        ++launches;
    }
    if (timed) SMK_CUDA(rec(ev[3]));

    // a: advection (:805-810).  With a host readback (rb_host) it runs in z-slabs: slab s
    // advects velocity chunks [c0, c1), then the density cells whose faces those chunks
    // finished (cell z reads the faces of planes z and z + 1), and its density planes go to the
    // host on rb_stream while the next slab computes.  Every cell's arithmetic is the same.
    const int chunks = advect_velocity_chunks(g), chunk_planes = advect_velocity_chunk_planes();
    const int nslab = rb_host ? std::max(1, std::min(readback_slabs(), chunks)) : 1;
    int zz_done = 0, plane_done = 0;
    for (int sl = 0; sl < nslab; ++sl) {
        const bool last_slab = sl == nslab - 1;
        const int c0 = (int)((long long)chunks * sl / nslab);
        const int c1 = last_slab ? -1 : (int)((long long)chunks * (sl + 1) / nslab);
        const int zz1 = last_slab ? -1 : c1 * chunk_planes - 1;  // density cells 1 .. zz1 are ready
        if (bf16) {
            if (launch_advect_velocity_tile(amaps, 0, g, pu, pv, pw, bf(u[past]), bf(v[past]), bf(w[past]), flags,
                                            dt, kerr, st, c0, c1) != 0)
                return fail(SMK_ERR_CUDA, "velocity advection launch failed");
            if (rho_bf16)
                launch_advect_density(g, (const __nv_bfloat16*)bf(rho[now]), bf(rho[past]),
                                      (const __nv_bfloat16*)bf(u[past]), (const __nv_bfloat16*)bf(v[past]),
                                      (const __nv_bfloat16*)bf(w[past]), flags, dt, st, zz_done, zz1);
            else
                launch_advect_density(g, (const float*)rho[now], rho[past], (const __nv_bfloat16*)bf(u[past]),
                                      (const __nv_bfloat16*)bf(v[past]), (const __nv_bfloat16*)bf(w[past]),
                                      flags, dt, st, zz_done, zz1);
        } else {
            if (launch_advect_velocity_tile(amaps, now, g, pu, pv, pw, u[past], v[past], w[past], flags, dt, kerr, st,
                                            c0, c1) != 0)
                return fail(SMK_ERR_CUDA, "velocity advection launch failed");
            launch_advect_density(g, (const float*)rho[now], rho[past], (const float*)u[past],
                                  (const float*)v[past], (const float*)w[past], flags, dt, st, zz_done, zz1);
        }
        launches += 2;
        if (rb_host) {
            // planes [plane_done, p1) of the density are final: the boundary planes z = 0 and
            // z = nz - 1 are not written by the advection
            const int p1 = last_slab ? g.nz : zz1 + 1;
            SMK_CUDA(cudaEventRecord(rb_fork, st));
            SMK_CUDA(cudaStreamWaitEvent(rb_stream, rb_fork, 0));
            auto m = copy3d(rb_host + (size_t)plane_done * g.nx * g.ny, (size_t)g.nx * 4, g.ny,
                            rho[past] + (size_t)plane_done * g.XY, (size_t)g.X * 4, g.ny + 1, (size_t)g.nx * 4, g.ny,
                            p1 - plane_done, cudaMemcpyDeviceToHost);
            SMK_CUDA(cudaMemcpy3DAsync(&m, rb_stream));
            plane_done = p1;
        }
        zz_done = zz1;
    }
    if (rb_host) {
        SMK_CUDA(cudaEventRecord(rb_join, rb_stream));
        SMK_CUDA(cudaStreamWaitEvent(st, rb_join, 0));
    }
    if (timed) SMK_CUDA(rec(ev[4]));
    SMK_CUDA(cudaGetLastError());
    ++steps;
    ++hist_steps;
    last_projection = p.projection;
    last_tol = p.tol;
    last_max_sweeps = p.max_sweeps;
    last_check_every = p.check_every;
    last_refine = p.projection == SMK_PROJECT_PRESSURE ? p.refine : 0;
    return SMK_OK;
}

int smk_sim::prepare_mask(cudaStream_t st) {
    int n = 0;
    std::vector<ObstacleObj> obstacles;
    for (const auto& o : objects)
        if (o.kind == OBJ_OBSTACLE) obstacles.push_back(o.obstacle);
    if (!obstacles.empty() && (obstacles_dirty || mask_dirty)) {
        launch_fill_obstacles(g, s, obstacles.data(), (int)obstacles.size(), st);
        ++n;
        mask_dirty = true;
    }
    obstacles_dirty = false;
    if (mask_dirty) {
        launch_build_flags(g, s, flags, st);
        ++n;
        mask_dirty = false;
    }
    launches += n;
    return n;
}

// Everything the step's kernels bake in as launch parameters: a captured graph is reused only
// while all of it is unchanged.
std::string smk_sim::graph_signature(float dt) const {
    std::string sig;
    auto put = [&sig](const void* p, size_t n) { sig.append(static_cast<const char*>(p), n); };
    put(&dt, sizeof(dt));
    put(&p, sizeof(p));
    const double om = pressure_omega();  // the over-relaxation this step's solve uses
    put(&om, sizeof(om));
    const float ea = extrapolation();  // and its warm start's extrapolation (a launch parameter)
    const char kh = keeps_history() ? 1 : 0;
    put(&ea, sizeof(ea));
    put(&kh, 1);
    put(&sweep_depth, sizeof(sweep_depth));
    put(&sweep_zchunk, sizeof(sweep_zchunk));
    put(&sweep_rows, sizeof(sweep_rows));
    put(&vsweep_depth, sizeof(vsweep_depth));
    put(&vsweep_zchunk, sizeof(vsweep_zchunk));
    const char t = timing ? 1 : 0;
    put(&t, 1);
    put(&rb_host, sizeof(rb_host));  // the host readback's copies are nodes of the graph
    const int nrb = rb_host ? readback_slabs() : 0;
    put(&nrb, sizeof(nrb));
    for (const Object& o : objects) put(&o, sizeof(o));
    return sig;
}

// One step.  Steady state replays a CUDA graph of the whole step (captured on an internal
// stream, launched on the caller's): one launch call instead of ~100 for a 256^3 step with the
// tolerance-driven solve, and the GPU runs the kernels back to back.  A step whose mask or
// obstacles changed runs directly (it includes the one-off mask kernels), and so does a step
// with stage timing on (events recorded inside a capture cannot be queried afterwards).
int smk_sim::step(float dt, cudaStream_t st) {
    if (pressure_clobbered && p.projection == SMK_PROJECT_PRESSURE) {
        // the blocked velocity sweep of earlier REFERENCE steps left its scratch in P, P2, b: the
        // pressure history starts over, as after smk_write_state
        SMK_CUDA(cudaMemsetAsync(P, 0, elems() * sizeof(float), st));
        SMK_CUDA(cudaMemsetAsync(P2, 0, elems() * sizeof(float), st));
        SMK_CUDA(cudaMemsetAsync(pcur, 0, sizeof(int), st));
        pressure_clobbered = false;
        hist_steps = 0;
    }
    if (!use_graphs || mask_dirty || obstacles_dirty) return enqueue(dt, st);
    GraphSlot& gs = graphs[index_now];
    std::string sig = graph_signature(dt);
    if (gs.exec == nullptr || gs.sig != sig) {
        const int idx0 = index_now, steps0 = steps;
        const long long hist0 = hist_steps;
        const long long l0 = launches;
        SMK_CUDA(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue(dt, cap_stream);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(cap_stream, &graph);
        if (rc != SMK_OK) {
            if (graph) cudaGraphDestroy(graph);
            index_now = idx0;
            steps = steps0;
            hist_steps = hist0;
            launches = l0;
            return rc;
        }
        if (ce != cudaSuccess) return fail(SMK_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(ce));
        gs.launches = launches - l0;
        gs.groups = last_groups;
        index_now = idx0;
        steps = steps0;
        hist_steps = hist0;
        launches = l0;
        if (gs.exec) cudaGraphExecDestroy(gs.exec);
        gs.exec = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&gs.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return fail(SMK_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        gs.sig.swap(sig);
    }
    SMK_CUDA(cudaGraphLaunch(gs.exec, st));
    index_now ^= 1;
    launches += gs.launches;
    ++steps;
    ++hist_steps;
    last_groups = gs.groups;
    last_projection = p.projection;
    last_tol = p.tol;
    last_max_sweeps = p.max_sweeps;
    last_check_every = p.check_every;
    last_refine = p.projection == SMK_PROJECT_PRESSURE ? p.refine : 0;
    return SMK_OK;
}

// ---- C ABI ----------------------------------------------------------------------------------

// After a synchronisation: report (and clear) a bounded device wait that gave up.
int check_kernel_error(smk_sim* sim) {
    int e = 0;
    SMK_CUDA(cudaMemcpy(&e, sim->kerr, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        SMK_CUDA(cudaMemset(sim->kerr, 0, sizeof(int)));
        return fail(SMK_ERR_TIMEOUT, "a bounded device wait (TMA loads or a grid barrier) gave up; "
                                     "the step's projection is incomplete");
    }
    return SMK_OK;
}

extern "C" {

void smk_default_params(smk_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->gravity = -9.82f;
    p->buoyancy = 2.0f;
    p->clamp_const = 3.0f;
    p->clamp_mode = SMK_CLAMP_REFERENCE;
    p->projection = SMK_PROJECT_REFERENCE;
    p->max_sweeps = 30;
    p->omega = 1.9;
    p->tol = 0.0f;
    p->check_every = 10;
    p->warm_start = 0;
    p->report_div = 0;
    p->storage = SMK_STORAGE_F32;
    p->refine = 0;
    p->refine_sweeps = 10;
    p->omega_warm = 0.0;
    p->omega_warm_after = 2;
    p->warm_extrapolate = 0.0f;
}

const char* smk_error_string(int code) {
    switch (code) {
        case SMK_OK: return "ok";
        case SMK_ERR_INVALID: return "invalid argument";
        case SMK_ERR_CUDA: return "CUDA error";
        case SMK_ERR_OOM: return "out of device memory";
        case SMK_ERR_STATE: return "invalid state";
        case SMK_ERR_TIMEOUT: return "device wait timed out";
        default: return "unknown error";
    }
}

const char* smk_last_error(void) { return g_last_error.c_str(); }

int smk_create(int nx, int ny, int nz, const smk_params* params, smk_sim** out) {
    if (!out) return fail(SMK_ERR_INVALID, "out is null");
    *out = nullptr;
    if (nx < 1 || ny < 1 || nz < 1) return fail(SMK_ERR_INVALID, "grid dimensions must be >= 1");
    smk_params p;
    if (params) p = *params; else smk_default_params(&p);
    int rc = check_params(&p);
    if (rc) return rc;
    long long X = ((long long)nx + 1 + 15) / 16 * 16;  // 16-element rows: TMA strides
    long long total = X * (ny + 1) * (long long)(nz + 1);
    if (total >= (1LL << 31)) return fail(SMK_ERR_INVALID, "grid too large for 32-bit indexing");
    for (int k = g_inject_alloc_failures.load(); k > 0; k = g_inject_alloc_failures.load())
        if (g_inject_alloc_failures.compare_exchange_weak(k, k - 1))
            return fail(SMK_ERR_OOM, "injected device allocation failure");
    smk_sim* sim = new smk_sim();
    sim->g.nx = nx;
    sim->g.ny = ny;
    sim->g.nz = nz;
    sim->g.X = (int)X;
    sim->g.XY = (int)(X * (ny + 1));
    sim->p = p;
    cudaGetDevice(&sim->device);
    rc = sim->alloc();
    if (rc) {
        sim->release();
        delete sim;
        return rc;
    }
    *out = sim;
    return SMK_OK;
}

int smk_destroy(smk_sim* sim) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    DeviceGuard dg(sim->device);
    cudaDeviceSynchronize();
    sim->release();
    delete sim;
    return SMK_OK;
}

int smk_set_params(smk_sim* sim, const smk_params* params) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    int rc = check_params(params);
    if (rc) return rc;
    if (params->storage != sim->p.storage)
        return fail(SMK_ERR_INVALID, "the storage precision is fixed when the simulation is created");
    const bool was = sim->p.warm_extrapolate > 0.0f;
    sim->p = *params;
    if (params->warm_extrapolate > 0.0f && !was) {
        DeviceGuard dg(sim->device);
        rc = sim->enable_pressure_history();
        if (rc) return rc;
    }
    return SMK_OK;
}

// FP32 view of a stored field for a device-to-host/device copy: the field itself, or (BF16
// storage) its conversion into the projection scratch buffer, stream-ordered on `st`.
static const float* fp32_source(smk_sim* sim, const float* field, bool is_bf16, cudaStream_t st) {
    if (!is_bf16) return field;
    launch_convert(reinterpret_cast<const __nv_bfloat16*>(field), sim->proj[0], sim->elems(), st);
    return sim->proj[0];
}
// Where a host-to-device copy of a field lands (the field, or the scratch for BF16), and the
// conversion that completes it.
static float* fp32_target(smk_sim* sim, float* field, bool is_bf16) { return is_bf16 ? sim->proj[0] : field; }
static void fp32_commit(smk_sim* sim, float* field, bool is_bf16, cudaStream_t st) {
    if (is_bf16) launch_convert(sim->proj[0], reinterpret_cast<__nv_bfloat16*>(field), sim->elems(), st);
}

int smk_get_params(const smk_sim* sim, smk_params* params) {
    if (!sim || !params) return fail(SMK_ERR_INVALID, "null argument");
    *params = sim->p;
    return SMK_OK;
}

int smk_get_dims(const smk_sim* sim, int* nx, int* ny, int* nz) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    if (nx) *nx = sim->g.nx;
    if (ny) *ny = sim->g.ny;
    if (nz) *nz = sim->g.nz;
    return SMK_OK;
}

int smk_set_density(smk_sim* sim, const float* host_rho) {
    if (!sim || !host_rho) return fail(SMK_ERR_INVALID, "null argument");
    DeviceGuard dg(sim->device);
    const Grid& g = sim->g;
    if (sim->rho_bf16) SMK_CUDA(cudaMemset(sim->proj[0], 0, sim->elems() * sizeof(float)));
    auto m = copy3d(fp32_target(sim, sim->rho[0], sim->rho_bf16), (size_t)g.X * 4, g.ny + 1, host_rho, (size_t)g.nx * 4, g.ny,
                    (size_t)g.nx * 4, g.ny, g.nz, cudaMemcpyHostToDevice);
    SMK_CUDA(cudaMemcpy3D(&m));
    fp32_commit(sim, sim->rho[0], sim->rho_bf16, nullptr);
    SMK_CUDA(cudaDeviceSynchronize());
    return SMK_OK;
}

int smk_set_solid_mask(smk_sim* sim, const uint8_t* host_s) {
    if (!sim || !host_s) return fail(SMK_ERR_INVALID, "null argument");
    DeviceGuard dg(sim->device);
    return sim->upload_mask(host_s);
}

static int add_object(smk_sim* sim, const smk_sim::Object& o, int* id) {
    sim->objects.push_back(o);
    if (id) *id = (int)sim->objects.size() - 1;
    return SMK_OK;
}

int smk_add_obstacle(smk_sim* sim, float x, float y, float z, float vx, float vy, float vz, float r,
                     int* id) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    smk_sim::Object o{};
    o.kind = smk_sim::OBJ_OBSTACLE;
    o.obstacle = ObstacleObj{x, y, z, vx, vy, vz, r};
    sim->obstacles_dirty = true;
    return add_object(sim, o, id);
}

int smk_add_smoke_source(smk_sim* sim, float x, float y, float z, float r, int* id) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    smk_sim::Object o{};
    o.kind = smk_sim::OBJ_SPHERE;
    o.sphere = SphereObj{x, y, z, r};
    return add_object(sim, o, id);
}

int smk_add_box_emitter(smk_sim* sim, int x0, int y0, int z0, int x1, int y1, int z1, float density,
                        float vy, int set_vy, int* id) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    smk_sim::Object o{};
    o.kind = smk_sim::OBJ_BOX;
    o.box = BoxObj{x0, y0, z0, x1, y1, z1, density, vy, set_vy ? 1 : 0};
    return add_object(sim, o, id);
}

int smk_update_object_pos(smk_sim* sim, int id, float x, float y, float z) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    if (id < 0 || id >= (int)sim->objects.size()) return fail(SMK_ERR_INVALID, "object id out of range");
    auto& o = sim->objects[id];
    if (o.kind == smk_sim::OBJ_SPHERE) {
        o.sphere.x = x; o.sphere.y = y; o.sphere.z = z;
    } else if (o.kind == smk_sim::OBJ_OBSTACLE) {
        o.obstacle.x = x; o.obstacle.y = y; o.obstacle.z = z;
        sim->obstacles_dirty = true;
    } else {
        int dx = (int)x - o.box.x0, dy = (int)y - o.box.y0, dz = (int)z - o.box.z0;
        o.box.x0 += dx; o.box.x1 += dx; o.box.y0 += dy; o.box.y1 += dy; o.box.z0 += dz; o.box.z1 += dz;
    }
    return SMK_OK;
}

int smk_clear_objects(smk_sim* sim) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    sim->objects.clear();
    sim->obstacles_dirty = true;
    return SMK_OK;
}

int smk_step(smk_sim* sim, float dt, void* stream) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    DeviceGuard dg(sim->device);
    return sim->step(dt, (cudaStream_t)stream);
}

int smk_read_density(smk_sim* sim, float* dst, int dst_on_device, void* stream) {
    if (!sim || !dst) return fail(SMK_ERR_INVALID, "null argument");
    DeviceGuard dg(sim->device);
    const Grid& g = sim->g;
    const float* src = fp32_source(sim, sim->rho[sim->index_now ^ 1], sim->rho_bf16, (cudaStream_t)stream);
    auto m = copy3d(dst, (size_t)g.nx * 4, g.ny, src, (size_t)g.X * 4, g.ny + 1, (size_t)g.nx * 4, g.ny,
                    g.nz, dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost);
    SMK_CUDA(cudaMemcpy3DAsync(&m, (cudaStream_t)stream));
    return SMK_OK;
}

int smk_sync(smk_sim* sim, void* stream) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    DeviceGuard dg(sim->device);
    SMK_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return check_kernel_error(sim);
}

// Both ends of [p, p + bytes) lie in page-locked (registered or cudaHostAlloc) host memory.
static bool pinned_host_range(const void* p, size_t bytes) {
    const char* ends[2] = {static_cast<const char*>(p), static_cast<const char*>(p) + bytes - 1};
    for (const char* q : ends) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost) return false;
    }
    return true;
}

int smk_simulate(smk_sim* sim, float* host_out, float dt) {
    if (!sim || !host_out) return fail(SMK_ERR_INVALID, "null argument");
    DeviceGuard dg(sim->device);
    const size_t bytes = (size_t)sim->g.nx * sim->g.ny * sim->g.nz * sizeof(float);
    if (sim->readback_slabs() > 0 && !sim->rho_bf16 && pinned_host_range(host_out, bytes)) {
        // the density is copied out slab by slab inside the step (smk_set_readback_slabs)
        sim->rb_host = host_out;
        const int rc = sim->step(dt, (cudaStream_t)0);
        sim->rb_host = nullptr;
        if (rc) return rc;
    } else {
        int rc = sim->step(dt, (cudaStream_t)0);
        if (rc) return rc;
        rc = smk_read_density(sim, host_out, 0, nullptr);
        if (rc) return rc;
    }
    // the error word travels with the step's copies: one synchronisation for both
    SMK_CUDA(cudaMemcpyAsync(sim->kerr_host, sim->kerr, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)0));
    SMK_CUDA(cudaStreamSynchronize((cudaStream_t)0));
    return *sim->kerr_host ? check_kernel_error(sim) : SMK_OK;
}

int smk_set_readback_slabs(smk_sim* sim, int slabs) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    if (slabs < -1 || slabs > 64) return fail(SMK_ERR_INVALID, "slabs must be in -1..64");
    sim->rb_slabs = slabs;
    return SMK_OK;
}

int smk_get_readback_slabs(const smk_sim* sim, int* slabs) {
    if (!sim || !slabs) return fail(SMK_ERR_INVALID, "null argument");
    *slabs = sim->readback_slabs();
    return SMK_OK;
}

static int state_copy(smk_sim* sim, const smk_host_state* st, bool to_device) {
    if (!sim || !st) return fail(SMK_ERR_INVALID, "null argument");
    DeviceGuard dg(sim->device);
    const Grid& g = sim->g;
    SMK_CUDA(cudaDeviceSynchronize());
    for (int k = 0; k < 2; ++k) {
        float* dev_c[1] = {sim->rho[k]};
        float* host_c[1] = {st->rho[k]};
        float* dev_f[3] = {sim->u[k], sim->v[k], sim->w[k]};
        float* host_f[3] = {st->u[k], st->v[k], st->w[k]};
        for (int j = 0; j < 1; ++j) {
            if (!host_c[j]) continue;
            if (to_device && sim->rho_bf16) SMK_CUDA(cudaMemset(sim->proj[0], 0, sim->elems() * sizeof(float)));
            cudaMemcpy3DParms m =
                to_device ? copy3d(fp32_target(sim, dev_c[j], sim->rho_bf16), (size_t)g.X * 4, g.ny + 1,
                                   host_c[j], (size_t)g.nx * 4, g.ny, (size_t)g.nx * 4, g.ny, g.nz,
                                   cudaMemcpyHostToDevice)
                          : copy3d(host_c[j], (size_t)g.nx * 4, g.ny,
                                   fp32_source(sim, dev_c[j], sim->rho_bf16, nullptr),
                                   (size_t)g.X * 4, g.ny + 1, (size_t)g.nx * 4, g.ny, g.nz,
                                   cudaMemcpyDeviceToHost);
            SMK_CUDA(cudaMemcpy3D(&m));
            if (to_device) fp32_commit(sim, dev_c[j], sim->rho_bf16, nullptr);
        }
        for (int j = 0; j < 3; ++j) {
            if (!host_f[j]) continue;
            size_t wb = (size_t)(g.nx + 1) * 4;
            if (to_device && sim->bf16) SMK_CUDA(cudaMemset(sim->proj[0], 0, sim->elems() * sizeof(float)));
            cudaMemcpy3DParms m =
                to_device ? copy3d(fp32_target(sim, dev_f[j], sim->bf16), (size_t)g.X * 4, g.ny + 1, host_f[j],
                                   wb, g.ny + 1, wb, g.ny + 1, g.nz + 1, cudaMemcpyHostToDevice)
                          : copy3d(host_f[j], wb, g.ny + 1, fp32_source(sim, dev_f[j], sim->bf16, nullptr),
                                   (size_t)g.X * 4, g.ny + 1, wb, g.ny + 1, g.nz + 1, cudaMemcpyDeviceToHost);
            SMK_CUDA(cudaMemcpy3D(&m));
            if (to_device) fp32_commit(sim, dev_f[j], sim->bf16, nullptr);
        }
        SMK_CUDA(cudaDeviceSynchronize());
    }
    if (st->s) {
        if (to_device) {
            int rc = sim->upload_mask(st->s);
            if (rc) return rc;
        } else {
            auto m = copy3d(st->s, g.nx, g.ny, sim->s, g.X, g.ny + 1, g.nx, g.ny, g.nz,
                            cudaMemcpyDeviceToHost);
            SMK_CUDA(cudaMemcpy3D(&m));
        }
    }
    return SMK_OK;
}

int smk_read_state(smk_sim* sim, const smk_host_state* st) {
    int rc = state_copy(sim, st, false);
    if (rc == SMK_OK) const_cast<smk_host_state*>(st)->index_now = sim->index_now;
    return rc;
}

int smk_write_state(smk_sim* sim, const smk_host_state* st) {
    if (st && st->index_now != 0 && st->index_now != 1)
        return fail(SMK_ERR_INVALID, "index_now must be 0 or 1");
    int rc = state_copy(sim, st, true);
    if (rc != SMK_OK) return rc;
    sim->index_now = st->index_now;
    // the solver's pressure history belongs to the old state: a warm-started step after a
    // write starts from zero, as the first step of a new simulation does
    SMK_CUDA(cudaMemset(sim->P, 0, sim->elems() * sizeof(float)));
    SMK_CUDA(cudaMemset(sim->P2, 0, sim->elems() * sizeof(float)));
    SMK_CUDA(cudaMemset(sim->pcur, 0, sizeof(int)));
    SMK_CUDA(cudaDeviceSynchronize());
    sim->hist_steps = 0;
    return SMK_OK;
}

int smk_get_stats(smk_sim* sim, smk_stats* out) {
    if (!sim || !out) return fail(SMK_ERR_INVALID, "null argument");
    DeviceGuard dg(sim->device);
    memset(out, 0, sizeof(*out));
    out->step_index = sim->steps;
    out->div_max = -1.0f;
    out->div64_max = -1.0f;
    if (sim->steps == 0) return SMK_OK;
    // the header words, the group residuals, and the fused-subtract word after them
    std::vector<unsigned> host(5 + sim->status_groups);
    SMK_CUDA(cudaDeviceSynchronize());
    int krc = check_kernel_error(sim);
    if (krc) return krc;
    SMK_CUDA(cudaMemcpy(host.data(), sim->status, sizeof(StepStatus) + sizeof(unsigned) * sim->status_groups,
                        cudaMemcpyDeviceToHost));
    out->subtract_fused = host[4 + sim->status_groups] != 0u ? 1 : 0;
    StepStatus hs;
    memcpy(&hs, host.data(), sizeof(StepStatus) - sizeof(unsigned));
    const unsigned* rmax = host.data() + 4;
    if (sim->p.report_div) {
        float d;
        memcpy(&d, &hs.div_bits, 4);
        out->div_max = d;
    }
    if (sim->last_projection == SMK_PROJECT_REFERENCE) {
        out->sweeps = sim->last_max_sweeps;
    } else if (sim->last_tol > 0) {
        int ng = sim->last_groups;
        int G = sim->last_check_every;
        if (hs.done) {
            out->sweeps = hs.done_group * G;
            out->converged = 1;
            memcpy(&out->resid_max, &rmax[hs.done_group], 4);
        } else {
            out->sweeps = sim->last_max_sweeps;
            float r = 0;
            if (ng > 0) memcpy(&r, &rmax[ng - 1], 4);
            out->resid_max = r;
            out->converged = (ng > 0 && r <= sim->last_tol) ? 1 : 0;
        }
    } else {
        out->sweeps = sim->last_max_sweeps;
    }
    if (sim->last_refine > 0) {
        RefineStatus rs;
        SMK_CUDA(cudaMemcpy(&rs, sim->refine, sizeof(rs), cudaMemcpyDeviceToHost));
        double d;
        memcpy(&d, &rs.div_bits, sizeof(d));
        out->div64_max = (float)d;
        out->refine_rounds = rs.rounds;
    }
    return SMK_OK;
}

int smk_set_timing(smk_sim* sim, int enable) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    sim->timing = enable != 0;
    return SMK_OK;
}

int smk_get_stage_times(smk_sim* sim, float* ms, int count) {
    if (!sim || !ms) return fail(SMK_ERR_INVALID, "null argument");
    if (!sim->timing || sim->steps == 0) return fail(SMK_ERR_STATE, "timing not enabled or no step taken");
    DeviceGuard dg(sim->device);
    SMK_CUDA(cudaEventSynchronize(sim->ev[4]));
    float t[6];
    for (int k = 0; k < 4; ++k) SMK_CUDA(cudaEventElapsedTime(&t[k], sim->ev[k], sim->ev[k + 1]));
    SMK_CUDA(cudaEventElapsedTime(&t[4], sim->ev[0], sim->ev[4]));
    t[5] = 0.0f;
    if (sim->last_projection == SMK_PROJECT_PRESSURE)
        SMK_CUDA(cudaEventElapsedTime(&t[5], sim->ev[5], sim->ev[6]));
    for (int k = 0; k < count && k < 6; ++k) ms[k] = t[k];
    return SMK_OK;
}

int smk_inject_alloc_failures(int count) {
    if (count < 0) return fail(SMK_ERR_INVALID, "count must be >= 0");
    g_inject_alloc_failures.store(count);
    return SMK_OK;
}

long long smk_launch_count(const smk_sim* sim) {
    if (!sim) return 0;
    // plus the launches of device-side group loops (counted on the device; reading synchronises)
    unsigned long long dev = 0;
    if (sim->loop_launches) {
        DeviceGuard dg(sim->device);
        if (cudaMemcpy(&dev, sim->loop_launches, sizeof(dev), cudaMemcpyDeviceToHost) != cudaSuccess) dev = 0;
    }
    return sim->launches + (long long)dev;
}

}  // extern "C"

extern "C" {

int smk_set_sweep_shape(smk_sim* sim, int depth, int rows, int zchunk) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    if (depth != 0 && !sweep_tb_shape_supported(depth, rows))
        return fail(SMK_ERR_INVALID, "sweep shape must be depth 0, depth 2/4/6 with 2 rows, depth 4 with 4 rows, "
                                     "or depth 6 with 2 rows | SMK_SWEEP_YCLUSTER [| SMK_SWEEP_YCLUSTER_N(2 or 4)]");
    if (depth != 0 && (rows & SWEEP_YCLUSTER)) {
        DeviceGuard dg(sim->device);
        if (sweep_ycluster_usable(sim->g, sweep_ycluster_n(rows)) < 1)
            return fail(SMK_ERR_INVALID, "the y-cluster sweep needs co-resident clusters (and ny <= 256 when one "
                                         "cluster spans y)");
    }
    if (zchunk < 1) return fail(SMK_ERR_INVALID, "zchunk must be >= 1");
    sim->sweep_depth = depth;
    sim->sweep_rows = depth != 0 ? rows : 2;
    sim->sweep_zchunk = zchunk;
    return SMK_OK;
}

int smk_set_velocity_sweep(smk_sim* sim, int depth, int zchunk) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    if (depth != 0 && !vsweep_depth_supported(depth))
        return fail(SMK_ERR_INVALID, "velocity sweep depth must be 0 (one colour pass per launch), 2 or 4");
    if (zchunk < 0) return fail(SMK_ERR_INVALID, "zchunk must be >= 0 (0: chosen from the grid)");
    if (depth != 0 && sim->vmaps == nullptr)
        return fail(SMK_ERR_INVALID, "the blocked velocity sweep needs FP32 storage");
    sim->vsweep_depth = depth;
    sim->vsweep_zchunk = zchunk;
    return SMK_OK;
}

int smk_get_velocity_sweep(const smk_sim* sim, int* depth, int* zchunk) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    const int d = sim->vmaps ? sim->vsweep_depth : 0;
    if (depth) *depth = d;
    if (zchunk) *zchunk = d == 0 ? 0 : (sim->vsweep_zchunk > 0 ? sim->vsweep_zchunk : default_vsweep_zchunk(sim->g, d));
    return SMK_OK;
}

int smk_set_sweep_kernel(smk_sim* sim, int depth, int zchunk) {
    return smk_set_sweep_shape(sim, depth, 2, zchunk);
}

int smk_set_graphs(smk_sim* sim, int enable) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    sim->use_graphs = enable != 0;
    return SMK_OK;
}

int smk_set_vector_stages(smk_sim* sim, int enable) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    sim->vec_stages = enable != 0;
    for (auto& gs : sim->graphs) gs.sig.clear();  // re-capture
    return SMK_OK;
}

int smk_set_fused_subtract(smk_sim* sim, int enable) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    sim->fuse_subtract = enable != 0;
    for (auto& gs : sim->graphs) gs.sig.clear();  // re-capture
    return SMK_OK;
}

int smk_set_graph_loops(smk_sim* sim, int enable) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    sim->graph_loops = enable != 0;
    for (auto& gs : sim->graphs) gs.sig.clear();  // re-capture
    return SMK_OK;
}

int smk_get_sweep_kernel(const smk_sim* sim, int* depth, int* zchunk) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    if (depth) *depth = sim->sweep_depth;
    if (zchunk) *zchunk = sim->sweep_zchunk;
    return SMK_OK;
}

int smk_get_sweep_shape(const smk_sim* sim, int* depth, int* rows, int* zchunk) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    if (depth) *depth = sim->sweep_depth;
    if (rows) *rows = sim->sweep_rows;
    if (zchunk) *zchunk = sim->sweep_zchunk;
    return SMK_OK;
}

}  // extern "C"

// ---- autotuner ------------------------------------------------------------------------------
//
// The blocked sweep kernel has two free parameters: the depth T (colour passes per HBM pass)
// and the z-chunk (planes per CTA).  Larger T moves fewer bytes per sweep but recomputes a
// wider halo; the z-chunk trades the pipeline's start-up planes against wave quantisation on
// the SM count.  Candidates are chunks with no unroll padding ((chunk + 2T + 1) a multiple of
// the ring length T + 4); each is timed on the simulation's own buffers with CUDA events and
// the fastest is kept.  Results are cached per grid shape for the process.  Tuning reads P, b
// and the flags and writes only the second pressure buffer, after moving a live pressure out
// of it, so the simulation's results do not depend on whether or when tuning ran.

#include <map>
#include <mutex>
#include <tuple>

namespace {
std::mutex g_tune_mutex;
// key: device, grid shape, tolerance group size (0 = no tolerance)
struct TunedShape { int depth, rows, zchunk; };
std::map<std::tuple<int, int, int, int, int>, TunedShape> g_tune_cache;
}  // namespace

extern "C" {

// REFERENCE scheme: time the velocity sweep's forms -- one colour pass per launch, and the
// temporally blocked kernel with depth 2 and 4 over z-chunks without unroll padding -- per
// iteration (red + black pass) and keep the fastest.  The blocked launches read the state and
// write the scratch arrays (P, P2, b); the one-pass kernel runs in place on the scratch arrays,
// so the state is untouched.  Cached per grid shape and device.
static int autotune_velocity_sweep(smk_sim* sim, int* depth_out, int* zchunk_out, float* us_out) {
    const Grid& g = sim->g;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, g.nx, g.ny, g.nz, -100000);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            sim->vsweep_depth = sim->vmaps ? it->second.depth : 0;
            sim->vsweep_zchunk = it->second.zchunk;
            if (depth_out) *depth_out = sim->vsweep_depth;
            if (zchunk_out) *zchunk_out = sim->vsweep_zchunk;
            if (us_out) *us_out = -1.0f;
            return SMK_OK;
        }
    }
    SMK_CUDA(cudaDeviceSynchronize());
    cudaStream_t st = nullptr;
    SMK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    SMK_CUDA(cudaEventCreate(&e0));
    SMK_CUDA(cudaEventCreate(&e1));
    const int now = sim->index_now;
    const OmegaSplit os = omega_split(sim->p.omega);
    // microseconds per iteration of one candidate, issued as a step issues it
    auto time_it = [&](int depth, int zc, float* us) -> int {
        const int iters = 4;
        auto run = [&]() -> int {
            if (depth == 0) {
                for (int it = 0; it < iters; ++it) {
                    launch_project_velocity(g, sim->P, sim->P2, sim->b, sim->flags, 0, sim->p.omega, st);
                    launch_project_velocity(g, sim->P, sim->P2, sim->b, sim->flags, 1, sim->p.omega, st);
                }
                return SMK_OK;
            }
            for (int h = 0; h < 2 * iters; h += depth)
                if (launch_vsweep_tb(sim->vmaps, g, now, true, sim->P, sim->P2, sim->b, depth, depth, h & 1, zc,
                                     sim->p.omega, os, sim->kerr, st) != 0)
                    return fail(SMK_ERR_CUDA, "velocity sweep kernel launch failed");
            return SMK_OK;
        };
        int rc = run();  // warm
        if (rc) return rc;
        SMK_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < 2 && rc == SMK_OK; ++r) rc = run();
        if (rc) return rc;
        SMK_CUDA(cudaEventRecord(e1, st));
        SMK_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        SMK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        *us = 1e3f * ms / (2 * iters);
        return SMK_OK;
    };
    // every candidate timed in three interleaved rounds, each keeping its best round (a single
    // timing flipped between forms within a few percent of each other)
    struct Cand {
        int d, zc;
        float us;
    };
    std::vector<Cand> cands{Cand{0, 0, 1e30f}};
    const int depths[2] = {2, 4};
    for (int di = 0; di < 2 && sim->vmaps != nullptr; ++di) {
        const int T = depths[di], R = T + 2;
        for (int m = 2; m <= 40; ++m) {
            const int zc = R * m - 2 * T - 1;
            if (zc < 4) continue;
            if (zc > g.nz + 1 + R) break;
            cands.push_back(Cand{T, zc, 1e30f});
            if (zc > g.nz + 1) break;
        }
    }
    int rc = SMK_OK;
    for (int round = 0; round < 3 && rc == SMK_OK; ++round)
        for (auto& c : cands) {
            float us = 0.0f;
            rc = time_it(c.d, c.zc, &us);
            if (rc != SMK_OK) break;
            c.us = std::min(c.us, us);
        }
    int best_d = 0, best_z = 0;
    float best = 1e30f;
    for (const auto& c : cands)
        if (c.us < best) {
            best = c.us;
            best_d = c.d;
            best_z = c.zc;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (rc) return rc;
    SMK_CUDA(cudaGetLastError());
    sim->pressure_clobbered = true;
    int krc = check_kernel_error(sim);
    if (krc) return krc;
    sim->vsweep_depth = best_d;
    sim->vsweep_zchunk = best_z;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = TunedShape{best_d, 2, best_z};
    }
    if (depth_out) *depth_out = best_d;
    if (zchunk_out) *zchunk_out = best_z;
    if (us_out) *us_out = best;
    return SMK_OK;
}

int smk_autotune(smk_sim* sim, int* depth_out, int* zchunk_out, float* us_per_sweep_out) {
    if (!sim) return fail(SMK_ERR_INVALID, "sim is null");
    DeviceGuard dg(sim->device);
    if (sim->p.projection == SMK_PROJECT_REFERENCE)
        return autotune_velocity_sweep(sim, depth_out, zchunk_out, us_per_sweep_out);
    const Grid& g = sim->g;
    int dev = 0;
    cudaGetDevice(&dev);
    const int gkey = sim->p.tol > 0.0f ? sim->p.check_every : -std::max(1, std::min(sim->p.max_sweeps, 20));
    const auto key = std::make_tuple(dev, g.nx, g.ny, g.nz, gkey);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            sim->sweep_depth = it->second.depth;
            sim->sweep_rows = it->second.rows;
            sim->sweep_zchunk = it->second.zchunk;
            if (depth_out) *depth_out = sim->sweep_depth;
            if (zchunk_out) *zchunk_out = sim->sweep_zchunk;
            if (us_per_sweep_out) *us_per_sweep_out = -1.0f;
            return SMK_OK;
        }
    }
    SMK_CUDA(cudaDeviceSynchronize());
    // a live pressure in the second buffer (warm start) moves to the first
    int pc = 0;
    SMK_CUDA(cudaMemcpy(&pc, sim->pcur, sizeof(int), cudaMemcpyDeviceToHost));
    if (pc == 1) {
        SMK_CUDA(cudaMemcpy(sim->P, sim->P2, sim->elems() * sizeof(float), cudaMemcpyDeviceToDevice));
        SMK_CUDA(cudaMemset(sim->pcur, 0, sizeof(int)));
    }
    float wacc[7];
    wacc[0] = 0.0f;
    for (int a = 1; a <= 6; ++a) wacc[a] = (float)sim->p.omega / (float)a;
    cudaStream_t st = nullptr;
    SMK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    SMK_CUDA(cudaEventCreate(&e0));
    SMK_CUDA(cudaEventCreate(&e1));
    int best_d = sim->sweep_depth, best_r = sim->sweep_rows, best_z = sim->sweep_zchunk;
    float best = 1e30f;
    int shapes[7][2] = {{2, 2}, {4, 2}, {6, 2}, {4, 4}, {0, 0}, {0, 0}, {0, 0}};  // (depth, patch rows)
    for (int c = 0; c < 3; ++c) {  // y-cluster forms: one cluster spanning y, clusters of 2 and of 4
        const int n = c * 2;
        if (sweep_ycluster_usable(g, n) > 0) {
            shapes[4 + c][0] = 6;
            shapes[4 + c][1] = 2 | SWEEP_YCLUSTER | (n << SWEEP_YCLUSTER_N_SHIFT);
        }
    }
    // time one tolerance group exactly as a step issues it: 2G colour passes in launches of
    // `d` (the first one partial when d does not divide 2G), the first with the fused residual,
    // ping-ponging between the two pressure buffers (what a launch reads, the one before wrote).
    // The pressure a warm start keeps is saved first and put back afterwards; without room for
    // the copy, every launch reads P and writes P2.
    struct Saved {
        float* p = nullptr;
        float* dst = nullptr;
        size_t bytes = 0;
        ~Saved() {
            if (p) {
                cudaDeviceSynchronize();  // the timing stream does not order with the default one
                cudaMemcpy(dst, p, bytes, cudaMemcpyDeviceToDevice);
                cudaFree(p);
            }
        }
    } saved;
    saved.bytes = sim->elems() * sizeof(float);
    saved.dst = sim->P;
    if (cudaMalloc((void**)&saved.p, saved.bytes) != cudaSuccess) {
        cudaGetLastError();
        saved.p = nullptr;
    } else {
        SMK_CUDA(cudaMemcpy(saved.p, sim->P, saved.bytes, cudaMemcpyDeviceToDevice));
    }
    const bool use_tol = sim->p.tol > 0.0f;
    const int G = use_tol ? sim->p.check_every : std::max(1, std::min(sim->p.max_sweeps, 20));
    int nl = 0;
    // tolerance -1: the check launch records its residual but never ends the timed solve
    auto run_group = [&](int d, int rows, int zc) -> int {
        if (use_tol) SMK_CUDA(cudaMemsetAsync(sim->tune_status, 0, sizeof(StepStatus) + sizeof(unsigned), st));
        for (int h = 0; h < 2 * G;) {
            const int nh = (h == 0 && (2 * G) % d != 0) ? (2 * G) % d : d;
            const bool in_a = saved.p == nullptr || (nl & 1) == 0;
            if (launch_sweep_tb(sim->maps, g, in_a, in_a ? sim->P2 : sim->P, d, rows, nh, h & 1, zc, wacc,
                                use_tol ? sim->tune_status : nullptr, use_tol && h == 0, 0, -1.0f,
                                nullptr, 0, sim->kerr, nullptr, st) != 0)
                return fail(SMK_ERR_CUDA, "sweep kernel configuration failed");
            h += nh;
            ++nl;
        }
        return SMK_OK;
    };
    // every (shape, z-chunk) candidate, timed in three interleaved rounds, each keeping its
    // best round: a single timing flipped between shapes within a few percent of each other
    struct Cand {
        int d, rows, zc;
        float us;
    };
    std::vector<Cand> cands;
    for (const auto& shape : shapes) {
        const int d = shape[0], rows = shape[1];
        if (d == 0) continue;
        const int R = d + 4;
        for (int m = 2; m <= 16; ++m) {
            const int zc = R * m - 2 * d - 1;
            if (zc < 8) continue;
            if (zc > g.nz + R) break;
            cands.push_back(Cand{d, rows, zc, 1e30f});
            if (zc > g.nz) break;
        }
    }
    for (int round = 0; round < 3; ++round) {
        for (auto& c : cands) {
            const int reps = 2;
            int rc = run_group(c.d, c.rows, c.zc);  // warm
            if (rc) return rc;
            SMK_CUDA(cudaEventRecord(e0, st));
            for (int r = 0; r < reps && rc == SMK_OK; ++r) rc = run_group(c.d, c.rows, c.zc);
            if (rc) return rc;
            SMK_CUDA(cudaEventRecord(e1, st));
            SMK_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            SMK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            c.us = std::min(c.us, 1e3f * ms / (reps * G));
        }
    }
    for (const auto& c : cands) {
        if (c.us < best) {
            best = c.us;
            best_d = c.d;
            best_r = c.rows;
            best_z = c.zc;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    SMK_CUDA(cudaGetLastError());
    int krc = check_kernel_error(sim);
    if (krc) return krc;
    sim->sweep_depth = best_d;
    sim->sweep_rows = best_r;
    sim->sweep_zchunk = best_z;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = TunedShape{best_d, best_r, best_z};
    }
    if (depth_out) *depth_out = best_d;
    if (zchunk_out) *zchunk_out = best_z;
    if (us_per_sweep_out) *us_per_sweep_out = best;
    return SMK_OK;
}

}  // extern "C"
