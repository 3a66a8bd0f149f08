// Batches: many independent grids of uneven sizes stepped together (smk_batch_*).
//
// GROUPED form: one persistent launch per stage over every member (kernels_group.cu).  The
// host writes a table with one record per member for the step's ping-pong parity (its
// buffers, parameters and emitters) and the per-stage tile prefix sums, and captures the five
// launches of a step as one CUDA graph.  Every member flips parity each step, so two tables
// and two graphs alternate; both are rebuilt when a member's signature (dt, parameters,
// objects) changes.
//
// BRANCHES form: every member's own single-grid step is a concurrent branch of one graph
// (fork/join with events from an origin stream).
//
// In both forms a member's results are the same as stepping it alone: the grouped tiles run
// the single-grid stage bodies on the same cells, and the grouped projection applies the same
// colour passes in the same order with the same tolerance rule.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/smoke_gb300.h"
#include "group.h"
#include "kernels.h"
#include "sim_internal.h"

using namespace smk;

struct smk_batch {
    std::vector<smk_sim*> sims;
    int device = 0;
    int mode = SMK_BATCH_AUTO;
    bool use_graphs = true;
    bool graphs_ok = true;  // false after a grouped capture failed: grouped steps run directly
    int last_mode = 0;
    long long launches = 0;

    // BRANCHES form
    std::vector<cudaStream_t> branch;
    std::vector<cudaEvent_t> join;
    cudaStream_t origin = nullptr;
    cudaStream_t body = nullptr;  // captures the grouped blocked solve's loop body
    unsigned long long* dev_launches = nullptr;  // kernels run inside device-side loops
    cudaEvent_t fork = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::string sig;
    std::vector<long long> branch_launches;
    std::vector<int> groups;

    // GROUPED form: one slot per ping-pong parity state
    struct Slot {
        std::string sig;
        void* dev = nullptr;
        size_t cap = 0;
        cudaGraphExec_t exec = nullptr;
        GroupArgs args{};
        GroupLaunch L{};
        GroupTBLaunch tb{};
        bool blocked = false;
        int kernels = 0;
        unsigned long long used = 0;
    };
    Slot slots[2];
    unsigned long long clock = 0;
    // schedule of the grouped projection; ctas_per_sm 0 = all resident CTAs
    GroupSchedule sched{0, 4, 0, 0};
};

namespace {

constexpr int MAX_GROUPED = 16384;  // one byte of shared memory per grid in the projection kernel

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Table of the grouped step for the members' current parities (host image of the device blob).
struct TableImage {
    std::vector<GroupGrid> grids;
    std::vector<int> starts;
    std::vector<BoxObj> boxes;
    std::vector<SphereObj> spheres;
    int zslab = 1, nwaves = 1;
    size_t off_grids = 0, off_starts = 0, off_boxes = 0, off_spheres = 0, bytes = 0;
    // blocked solve: one record per grid (tensor maps, buffers), tile prefix sums, loop counter
    bool blocked = false;
    int tb_zchunk = 0, tb_total = 0, tb_check_every = 0, tb_max_sweeps = 0;
    std::vector<unsigned char> tb_recs;
    std::vector<int> tb_starts;
    std::vector<int> tb_order;  // member of each record
    size_t off_tb = 0, off_tb_starts = 0, off_tb_counter = 0;
};

// The blocked solve needs every member to share the tolerance group size and the sweep cap,
// with a tolerance rule (the launches of a group run in lockstep over all grids).
bool blocked_eligible(smk_sim* const* sims, int n) {
    if (n <= 0) return false;
    for (int i = 0; i < n; ++i) {
        const smk_params& p = sims[i]->p;
        if (!sims[i]->maps || p.tol <= 0.0f || p.max_sweeps <= 0 || p.check_every < 1 ||
            p.check_every != sims[0]->p.check_every || p.max_sweeps != sims[0]->p.max_sweeps)
            return false;
    }
    return true;
}

// Solve waves: first-fit decreasing on each grid's solver working set (P, b: 4 bytes, flags:
// 1 byte per element), so that one wave's passes can stay in L2.  A grid larger than the
// budget gets a wave of its own.  Returns the number of waves.
int assign_waves(std::vector<GroupGrid>& grids, long long budget) {
    const int n = (int)grids.size();
    if (budget <= 0) {
        for (auto& d : grids) d.wave = 0;
        return 1;
    }
    std::vector<long long> bytes(n);
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) {
        bytes[i] = 9LL * grids[i].g.XY * (grids[i].g.nz + 1);
        order[i] = i;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return bytes[a] > bytes[b]; });
    std::vector<long long> room;
    for (int i : order) {
        int w = 0;
        while (w < (int)room.size() && room[w] < bytes[i]) ++w;
        if (w == (int)room.size()) room.push_back(budget);
        room[w] -= bytes[i];
        grids[i].wave = w;
    }
    return (int)room.size();
}

void fill_record(smk_sim* s, float dt, TableImage& t, GroupGrid& d) {
    const smk_params& p = s->p;
    const int past = s->index_now, now = past ^ 1;  // the parities smk_sim::enqueue uses
    memset(&d, 0, sizeof(d));
    d.g = s->g;
    d.kind = p.storage;
    d.report_div = p.report_div ? 1 : 0;
    d.rho0 = s->rho[0];
    d.rho1 = s->rho[1];
    d.rho_now = s->rho[now];
    d.rho_past = s->rho[past];
    d.u_now = s->u[now];
    d.v_now = s->v[now];
    d.w_now = s->w[now];
    d.u_past = s->u[past];
    d.v_past = s->v[past];
    d.w_past = s->w[past];
    d.pu = s->bf16 ? s->proj[0] : s->u[now];
    d.pv = s->bf16 ? s->proj[1] : s->v[now];
    d.pw = s->bf16 ? s->proj[2] : s->w[now];
    d.P = s->P;
    d.b = s->b;
    d.P2 = s->P2;
    d.pcur = s->pcur;
    d.Ph = s->keeps_history() ? s->Ph : nullptr;  // smk_params.warm_extrapolate
    d.extrap = s->extrapolation();
    d.flags = s->flags;
    d.status = s->status;
    const bool use_tol = p.tol > 0.0f;
    const int ngroups = use_tol ? (p.max_sweeps + p.check_every - 1) / p.check_every : 0;
    d.status_words = 4 + std::min(ngroups + 1, s->status_groups);
    d.kerr = s->kerr;
    d.dt = dt;
    d.gravity = p.gravity;
    d.alpha = p.buoyancy;
    d.lim_sq = p.clamp_const * p.clamp_const;
    d.lim = p.clamp_const;
    d.clamp_mode = p.clamp_mode;
    d.wacc[0] = 0.0f;
    const double om = s->pressure_omega();  // omega, or omega_warm once the history is long enough
    for (int a = 1; a <= 6; ++a) d.wacc[a] = (float)om / (float)a;
    d.wacc[7] = 0.0f;
    d.tol = p.tol;
    d.check_every = p.check_every > 0 ? p.check_every : 1;
    d.max_sweeps = p.max_sweeps;
    d.warm = p.warm_start;
    // the 4-wide forcing, rhs and subtract / BF16 projection bodies (as the single-grid launchers)
    typedef __nv_bfloat16 h;
    if (!s->vec_stages)
        d.vec4 = 0;
    else if (d.kind == GK_F32)
        d.vec4 = vec4_layout(s->g, {d.u_now, d.v_now, d.w_now, d.rho_now, d.P, d.P2, d.b, d.Ph}, d.flags);
    else
        d.vec4 = vec4_layout_of<h>(s->g, {(const h*)d.u_now, (const h*)d.v_now, (const h*)d.w_now},
                                   {d.P, d.P2, d.b, d.pu, d.pv, d.pw, d.Ph}, d.flags) &&
                 (d.kind == GK_BF16 ? vec4_layout_of<h>(s->g, {(const h*)d.rho_now}, {}, d.flags)
                                    : vec4_layout(s->g, {d.rho_now}, d.flags));

    // emitters: boxes clipped to the grid (as the single-grid launcher does), then spheres
    const Grid& g = s->g;
    d.box0 = (int)t.boxes.size();
    int lo[3] = {g.nx, g.ny, g.nz}, hi[3] = {0, 0, 0};
    for (const auto& o : s->objects) {
        if (o.kind != smk_sim::OBJ_BOX) continue;
        BoxObj b = o.box;
        b.x0 = std::max(b.x0, 0); b.y0 = std::max(b.y0, 0); b.z0 = std::max(b.z0, 0);
        b.x1 = std::min(b.x1, g.nx); b.y1 = std::min(b.y1, g.ny); b.z1 = std::min(b.z1, g.nz);
        t.boxes.push_back(b);
        if (b.x0 < b.x1 && b.y0 < b.y1 && b.z0 < b.z1) {
            lo[0] = std::min(lo[0], b.x0); lo[1] = std::min(lo[1], b.y0); lo[2] = std::min(lo[2], b.z0);
            hi[0] = std::max(hi[0], b.x1); hi[1] = std::max(hi[1], b.y1); hi[2] = std::max(hi[2], b.z1);
        }
    }
    d.nbox = (int)t.boxes.size() - d.box0;
    const bool has_box = lo[0] < hi[0] && lo[1] < hi[1] && lo[2] < hi[2];
    if (has_box) {
        d.bx0 = lo[0]; d.by0 = lo[1]; d.bz0 = lo[2];
        d.bx1 = hi[0]; d.by1 = hi[1]; d.bz1 = hi[2];
    }
    d.sph0 = (int)t.spheres.size();
    for (const auto& o : s->objects)
        if (o.kind == smk_sim::OBJ_SPHERE) t.spheres.push_back(o.sphere);
    d.nsph = (int)t.spheres.size() - d.sph0;
    int a0[3], a1[3];
    const bool has_sph = d.nsph > 0 && sphere_bounds(g, &t.spheres[d.sph0], d.nsph, a0, a1);
    if (has_sph) {
        d.sx0 = a0[0]; d.sy0 = a0[1]; d.sz0 = a0[2];
        d.sx1 = a1[0]; d.sy1 = a1[1]; d.sz1 = a1[2];
    }
    if (has_box || has_sph) {
        d.ox0 = has_box ? d.bx0 : d.sx0; d.oy0 = has_box ? d.by0 : d.sy0; d.oz0 = has_box ? d.bz0 : d.sz0;
        d.ox1 = has_box ? d.bx1 : d.sx1; d.oy1 = has_box ? d.by1 : d.sy1; d.oz1 = has_box ? d.bz1 : d.sz1;
        if (has_sph) {
            d.ox0 = std::min(d.ox0, d.sx0); d.oy0 = std::min(d.oy0, d.sy0); d.oz0 = std::min(d.oz0, d.sz0);
            d.ox1 = std::max(d.ox1, d.sx1); d.oy1 = std::max(d.oy1, d.sy1); d.oz1 = std::max(d.oz1, d.sz1);
        }
    }
}

int build_table(smk_sim* const* sims, int n, const float* dts, float dt_all, const GroupSchedule& sch,
                TableImage& t) {
    t.grids.resize(n);
    t.boxes.clear();
    t.spheres.clear();
    for (int i = 0; i < n; ++i) fill_record(sims[i], dts ? dts[i] : dt_all, t, t.grids[i]);
    t.zslab = std::max(1, sch.zslab);
    t.nwaves = assign_waves(t.grids, sch.wave_bytes);
    t.blocked = sch.blocked_zchunk > 0 && blocked_eligible(sims, n);
    if (t.blocked) {
        const size_t rb = group_tb_record_bytes();
        t.tb_zchunk = sch.blocked_zchunk;
        t.tb_check_every = sims[0]->p.check_every;
        t.tb_max_sweeps = sims[0]->p.max_sweeps;
        t.tb_recs.assign(rb * n, 0);
        t.tb_starts.assign(n + 1, 0);
        // grids with the longest tiles (most planes per z-chunk) first: CTAs are dispatched in
        // index order, so the short tiles fill the last wave
        t.tb_order.resize(n);
        for (int i = 0; i < n; ++i) t.tb_order[i] = i;
        std::stable_sort(t.tb_order.begin(), t.tb_order.end(), [&](int a, int c) {
            return std::min(sims[a]->g.nz, t.tb_zchunk) > std::min(sims[c]->g.nz, t.tb_zchunk);
        });
        long long acc = 0;
        for (int i = 0; i < n; ++i) {
            smk_sim* sm = sims[t.tb_order[i]];
            float wacc[7];
            wacc[0] = 0.0f;
            const double om = sm->pressure_omega();
            for (int a = 1; a <= 6; ++a) wacc[a] = (float)om / (float)a;
            t.tb_starts[i] = (int)acc;
            acc += group_tb_fill(&t.tb_recs[rb * i], sm->maps, sm->g, sm->P, sm->P2, sm->status, sm->pcur, sm->kerr,
                                 wacc, sm->p.tol, t.tb_zchunk);
            if (acc > INT_MAX / 2) return smk_fail(SMK_ERR_INVALID, "batch too large for one blocked launch");
        }
        t.tb_starts[n] = (int)acc;
        t.tb_total = (int)acc;
    }
    t.starts.assign((size_t)GS_COUNT * (n + 1), 0);
    for (int s = 0; s < GS_COUNT; ++s) {
        long long acc = 0;
        for (int i = 0; i < n; ++i) {
            t.starts[(size_t)s * (n + 1) + i] = (int)acc;
            acc += group_tiles(s, t.grids[i], t.zslab);
            if (acc > INT_MAX / 2) return smk_fail(SMK_ERR_INVALID, "batch too large for one grouped launch");
        }
        t.starts[(size_t)s * (n + 1) + n] = (int)acc;
    }
    size_t off = align_up(sizeof(GroupSync), 256);
    t.off_grids = off;
    off = align_up(off + sizeof(GroupGrid) * n, 256);
    t.off_starts = off;
    off = align_up(off + sizeof(int) * t.starts.size(), 256);
    t.off_boxes = off;
    off = align_up(off + sizeof(BoxObj) * std::max<size_t>(1, t.boxes.size()), 256);
    t.off_spheres = off;
    off = align_up(off + sizeof(SphereObj) * std::max<size_t>(1, t.spheres.size()), 256);
    if (t.blocked) {
        t.off_tb = off;  // 256-byte aligned: the tensor maps in the records need 64
        off = align_up(off + t.tb_recs.size(), 256);
        t.off_tb_starts = off;
        off = align_up(off + sizeof(int) * t.tb_starts.size(), 256);
        t.off_tb_counter = off;
        off = align_up(off + sizeof(int), 256);
    }
    t.bytes = off;
    return SMK_OK;
}

// Lay a table image out in `blob` (t.bytes bytes) as the device copy will hold it.
void pack_table(const TableImage& t, char* blob) {
    memset(blob, 0, t.bytes);
    memcpy(blob + t.off_grids, t.grids.data(), sizeof(GroupGrid) * t.grids.size());
    memcpy(blob + t.off_starts, t.starts.data(), sizeof(int) * t.starts.size());
    if (!t.boxes.empty()) memcpy(blob + t.off_boxes, t.boxes.data(), sizeof(BoxObj) * t.boxes.size());
    if (!t.spheres.empty()) memcpy(blob + t.off_spheres, t.spheres.data(), sizeof(SphereObj) * t.spheres.size());
    if (t.blocked) {
        memcpy(blob + t.off_tb, t.tb_recs.data(), t.tb_recs.size());
        memcpy(blob + t.off_tb_starts, t.tb_starts.data(), sizeof(int) * t.tb_starts.size());
    }
}

// Blocked-solve launch description for a table whose device copy starts at `dev`.
GroupTBLaunch tb_launch(const TableImage& t, void* dev, int n, cudaStream_t body) {
    GroupTBLaunch tb{};
    char* base = static_cast<char*>(dev);
    tb.grids = base + t.off_tb;
    tb.starts = reinterpret_cast<const int*>(base + t.off_tb_starts);
    tb.n = n;
    tb.total = t.tb_total;
    tb.zchunk = t.tb_zchunk;
    tb.check_every = t.tb_check_every;
    tb.max_sweeps = t.tb_max_sweeps;
    tb.counter = reinterpret_cast<int*>(base + t.off_tb_counter);
    tb.body = body;
    return tb;
}

// Kernel arguments for a table whose device copy starts at `dev`.
void table_args(const TableImage& t, void* dev, GroupArgs& a, int n) {
    char* base = static_cast<char*>(dev);
    a.sync = reinterpret_cast<GroupSync*>(base);
    a.grids = reinterpret_cast<const GroupGrid*>(base + t.off_grids);
    a.starts = reinterpret_cast<const int*>(base + t.off_starts);
    a.boxes = reinterpret_cast<const BoxObj*>(base + t.off_boxes);
    a.spheres = reinterpret_cast<const SphereObj*>(base + t.off_spheres);
    a.n = n;
    a.zslab = t.zslab;
    a.nwaves = t.nwaves;
    a.sweeps_only = 0;
    a.phases = GP_ALL;
}

// Copy a table image into `dev` (synchronous; callers hold no step that reads it in flight).
int upload_table(const TableImage& t, void* dev, GroupArgs& a, int n) {
    std::vector<char> blob(t.bytes);
    pack_table(t, blob.data());
    SMK_CUDA(cudaMemcpy(dev, blob.data(), t.bytes, cudaMemcpyHostToDevice));
    table_args(t, dev, a, n);
    return SMK_OK;
}

int launch_config(const GroupSchedule& sched, const TableImage& t, GroupLaunch& L, int& kernels) {
    int coop = 0, stage = 0, sms = 0;
    const int rc = group_occupancy(&coop, &stage, &sms);
    if (rc) return smk_fail(SMK_ERR_CUDA, std::string("grouped kernels: ") + cudaGetErrorString((cudaError_t)rc));
    if (coop < 1) return smk_fail(SMK_ERR_CUDA, "grouped projection kernel cannot be resident");
    const int n = (int)t.grids.size();
    kernels = 1;  // the projection
    for (int s = 0; s < GS_COUNT; ++s) {
        L.total[s] = t.starts[(size_t)s * (n + 1) + n];
        L.ctas[s] = 0;
    }
    const int launched[4] = {GS_OBJECTS, GS_FORCE, GS_ADV_VEL, GS_ADV_RHO};
    for (int s : launched) kernels += L.total[s] > 0 ? 1 : 0;
    const int per_sm = sched.ctas_per_sm > 0 ? std::min(sched.ctas_per_sm, coop) : coop;
    L.coop_ctas = per_sm * sms;
    return SMK_OK;
}

// The grouped kernels run the PRESSURE projection's red-black solve: no refinement,
// moving-boundary velocities or Jacobi solver.
bool grouped_eligible(smk_sim* const* sims, int n) {
    if (n > MAX_GROUPED) return false;
    for (int i = 0; i < n; ++i)
        if (sims[i]->p.projection != SMK_PROJECT_PRESSURE || sims[i]->p.refine > 0 || sims[i]->p.obstacle_velocity ||
            sims[i]->p.solver != SMK_SOLVER_RBSOR)
            return false;
    return true;
}

bool grouped_eligible(const smk_batch* b) { return grouped_eligible(b->sims.data(), (int)b->sims.size()); }

void after_step(smk_sim* s) {
    s->index_now ^= 1;
    ++s->steps;
    ++s->hist_steps;
    const bool use_tol = s->p.tol > 0.0f;
    const int G = use_tol ? s->p.check_every : (s->p.max_sweeps > 0 ? s->p.max_sweeps : 1);
    s->last_groups = s->p.max_sweeps > 0 ? (s->p.max_sweeps + G - 1) / G : 0;
    s->last_projection = s->p.projection;
    s->last_tol = s->p.tol;
    s->last_max_sweeps = s->p.max_sweeps;
    s->last_check_every = s->p.check_every;
    s->last_refine = 0;
}

int grouped_step(smk_batch* b, const float* dts, float dt_all, cudaStream_t st) {
    const int n = (int)b->sims.size();
    // one-off mask / obstacle kernels of members with a pending change, ahead of the step
    for (smk_sim* s : b->sims)
        if (s->mask_dirty || s->obstacles_dirty) b->launches += s->prepare_mask(st);
    std::string sig;
    for (int i = 0; i < n; ++i) {
        smk_sim* s = b->sims[i];
        std::string gs = s->graph_signature(dts ? dts[i] : dt_all);
        const int len = (int)gs.size();
        sig.append(reinterpret_cast<const char*>(&len), sizeof(len));
        sig += gs;
        sig.push_back((char)s->index_now);
    }
    sig.append(reinterpret_cast<const char*>(&b->sched), sizeof(b->sched));
    smk_batch::Slot* slot = nullptr;
    for (auto& sl : b->slots)
        if (sl.dev && sl.sig == sig) slot = &sl;
    if (!slot) {
        slot = b->slots[0].used <= b->slots[1].used ? &b->slots[0] : &b->slots[1];
        TableImage t;
        int rc = build_table(b->sims.data(), n, dts, dt_all, b->sched, t);
        if (rc) return rc;
        // the slot being replaced may still be read by a step in flight
        SMK_CUDA(cudaDeviceSynchronize());
        if (slot->exec) {
            cudaGraphExecDestroy(slot->exec);
            slot->exec = nullptr;
        }
        slot->sig.clear();
        if (slot->cap < t.bytes) {
            if (slot->dev) cudaFree(slot->dev);
            slot->dev = nullptr;
            slot->cap = 0;
            SMK_CUDA(cudaMalloc(&slot->dev, t.bytes));
            slot->cap = t.bytes;
        }
        rc = upload_table(t, slot->dev, slot->args, n);
        if (rc) return rc;
        rc = launch_config(b->sched, t, slot->L, slot->kernels);
        if (rc) return rc;
        slot->blocked = t.blocked;
        if (t.blocked) {
            slot->tb = tb_launch(t, slot->dev, n, b->body);
            slot->tb.launches = b->dev_launches;
            slot->kernels += 1;  // the projection's second cooperative launch
        }
        if (b->use_graphs && b->graphs_ok) {
            cudaGraph_t graph = nullptr;
            SMK_CUDA(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
            const int lrc = launch_group_step(slot->args, slot->L, b->origin, slot->blocked ? &slot->tb : nullptr);
            if (lrc == 0 && slot->blocked) slot->kernels += slot->tb.issued;  // outside the loop
            const cudaError_t ee = cudaStreamEndCapture(b->origin, &graph);
            cudaError_t ie = cudaErrorUnknown;
            if (lrc == 0 && ee == cudaSuccess) ie = cudaGraphInstantiate(&slot->exec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (ie != cudaSuccess) {
                // capture of the cooperative launch is not available: run grouped steps directly
                slot->exec = nullptr;
                b->graphs_ok = false;
                cudaGetLastError();
            }
        }
        slot->sig.swap(sig);
    }
    slot->used = ++b->clock;
    if (slot->exec) {
        SMK_CUDA(cudaGraphLaunch(slot->exec, st));
    } else {
        const int lrc = launch_group_step(slot->args, slot->L, st, slot->blocked ? &slot->tb : nullptr);
        if (lrc) return smk_fail(SMK_ERR_CUDA, std::string("grouped step: ") + cudaGetErrorString((cudaError_t)lrc));
        if (slot->blocked) b->launches += slot->tb.issued;  // direct: every group issued
    }
    b->launches += slot->kernels;
    for (smk_sim* s : b->sims) after_step(s);
    b->last_mode = SMK_BATCH_GROUPED;
    return SMK_OK;
}

int branches_step(smk_batch* b, const float* dts, float dt_all, cudaStream_t st) {
    const int n = (int)b->sims.size();
    bool direct = !b->use_graphs;
    std::string sig;
    for (int i = 0; i < n; ++i) {
        smk_sim* s = b->sims[i];
        if (s->timing || s->mask_dirty || s->obstacles_dirty || !s->use_graphs) direct = true;
        std::string gs = s->graph_signature(dts ? dts[i] : dt_all);
        const int len = (int)gs.size();
        sig.append(reinterpret_cast<const char*>(&len), sizeof(len));
        sig += gs;
        sig.push_back((char)s->index_now);
    }
    b->last_mode = SMK_BATCH_BRANCHES;
    if (direct) {
        // direct launches on the branch streams, ordered after `st`
        SMK_CUDA(cudaEventRecord(b->fork, st));
        for (int i = 0; i < n; ++i) {
            smk_sim* s = b->sims[i];
            const long long l0 = s->launches;
            SMK_CUDA(cudaStreamWaitEvent(b->branch[i], b->fork, 0));
            const int rc = s->step(dts ? dts[i] : dt_all, b->branch[i]);
            if (rc) return rc;
            b->launches += s->launches - l0;
            SMK_CUDA(cudaEventRecord(b->join[i], b->branch[i]));
            SMK_CUDA(cudaStreamWaitEvent(st, b->join[i], 0));
        }
        return SMK_OK;
    }
    if (b->exec == nullptr || sig != b->sig) {
        std::vector<int> idx0(n), steps0(n);
        std::vector<long long> l0(n), hist0(n);
        for (int i = 0; i < n; ++i) {
            idx0[i] = b->sims[i]->index_now;
            steps0[i] = b->sims[i]->steps;
            hist0[i] = b->sims[i]->hist_steps;
            l0[i] = b->sims[i]->launches;
        }
        SMK_CUDA(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
        int rc = SMK_OK;
        cudaError_t ce = cudaEventRecord(b->fork, b->origin);
        for (int i = 0; i < n && rc == SMK_OK && ce == cudaSuccess; ++i) {
            ce = cudaStreamWaitEvent(b->branch[i], b->fork, 0);
            if (ce != cudaSuccess) break;
            // concurrent branches: unrolled group launches (a device-side loop per branch costs
            // more than the launches it saves when many graphs run at once)
            const bool loops = b->sims[i]->graph_loops;
            b->sims[i]->graph_loops = false;
            rc = b->sims[i]->enqueue(dts ? dts[i] : dt_all, b->branch[i]);
            b->sims[i]->graph_loops = loops;
            if (rc == SMK_OK) ce = cudaEventRecord(b->join[i], b->branch[i]);
            if (rc == SMK_OK && ce == cudaSuccess) ce = cudaStreamWaitEvent(b->origin, b->join[i], 0);
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(b->origin, &graph);
        for (int i = 0; i < n; ++i) {
            smk_sim* s = b->sims[i];
            b->branch_launches[i] = s->launches - l0[i];
            b->groups[i] = s->last_groups;
            s->index_now = idx0[i];
            s->steps = steps0[i];
            s->hist_steps = hist0[i];
            s->launches = l0[i];
        }
        if (rc != SMK_OK || ce != cudaSuccess || ee != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            if (rc) return rc;
            return smk_fail(SMK_ERR_CUDA, std::string("batch capture: ") +
                                              cudaGetErrorString(ce != cudaSuccess ? ce : ee));
        }
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return smk_fail(SMK_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(ie));
        b->sig.swap(sig);
    }
    SMK_CUDA(cudaGraphLaunch(b->exec, st));
    for (int i = 0; i < n; ++i) {
        smk_sim* s = b->sims[i];
        s->index_now ^= 1;
        s->launches += b->branch_launches[i];
        b->launches += b->branch_launches[i];
        ++s->steps;
        ++s->hist_steps;
        s->last_groups = b->groups[i];
        s->last_projection = s->p.projection;
        s->last_tol = s->p.tol;
        s->last_max_sweeps = s->p.max_sweeps;
        s->last_check_every = s->p.check_every;
        s->last_refine = s->p.projection == SMK_PROJECT_PRESSURE ? s->p.refine : 0;
    }
    return SMK_OK;
}

void release_slots(smk_batch* b) {
    for (auto& sl : b->slots) {
        if (sl.exec) cudaGraphExecDestroy(sl.exec);
        if (sl.dev) cudaFree(sl.dev);
        sl = smk_batch::Slot();
    }
}

}  // namespace

// ---- grouped steps over a changing set of simulations (the serving loop) ----------------------

struct GroupRunner {
    struct Slot {
        void* dev = nullptr;
        char* host = nullptr;  // pinned staging of the table copy
        size_t cap = 0;
        cudaEvent_t done = nullptr;
        bool used = false;
    };
    static constexpr int RING = 4;
    Slot ring[RING];
    int next = 0;
};

GroupRunner* group_runner_create() {
    GroupRunner* r = new GroupRunner();
    for (auto& sl : r->ring) {
        if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            group_runner_destroy(r);
            return nullptr;
        }
    }
    return r;
}

void group_runner_destroy(GroupRunner* r) {
    if (!r) return;
    for (auto& sl : r->ring) {
        if (sl.done) {
            if (sl.used) cudaEventSynchronize(sl.done);
            cudaEventDestroy(sl.done);
        }
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
    }
    delete r;
}

bool group_runner_eligible(smk_sim* sim) { return grouped_eligible(&sim, 1); }

int group_runner_step(GroupRunner* r, smk_sim* const* sims, const float* dts, int n,
                      const GroupSchedule& sched, cudaStream_t st, int* kernels) {
    if (kernels) *kernels = 0;
    if (!r || n <= 0) return SMK_OK;
    if (!grouped_eligible(sims, n))
        return smk_fail(SMK_ERR_INVALID, "a grouped step needs the PRESSURE projection in every member");
    int k = 0;
    for (int i = 0; i < n; ++i)
        if (sims[i]->mask_dirty || sims[i]->obstacles_dirty) k += sims[i]->prepare_mask(st);
    TableImage t;
    int rc = build_table(sims, n, dts, 0.0f, sched, t);
    if (rc) return rc;
    GroupRunner::Slot& sl = r->ring[r->next];
    r->next = (r->next + 1) % GroupRunner::RING;
    if (sl.used) SMK_CUDA(cudaEventSynchronize(sl.done));  // the step that last read it is done
    if (sl.cap < t.bytes) {
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
        sl.dev = nullptr;
        sl.host = nullptr;
        sl.cap = 0;
        SMK_CUDA(cudaMalloc(&sl.dev, t.bytes));
        SMK_CUDA(cudaMallocHost((void**)&sl.host, t.bytes));
        sl.cap = t.bytes;
    }
    pack_table(t, sl.host);
    SMK_CUDA(cudaMemcpyAsync(sl.dev, sl.host, t.bytes, cudaMemcpyHostToDevice, st));
    GroupArgs a{};
    table_args(t, sl.dev, a, n);
    GroupLaunch L{};
    int nk = 0;
    rc = launch_config(sched, t, L, nk);
    if (rc) return rc;
    GroupTBLaunch tb{};
    if (t.blocked) tb = tb_launch(t, sl.dev, n, nullptr);
    const int lrc = launch_group_step(a, L, st, t.blocked ? &tb : nullptr);
    if (lrc) return smk_fail(SMK_ERR_CUDA, std::string("grouped step: ") + cudaGetErrorString((cudaError_t)lrc));
    SMK_CUDA(cudaEventRecord(sl.done, st));
    sl.used = true;
    for (int i = 0; i < n; ++i) after_step(sims[i]);
    if (kernels) *kernels = k + nk + (t.blocked ? 1 + tb.issued : 0);
    return SMK_OK;
}

extern "C" {

int smk_batch_create(int count, smk_sim* const* sims, smk_batch** out) {
    if (!out || count <= 0 || !sims) return smk_fail(SMK_ERR_INVALID, "need at least one simulation");
    *out = nullptr;
    smk_batch* b = new smk_batch();
    cudaGetDevice(&b->device);
    for (int i = 0; i < count; ++i) {
        if (!sims[i] || sims[i]->device != b->device) {
            delete b;
            return smk_fail(SMK_ERR_INVALID, "batch members must be valid simulations on the current device");
        }
        b->sims.push_back(sims[i]);
    }
    auto cleanup = [b]() {
        for (auto s : b->branch) if (s) cudaStreamDestroy(s);
        for (auto e : b->join) if (e) cudaEventDestroy(e);
        if (b->origin) cudaStreamDestroy(b->origin);
        if (b->body) cudaStreamDestroy(b->body);
        if (b->fork) cudaEventDestroy(b->fork);
        if (b->dev_launches) cudaFree(b->dev_launches);
        delete b;
    };
    if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->body, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc((void**)&b->dev_launches, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(b->dev_launches, 0, sizeof(unsigned long long)) != cudaSuccess) {
        cleanup();
        return smk_fail(SMK_ERR_CUDA, "batch stream/event creation failed");
    }
    b->branch.assign(count, nullptr);
    b->join.assign(count, nullptr);
    for (int i = 0; i < count; ++i) {
        if (cudaStreamCreateWithFlags(&b->branch[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) != cudaSuccess) {
            cleanup();
            return smk_fail(SMK_ERR_CUDA, "batch stream/event creation failed");
        }
    }
    b->branch_launches.assign(count, 0);
    b->groups.assign(count, 0);
    *out = b;
    return SMK_OK;
}

int smk_batch_destroy(smk_batch* b) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    DeviceGuard dg(b->device);
    cudaDeviceSynchronize();
    release_slots(b);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (auto s : b->branch) cudaStreamDestroy(s);
    for (auto e : b->join) cudaEventDestroy(e);
    cudaStreamDestroy(b->origin);
    cudaStreamDestroy(b->body);
    cudaEventDestroy(b->fork);
    cudaFree(b->dev_launches);
    delete b;
    return SMK_OK;
}

int smk_batch_set_mode(smk_batch* b, int mode) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    if (mode != SMK_BATCH_AUTO && mode != SMK_BATCH_GROUPED && mode != SMK_BATCH_BRANCHES)
        return smk_fail(SMK_ERR_INVALID, "unknown batch mode");
    if (mode == SMK_BATCH_GROUPED && !grouped_eligible(b))
        return smk_fail(SMK_ERR_INVALID, "the grouped form needs the PRESSURE projection without "
                                         "refinement in every member (and at most 16384 members)");
    b->mode = mode;
    return SMK_OK;
}

int smk_batch_set_graphs(smk_batch* b, int enable) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    b->use_graphs = enable != 0;
    return SMK_OK;
}

int smk_batch_get_info(const smk_batch* b, int* last_mode, long long* launches) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    if (last_mode) *last_mode = b->last_mode;
    if (launches) {
        // plus the kernels run inside device-side loops (counted on the device)
        unsigned long long dev = 0;
        if (b->dev_launches) {
            DeviceGuard dg(b->device);
            SMK_CUDA(cudaMemcpy(&dev, b->dev_launches, sizeof(dev), cudaMemcpyDeviceToHost));
        }
        *launches = b->launches + (long long)dev;
    }
    return SMK_OK;
}

// dts: one dt per grid (NULL: every grid uses dt_all).  Stream-ordered on `stream`.
int smk_batch_step(smk_batch* b, const float* dts, float dt_all, void* stream) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    DeviceGuard dg(b->device);
    cudaStream_t st = (cudaStream_t)stream;
    bool grouped = b->mode != SMK_BATCH_BRANCHES && grouped_eligible(b);
    // stage timing is per member: per-member steps
    for (const smk_sim* s : b->sims)
        if (s->timing) grouped = false;
    if (grouped) return grouped_step(b, dts, dt_all, st);
    return branches_step(b, dts, dt_all, st);
}

// Times the cooperative projection kernel running a fixed number of sweeps over every member
// (no tolerance checks) on the members' second pressure buffers, which hold no live state
// once a pressure left there by a blocked sweep kernel has been moved to the first buffer.
// Searched: CTAs per SM x z planes per tile x solve-wave budget; the fastest is kept.
int smk_batch_autotune(smk_batch* b, int* ctas_per_sm, float* us_per_sweep) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    if (!grouped_eligible(b)) return smk_fail(SMK_ERR_INVALID, "the batch cannot use the grouped form");
    DeviceGuard dg(b->device);
    SMK_CUDA(cudaDeviceSynchronize());
    const int n = (int)b->sims.size();
    for (smk_sim* s : b->sims) {
        int pc = 0;
        SMK_CUDA(cudaMemcpy(&pc, s->pcur, sizeof(int), cudaMemcpyDeviceToHost));
        if (pc == 1) {
            SMK_CUDA(cudaMemcpy(s->P, s->P2, s->elems() * sizeof(float), cudaMemcpyDeviceToDevice));
            SMK_CUDA(cudaMemset(s->pcur, 0, sizeof(int)));
        }
    }
    int coop = 0, stage = 0, sms = 0;
    if (group_occupancy(&coop, &stage, &sms) != 0 || coop < 1)
        return smk_fail(SMK_ERR_CUDA, "grouped kernels: occupancy query failed");
    std::vector<int> ctas;
    for (int c : {2, 4, coop})
        if (c <= coop && std::find(ctas.begin(), ctas.end(), c) == ctas.end()) ctas.push_back(c);
    const int zslabs[] = {1, 4, 8, 16};
    const long long waves[] = {0, 32LL << 20, 64LL << 20, 96LL << 20};
    const int sweeps = 8;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    void* dev = nullptr;
    size_t cap = 0;
    int rc = SMK_OK;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        rc = smk_fail(SMK_ERR_CUDA, "autotune stream/event creation failed");
    GroupSchedule best_s = b->sched;
    float best = 1e30f;
    for (int zs : zslabs) {
        for (long long wb : waves) {
            if (rc) break;
            TableImage t;
            rc = build_table(b->sims.data(), n, nullptr, 0.0f, GroupSchedule{0, zs, wb}, t);
            if (rc) break;
            if (wb > 0 && t.nwaves == 1) continue;  // same schedule as one wave
            for (GroupGrid& d : t.grids) {
                d.P = const_cast<float*>(d.P2);  // scratch
                d.tol = 0.0f;
                d.max_sweeps = sweeps;
            }
            if (cap < t.bytes) {
                if (dev) cudaFree(dev);
                dev = nullptr;
                if (cudaMalloc(&dev, t.bytes) != cudaSuccess) {
                    rc = smk_fail(SMK_ERR_OOM, "autotune table allocation failed");
                    break;
                }
                cap = t.bytes;
            }
            GroupArgs a{};
            rc = upload_table(t, dev, a, n);
            if (rc) break;
            a.sweeps_only = 1;
            for (int c : ctas) {
                GroupLaunch L{};
                L.coop_ctas = c * sms;
                const int reps = 3;
                int lrc = launch_group_sweeps_only(a, L, st);  // warm
                if (!lrc) lrc = (int)cudaEventRecord(e0, st);
                for (int r = 0; r < reps && !lrc; ++r) lrc = launch_group_sweeps_only(a, L, st);
                if (!lrc) lrc = (int)cudaEventRecord(e1, st);
                if (!lrc) lrc = (int)cudaEventSynchronize(e1);
                if (lrc) {
                    rc = smk_fail(SMK_ERR_CUDA, std::string("autotune launch: ") +
                                                    cudaGetErrorString((cudaError_t)lrc));
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                const float us = 1e3f * ms / (reps * sweeps);
                if (us < best) {
                    best = us;
                    best_s = GroupSchedule{c, zs, wb};
                }
            }
        }
    }
    // the blocked solve (when every member can use it): depth-6 launches over all grids' tiles,
    // timed without tolerance checks, reading P and writing the scratch P2 (no status, no pcur)
    const int zchunks[] = {17, 27, 37, 57, 117, 137, 257};  // 10 m - 13: no padding of the 10-plane unroll
    if (!rc && blocked_eligible(b->sims.data(), n)) {
        for (int zc : zchunks) {
            TableImage t;
            rc = build_table(b->sims.data(), n, nullptr, 0.0f, GroupSchedule{0, 4, 0, zc}, t);
            if (rc) break;
            const size_t rb = group_tb_record_bytes();
            for (int i = 0; i < n; ++i) {
                smk_sim* sm = b->sims[t.tb_order[i]];
                float wacc[7];
                wacc[0] = 0.0f;
                for (int a = 1; a <= 6; ++a) wacc[a] = (float)sm->p.omega / (float)a;
                group_tb_fill(&t.tb_recs[rb * i], sm->maps, sm->g, sm->P, sm->P2, nullptr, nullptr, sm->kerr, wacc,
                              sm->p.tol, zc);
            }
            if (cap < t.bytes) {
                if (dev) cudaFree(dev);
                dev = nullptr;
                if (cudaMalloc(&dev, t.bytes) != cudaSuccess) {
                    rc = smk_fail(SMK_ERR_OOM, "autotune table allocation failed");
                    break;
                }
                cap = t.bytes;
            }
            GroupArgs a{};
            rc = upload_table(t, dev, a, n);
            if (rc) break;
            const GroupTBLaunch tb = tb_launch(t, dev, n, nullptr);
            const int reps = 3, launches = 3;  // 9 sweeps per repetition
            int lrc = launch_group_tb_sweeps(tb, launches, st);  // warm
            if (!lrc) lrc = (int)cudaEventRecord(e0, st);
            for (int r = 0; r < reps && !lrc; ++r) lrc = launch_group_tb_sweeps(tb, launches, st);
            if (!lrc) lrc = (int)cudaEventRecord(e1, st);
            if (!lrc) lrc = (int)cudaEventSynchronize(e1);
            if (lrc) {
                rc = smk_fail(SMK_ERR_CUDA, std::string("autotune launch: ") + cudaGetErrorString((cudaError_t)lrc));
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            const float us = 1e3f * ms / (reps * launches * 3);
            if (us < best) {
                best = us;
                best_s = GroupSchedule{0, 4, 0, zc};
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (dev) cudaFree(dev);
    if (rc) return rc;
    for (smk_sim* s : b->sims) {
        int e = 0;
        SMK_CUDA(cudaMemcpy(&e, s->kerr, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) return smk_fail(SMK_ERR_TIMEOUT, "a grid barrier of the grouped projection gave up during tuning");
    }
    b->sched = best_s;
    if (ctas_per_sm) *ctas_per_sm = best_s.ctas_per_sm;
    if (us_per_sweep) *us_per_sweep = best;
    return SMK_OK;
}

/* The grouped projection's schedule (after smk_batch_autotune, or the defaults). */
int smk_batch_get_schedule(const smk_batch* b, int* ctas_per_sm, int* zslab, long long* wave_bytes) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    if (ctas_per_sm) *ctas_per_sm = b->sched.ctas_per_sm;
    if (zslab) *zslab = b->sched.zslab;
    if (wave_bytes) *wave_bytes = b->sched.wave_bytes;
    return SMK_OK;
}

int smk_batch_set_schedule(smk_batch* b, int ctas_per_sm, int zslab, long long wave_bytes) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    if (ctas_per_sm < 0 || zslab < 1 || zslab > 4096 || wave_bytes < 0)
        return smk_fail(SMK_ERR_INVALID, "invalid grouped schedule");
    b->sched = GroupSchedule{ctas_per_sm, zslab, wave_bytes, 0};
    return SMK_OK;
}

int smk_batch_set_blocked(smk_batch* b, int zchunk) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    if (zchunk < 0) return smk_fail(SMK_ERR_INVALID, "zchunk must be >= 0");
    b->sched.blocked_zchunk = zchunk;
    return SMK_OK;
}

int smk_batch_get_blocked(const smk_batch* b, int* zchunk) {
    if (!b) return smk_fail(SMK_ERR_INVALID, "batch is null");
    if (zchunk) *zchunk = b->sched.blocked_zchunk;
    return SMK_OK;
}

}  // extern "C"
