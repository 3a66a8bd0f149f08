// Continuous-batching serving loop for smoke simulations (smk_server_*).
//
// The reference runs one simulation per process, stepped from the render loop at 20 Hz
// (project/main.cpp:93, :889-896).  A server instead keeps many simulations resident on one GPU
// and admits new ones while others run:
//   - submit() queues a request (grid size, step count, scene, parameters);
//   - tick() (1) collects the steps that completed and retires requests whose last step has
//     completed: their density is copied to the caller's host buffer and their device memory is
//     freed; (2) admits queued requests in arrival order while the device-memory budget and the
//     slot limit allow; (3) issues the next step of every active request, in one of two forms:
//       STREAMS (default): each request's own step (its captured graph of single-grid kernels,
//         with the blocked sweep kernel) on its own stream, so the requests' kernels overlap;
//         latency = device time of the request's step, events on its stream;
//       GROUPED: ONE grouped step over every active request (one persistent launch per stage
//         over all the requests' grids, kernels_group.cu), so the requests share every launch;
//         latency = device time of that step, for every member;
//     a request admitted now joins the next step.  Up to two steps per request (STREAMS) or per
//     server (GROUPED) are in flight, so the host prepares the next step while the device runs.
// Each request is an independent simulation with its own buffers, and the grouped kernels give
// every grid the results it gets alone (tested: alone vs in the mix).  Host-side failures (a
// request that does not fit the budget at all, allocation failure, invalid input) are reported
// per request.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "../../include/smoke_gb300.h"
#include "group.h"
#include "sim_internal.h"

namespace {

thread_local std::string g_srv_err;

int sfail(int code, const std::string& m) {
    g_srv_err = m;
    return code;
}

struct Request {
    int id = 0;
    int nx = 0, ny = 0, nz = 0, steps = 0;
    float dt = 0.0f;
    smk_params params{};
    std::vector<uint8_t> mask;  // empty: reference initial mask
    std::vector<float> spheres, boxes, obstacles;  // reference packing (4 / 9 / 7 floats)
    float* out = nullptr;                          // caller's buffer for the final density
    bool out_on_device = false;
    bool out_pinned = false;                       // out was page-locked by the server
    bool retiring = false;                         // final density copy in flight (retire_ev)
    cudaEvent_t retire_ev = nullptr;
    int state = SMK_REQ_QUEUED;
    int steps_issued = 0;
    int steps_done = 0;
    int error = SMK_OK;
    size_t bytes = 0;
    bool cancel = false;  // smk_server_cancel on an active request: no new steps, then released
    smk_sim* sim = nullptr;
    // STREAMS form: the request's own stream and two step slots (issue / collect)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start[2] = {nullptr, nullptr};
    cudaEvent_t ev_end[2] = {nullptr, nullptr};
    bool pending[2] = {false, false};
    std::chrono::steady_clock::time_point submitted;  // host clock at smk_server_submit
};

// One issued server step: its events and the requests it advanced.
struct TickRec {
    cudaEvent_t start = nullptr, end = nullptr;
    std::vector<Request*> members;
    bool pending = false;
};

size_t footprint(int nx, int ny, int nz) {
    const size_t X = ((size_t)nx + 1 + 15) / 16 * 16;
    const size_t elems = X * (size_t)(ny + 1) * (size_t)(nz + 1);
    return elems * (11 * sizeof(float) + 2) + (1u << 20);
}

}  // namespace

struct smk_server {
    size_t budget = 0;
    size_t used = 0;
    int max_active = 0;
    int next_id = 1;
    int device = 0;
    std::deque<Request*> queue;
    std::vector<Request*> active;
    std::vector<Request*> all;  // owned
    std::vector<float> latencies_ms;
    std::vector<float> queue_ms;  // per admitted request: submission to admission (host clock)
    int peak_active = 0, peak_queued = 0;
    size_t peak_bytes = 0;
    double cell_updates = 0.0;
    long long steps_completed = 0;
    int requests_completed = 0;
    int mode = SMK_SERVE_STREAMS;
    // smk_set_graph_loops for every admitted request.  Off by default: with many requests'
    // graphs running concurrently, each iteration of a device-side loop costs more than the
    // launches it saves (measured: 40-request stream 3.0 vs 3.6 G cell-updates/s).
    int graph_loops = 0;
    bool started = false;  // the form is fixed once a request was admitted
    cudaStream_t stream = nullptr;
    GroupRunner* runner = nullptr;
    // GROUPED form: the blocked solve with 137-plane z-chunks (the batch autotuner's choice on a
    // 64-grid batch of cubes of side 32..128); ticks whose requests do not share a tolerance
    // group size and sweep cap use the colour passes
    smk::GroupSchedule sched{0, 4, 0, 137};
    TickRec ticks[2];
    int tick_next = 0;
};

extern "C" {

const char* smk_server_last_error(void) { return g_srv_err.c_str(); }

static void destroy_server(smk_server* s) {
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (Request* r : s->all) {
        if (r->sim) smk_destroy(r->sim);
        for (int k = 0; k < 2; ++k) {
            if (r->ev_start[k]) cudaEventDestroy(r->ev_start[k]);
            if (r->ev_end[k]) cudaEventDestroy(r->ev_end[k]);
        }
        if (r->stream) cudaStreamDestroy(r->stream);
        delete r;
    }
    for (TickRec& t : s->ticks) {
        if (t.start) cudaEventDestroy(t.start);
        if (t.end) cudaEventDestroy(t.end);
    }
    if (s->runner) group_runner_destroy(s->runner);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int smk_server_create(size_t budget_bytes, int max_active, smk_server** out) {
    if (!out || budget_bytes == 0 || max_active < 1) return sfail(SMK_ERR_INVALID, "bad server limits");
    *out = nullptr;
    smk_server* s = new smk_server();
    s->budget = budget_bytes;
    s->max_active = max_active;
    cudaGetDevice(&s->device);
    *out = s;
    return SMK_OK;
}

// The server's stream, step events and grouped-step runner, created with the first step.
static int ensure_device_state(smk_server* s) {
    if (s->runner) return SMK_OK;
    bool ok = s->stream || cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess;
    for (TickRec& t : s->ticks) {
        ok = ok && (t.start || cudaEventCreate(&t.start) == cudaSuccess);
        ok = ok && (t.end || cudaEventCreate(&t.end) == cudaSuccess);
    }
    if (ok) s->runner = group_runner_create();
    return ok && s->runner ? SMK_OK : sfail(SMK_ERR_CUDA, "server stream/event creation failed");
}

static void release_request(smk_server* s, Request* r) {
    if (r->sim) {
        smk_destroy(r->sim);
        r->sim = nullptr;
        s->used -= r->bytes;
    }
    if (r->out_pinned) {
        cudaHostUnregister(r->out);
        r->out_pinned = false;
    }
    if (r->retire_ev) cudaEventDestroy(r->retire_ev);
    r->retire_ev = nullptr;
    for (int k = 0; k < 2; ++k) {
        if (r->ev_start[k]) cudaEventDestroy(r->ev_start[k]);
        if (r->ev_end[k]) cudaEventDestroy(r->ev_end[k]);
        r->ev_start[k] = r->ev_end[k] = nullptr;
    }
    if (r->stream) cudaStreamDestroy(r->stream);
    r->stream = nullptr;
}

int smk_server_cancel(smk_server* s, int id) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        if ((*it)->id == id) {
            (*it)->state = SMK_REQ_CANCELLED;
            s->queue.erase(it);
            return SMK_OK;
        }
    }
    for (Request* r : s->active) {
        if (r->id == id) {
            r->cancel = true;  // released by a later tick once its issued steps have completed
            return SMK_OK;
        }
    }
    for (Request* r : s->all)
        if (r->id == id) return SMK_OK;  // already finished, failed or cancelled
    return sfail(SMK_ERR_INVALID, "unknown request id");
}

int smk_server_set_graph_loops(smk_server* s, int enable) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    s->graph_loops = enable != 0;
    return SMK_OK;
}

int smk_server_set_blocked(smk_server* s, int zchunk) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    if (zchunk < 0) return sfail(SMK_ERR_INVALID, "zchunk must be >= 0");
    s->sched.blocked_zchunk = zchunk;
    return SMK_OK;
}

int smk_server_set_mode(smk_server* s, int mode) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    if (mode != SMK_SERVE_STREAMS && mode != SMK_SERVE_GROUPED) return sfail(SMK_ERR_INVALID, "unknown serving form");
    if (s->started && mode != s->mode) return sfail(SMK_ERR_INVALID, "the serving form is fixed once requests run");
    s->mode = mode;
    return SMK_OK;
}

int smk_server_destroy(smk_server* s) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    destroy_server(s);
    return SMK_OK;
}

int smk_server_submit(smk_server* s, const smk_request_desc* d, int* id) {
    if (!s || !d) return sfail(SMK_ERR_INVALID, "null argument");
    if (d->nx < 3 || d->ny < 3 || d->nz < 3 || d->steps < 1 || !(d->dt > 0.0f) || !std::isfinite(d->dt))
        return sfail(SMK_ERR_INVALID, "request needs a grid of at least 3^3 cells, steps >= 1, finite dt > 0");
    if (d->n_spheres < 0 || d->n_boxes < 0 || d->n_obstacles < 0 ||
        (d->n_spheres > 0 && !d->spheres) || (d->n_boxes > 0 && !d->boxes) || (d->n_obstacles > 0 && !d->obstacles))
        return sfail(SMK_ERR_INVALID, "object counts and arrays do not match");
    // non-finite host inputs are rejected here rather than propagated into the simulation
    auto finite = [](const float* a, size_t n) {
        for (size_t k = 0; k < n; ++k)
            if (!std::isfinite(a[k])) return false;
        return true;
    };
    if ((d->n_spheres > 0 && !finite(d->spheres, 4 * (size_t)d->n_spheres)) ||
        (d->n_boxes > 0 && !finite(d->boxes, 9 * (size_t)d->n_boxes)) ||
        (d->n_obstacles > 0 && !finite(d->obstacles, 7 * (size_t)d->n_obstacles)))
        return sfail(SMK_ERR_INVALID, "non-finite value in the request's objects");
    if (d->params && (!std::isfinite(d->params->gravity) || !std::isfinite(d->params->buoyancy) ||
                      !std::isfinite(d->params->clamp_const) || !std::isfinite(d->params->omega) ||
                      !std::isfinite(d->params->tol)))
        return sfail(SMK_ERR_INVALID, "non-finite value in the request's parameters");
    Request* r = new Request();
    r->id = s->next_id++;
    r->nx = d->nx;
    r->ny = d->ny;
    r->nz = d->nz;
    r->steps = d->steps;
    r->dt = d->dt;
    if (d->params) r->params = *d->params;
    else smk_default_params(&r->params);
    const size_t cells = (size_t)d->nx * d->ny * d->nz;
    if (d->mask) r->mask.assign(d->mask, d->mask + cells);
    if (d->n_spheres > 0) r->spheres.assign(d->spheres, d->spheres + 4 * d->n_spheres);
    if (d->n_boxes > 0) r->boxes.assign(d->boxes, d->boxes + 9 * d->n_boxes);
    if (d->n_obstacles > 0) r->obstacles.assign(d->obstacles, d->obstacles + 7 * d->n_obstacles);
    r->out = d->out_density;
    r->out_on_device = d->out_on_device != 0;
    r->bytes = footprint(d->nx, d->ny, d->nz);
    r->submitted = std::chrono::steady_clock::now();
    s->all.push_back(r);
    if (r->bytes > s->budget) {
        r->state = SMK_REQ_FAILED;
        r->error = SMK_ERR_OOM;
    } else {
        s->queue.push_back(r);
    }
    if (id) *id = r->id;
    return SMK_OK;
}

// A completed server step: its device time is each member's step latency.
static void collect(smk_server* s, TickRec& t) {
    if (!t.pending) return;
    float ms = 0.0f;
    const bool timed = cudaEventElapsedTime(&ms, t.start, t.end) == cudaSuccess;
    for (Request* r : t.members) {
        if (timed) s->latencies_ms.push_back(ms);
        r->steps_done++;
        s->steps_completed++;
        s->cell_updates += (double)r->nx * r->ny * r->nz;
    }
    t.members.clear();
    t.pending = false;
}

// Queueing delay and occupancy bookkeeping of an admission.
static void note_admission(smk_server* s, Request* r) {
    const auto now = std::chrono::steady_clock::now();
    s->queue_ms.push_back(std::chrono::duration<float, std::milli>(now - r->submitted).count());
    s->peak_active = std::max(s->peak_active, (int)s->active.size());
    s->peak_bytes = std::max(s->peak_bytes, s->used);
}

static int admit(smk_server* s, Request* r) {
    int rc = smk_create(r->nx, r->ny, r->nz, &r->params, &r->sim);
    if (rc == SMK_OK) rc = smk_set_graph_loops(r->sim, s->graph_loops);
    if (rc == SMK_OK && !r->mask.empty()) rc = smk_set_solid_mask(r->sim, r->mask.data());
    for (size_t k = 0; rc == SMK_OK && k < r->boxes.size() / 9; ++k) {
        const float* b = &r->boxes[9 * k];
        rc = smk_add_box_emitter(r->sim, (int)b[0], (int)b[1], (int)b[2], (int)b[3], (int)b[4], (int)b[5],
                                 b[6], b[7], b[8] != 0.0f, nullptr);
    }
    for (size_t k = 0; rc == SMK_OK && k < r->spheres.size() / 4; ++k) {
        const float* p = &r->spheres[4 * k];
        rc = smk_add_smoke_source(r->sim, p[0], p[1], p[2], p[3], nullptr);
    }
    for (size_t k = 0; rc == SMK_OK && k < r->obstacles.size() / 7; ++k) {
        const float* o = &r->obstacles[7 * k];
        rc = smk_add_obstacle(r->sim, o[0], o[1], o[2], o[3], o[4], o[5], o[6], nullptr);
    }
    if (rc == SMK_OK && cudaEventCreateWithFlags(&r->retire_ev, cudaEventDisableTiming) != cudaSuccess)
        rc = SMK_ERR_CUDA;
    if (rc == SMK_OK && r->out && !r->out_on_device) {
        // page-lock the caller's buffer so the final copy does not block the host; if that is not
        // possible the copy is made synchronously at retirement
        const size_t bytes = (size_t)r->nx * r->ny * r->nz * sizeof(float);
        r->out_pinned = cudaHostRegister(r->out, bytes, cudaHostRegisterDefault) == cudaSuccess;
        if (!r->out_pinned) cudaGetLastError();
    }
    if (rc == SMK_OK && s->mode == SMK_SERVE_STREAMS) {
        if (cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess) rc = SMK_ERR_CUDA;
        for (int k = 0; rc == SMK_OK && k < 2; ++k)
            if (cudaEventCreate(&r->ev_start[k]) != cudaSuccess || cudaEventCreate(&r->ev_end[k]) != cudaSuccess)
                rc = SMK_ERR_CUDA;
    }
    if (rc == SMK_OK) s->used += r->bytes;
    if (rc != SMK_OK) {
        if (r->sim) {
            smk_destroy(r->sim);
            r->sim = nullptr;
        }
        r->error = rc;
        r->state = SMK_REQ_FAILED;
        release_request(s, r);
        return rc;
    }
    r->state = SMK_REQ_ACTIVE;
    return SMK_OK;
}

// ---- retirement: the final density handoff -----------------------------------------------

static void finish(smk_server* s, Request* r, int rc) {
    r->error = rc;
    r->state = rc == SMK_OK ? SMK_REQ_DONE : SMK_REQ_FAILED;
    s->requests_completed++;
    release_request(s, r);
}

// A request whose last step has completed: its final density goes to the caller's buffer by a
// stream-ordered copy followed by an event, and a later tick releases the request once the
// event has completed, so the host never waits for the copy.  A pageable host buffer that could
// not be page-locked is copied synchronously.  Returns true when the request is finished.
static bool retire(smk_server* s, Request* r, cudaStream_t st) {
    if (!r->retiring) {
        if (!r->out) {
            finish(s, r, check_kernel_error(r->sim));
            return true;
        }
        int rc = smk_read_density(r->sim, r->out, r->out_on_device ? 1 : 0, st);
        const bool async = r->out_on_device || r->out_pinned;
        if (rc == SMK_OK && !async) rc = smk_sync(r->sim, st);
        if (rc == SMK_OK && async && cudaEventRecord(r->retire_ev, st) != cudaSuccess) rc = SMK_ERR_CUDA;
        if (rc != SMK_OK || !async) {
            finish(s, r, rc);
            return true;
        }
        r->retiring = true;
        return false;
    }
    const cudaError_t q = cudaEventQuery(r->retire_ev);
    if (q == cudaErrorNotReady) return false;
    finish(s, r, q == cudaSuccess ? check_kernel_error(r->sim) : SMK_ERR_CUDA);
    return true;
}

// ---- STREAMS form: every request's own step on its own stream ------------------------------

// Collect the latency of a finished step (slot k) of request r.
static void collect_req(smk_server* s, Request* r, int k) {
    if (!r->pending[k]) return;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, r->ev_start[k], r->ev_end[k]) == cudaSuccess) s->latencies_ms.push_back(ms);
    r->pending[k] = false;
    r->steps_done++;
    s->steps_completed++;
    s->cell_updates += (double)r->nx * r->ny * r->nz;
}

static int tick_streams(smk_server* s) {
    // (1) collect finished steps and retire finished requests.  A request keeps at most one
    // step in flight while the next is issued: the step issued two ticks ago is waited for,
    // the one issued last tick is collected if it has already finished.
    std::vector<Request*> still;
    for (Request* r : s->active) {
        bool failed = false;
        const int k_old = (r->steps_issued - 2) & 1;
        if (r->steps_issued >= 2 && r->pending[k_old]) {
            if (cudaEventSynchronize(r->ev_end[k_old]) != cudaSuccess) failed = true;
            else collect_req(s, r, k_old);
        }
        const int k_new = (r->steps_issued - 1) & 1;
        if (!failed && r->steps_issued >= 1 && r->pending[k_new]) {
            const bool last = r->steps_issued >= r->steps;
            const cudaError_t q = last ? cudaEventSynchronize(r->ev_end[k_new]) : cudaEventQuery(r->ev_end[k_new]);
            if (q == cudaSuccess) collect_req(s, r, k_new);
            else if (q != cudaErrorNotReady) failed = true;
        }
        if (failed) {
            r->error = SMK_ERR_CUDA;
            r->state = SMK_REQ_FAILED;
            release_request(s, r);
            continue;
        }
        if (r->cancel && r->steps_done >= r->steps_issued) {
            r->state = SMK_REQ_CANCELLED;
            release_request(s, r);
            continue;
        }
        if (r->steps_done >= r->steps || r->retiring) {
            if (!retire(s, r, r->stream)) still.push_back(r);
        } else {
            still.push_back(r);
        }
    }
    s->active.swap(still);
    // (2) admit in arrival order while memory and slots allow
    while (!s->queue.empty() && (int)s->active.size() < s->max_active &&
           s->used + s->queue.front()->bytes <= s->budget) {
        Request* r = s->queue.front();
        s->queue.pop_front();
        if (admit(s, r) == SMK_OK) {
            s->active.push_back(r);
            note_admission(s, r);
        }
    }
    s->peak_queued = std::max(s->peak_queued, (int)s->queue.size());
    // (3) one step per active request, each on its own stream
    for (Request* r : s->active) {
        if (r->steps_issued >= r->steps || r->cancel) continue;
        const int k = r->steps_issued & 1;
        if (r->pending[k]) {  // its previous use is still in flight (not collected yet)
            if (cudaEventSynchronize(r->ev_end[k]) != cudaSuccess) {
                r->error = SMK_ERR_CUDA;
                r->state = SMK_REQ_FAILED;
                continue;
            }
            collect_req(s, r, k);
        }
        cudaEventRecord(r->ev_start[k], r->stream);
        int rc = smk_step(r->sim, r->dt, r->stream);
        cudaEventRecord(r->ev_end[k], r->stream);
        if (rc != SMK_OK) {
            r->error = rc;
            r->state = SMK_REQ_FAILED;
            continue;
        }
        r->pending[k] = true;
        r->steps_issued++;
    }
    // drop requests that failed while stepping
    std::vector<Request*> ok;
    for (Request* r : s->active) {
        if (r->state == SMK_REQ_FAILED) release_request(s, r);
        else ok.push_back(r);
    }
    s->active.swap(ok);
    return SMK_OK;
}

// ---- GROUPED form: one grouped step over every active request --------------------------------

static int tick_grouped(smk_server* s) {
    // (1) collect completed steps (oldest first); with both slots in flight and nothing else to
    // do, wait for the older one instead of returning to a host that would spin on tick()
    const int older = s->tick_next, newer = s->tick_next ^ 1;
    for (int k : {older, newer}) {
        TickRec& t = s->ticks[k];
        if (!t.pending) continue;
        const cudaError_t q = cudaEventQuery(t.end);
        if (q == cudaSuccess) collect(s, t);
        else if (q != cudaErrorNotReady) return sfail(SMK_ERR_CUDA, std::string("server step: ") + cudaGetErrorString(q));
    }
    bool work = false;
    for (Request* r : s->active) work = work || (r->steps_issued < r->steps && !r->cancel);
    if (!work && s->queue.empty()) {
        for (int k : {older, newer}) {
            TickRec& t = s->ticks[k];
            if (!t.pending) continue;
            if (cudaEventSynchronize(t.end) != cudaSuccess) return sfail(SMK_ERR_CUDA, "server step failed");
            collect(s, t);
        }
    }
    // retire requests whose last step completed
    std::vector<Request*> still;
    for (Request* r : s->active) {
        if (r->cancel && r->steps_done >= r->steps_issued) {
            r->state = SMK_REQ_CANCELLED;
            release_request(s, r);
            continue;
        }
        if (r->steps_done >= r->steps || r->retiring) {
            if (!retire(s, r, s->stream)) still.push_back(r);
        } else {
            still.push_back(r);
        }
    }
    s->active.swap(still);
    // (2) admit in arrival order while memory and slots allow
    while (!s->queue.empty() && (int)s->active.size() < s->max_active &&
           s->used + s->queue.front()->bytes <= s->budget) {
        Request* r = s->queue.front();
        s->queue.pop_front();
        if (admit(s, r) == SMK_OK) {
            s->active.push_back(r);
            note_admission(s, r);
        }
    }
    s->peak_queued = std::max(s->peak_queued, (int)s->queue.size());
    // (3) one grouped step over every active request with steps left (requests whose
    // parameters the grouped kernels do not run, such as the reference projection, step on
    // their own)
    std::vector<smk_sim*> grouped;
    std::vector<float> dts;
    std::vector<Request*> members, single;
    for (Request* r : s->active) {
        if (r->steps_issued >= r->steps || r->cancel) continue;
        members.push_back(r);
        if (group_runner_eligible(r->sim)) {
            grouped.push_back(r->sim);
            dts.push_back(r->dt);
        } else {
            single.push_back(r);
        }
    }
    if (!members.empty()) {
        const int drc = ensure_device_state(s);
        if (drc) return drc;
        TickRec& t = s->ticks[s->tick_next];
        if (t.pending) {  // both slots in flight: the older step must finish first
            if (cudaEventSynchronize(t.end) != cudaSuccess) return sfail(SMK_ERR_CUDA, "server step failed");
            collect(s, t);
        }
        cudaEventRecord(t.start, s->stream);
        int rc = group_runner_step(s->runner, grouped.data(), dts.data(), (int)grouped.size(), s->sched,
                                   s->stream, nullptr);
        for (size_t k = 0; rc == SMK_OK && k < single.size(); ++k) rc = smk_step(single[k]->sim, single[k]->dt, s->stream);
        cudaEventRecord(t.end, s->stream);
        if (rc != SMK_OK) {
            // the step's members cannot continue: report and release them
            cudaStreamSynchronize(s->stream);
            std::vector<Request*> ok;
            for (Request* r : s->active) {
                if (std::find(members.begin(), members.end(), r) != members.end()) {
                    r->error = rc;
                    r->state = SMK_REQ_FAILED;
                    release_request(s, r);
                } else {
                    ok.push_back(r);
                }
            }
            s->active.swap(ok);
        } else {
            for (Request* r : members) r->steps_issued++;
            t.members = members;
            t.pending = true;
            s->tick_next ^= 1;
        }
    }
    return SMK_OK;
}

int smk_server_tick(smk_server* s, int* n_active, int* n_queued) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    DeviceGuard dg(s->device);
    if (!s->queue.empty()) s->started = true;
    const int rc = s->mode == SMK_SERVE_GROUPED ? tick_grouped(s) : tick_streams(s);
    if (n_active) *n_active = (int)s->active.size();
    if (n_queued) *n_queued = (int)s->queue.size();
    return rc;
}

int smk_server_request_status(smk_server* s, int id, int* state, int* steps_done, int* error) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    for (Request* r : s->all) {
        if (r->id == id) {
            if (state) *state = r->state;
            if (steps_done) *steps_done = r->steps_done;
            if (error) *error = r->error;
            return SMK_OK;
        }
    }
    return sfail(SMK_ERR_INVALID, "unknown request id");
}

int smk_server_get_stats(smk_server* s, smk_server_stats* out) {
    if (!s || !out) return sfail(SMK_ERR_INVALID, "null argument");
    memset(out, 0, sizeof(*out));
    out->steps_completed = s->steps_completed;
    out->requests_completed = s->requests_completed;
    out->cell_updates = s->cell_updates;
    out->active = (int)s->active.size();
    out->queued = (int)s->queue.size();
    out->bytes_in_use = s->used;
    auto pct = [](std::vector<float> v, double q) {
        size_t i = (size_t)std::min<double>((double)v.size() - 1, q * (double)(v.size() - 1) + 0.5);
        std::nth_element(v.begin(), v.begin() + i, v.end());
        return v[i];
    };
    if (!s->latencies_ms.empty()) {
        out->p50_step_ms = pct(s->latencies_ms, 0.50);
        out->p99_step_ms = pct(s->latencies_ms, 0.99);
        out->max_step_ms = *std::max_element(s->latencies_ms.begin(), s->latencies_ms.end());
    }
    if (!s->queue_ms.empty()) {
        out->p50_queue_ms = pct(s->queue_ms, 0.50);
        out->p99_queue_ms = pct(s->queue_ms, 0.99);
        out->max_queue_ms = *std::max_element(s->queue_ms.begin(), s->queue_ms.end());
    }
    out->peak_active = s->peak_active;
    out->peak_queued = s->peak_queued;
    out->peak_bytes = s->peak_bytes;
    return SMK_OK;
}

}  // extern "C"
