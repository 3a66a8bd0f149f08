// Continuous-batching serving loop for smoke simulations (smk_server_*).
//
// The reference runs one simulation per process, stepped from the render loop at 20 Hz
// (project/main.cpp:93, :889-896).  A server instead keeps many simulations resident on one GPU
// and admits new ones while others run:
//   - submit() queues a request (grid size, step count, scene, parameters);
//   - tick() (1) retires requests whose last step has completed: their density is copied to the
//     caller's host buffer and their device memory is freed; (2) admits queued requests in
//     arrival order while the device-memory budget and the slot limit allow; (3) issues one step
//     for every active request, each on its own stream, so the work of different requests
//     overlaps on the device;
//   - every issued step is bracketed by CUDA events on its stream; its latency (device time from
//     the step's first kernel being ready to its last kernel finishing, including time shared
//     with other requests) is collected for p50/p99.
// Each request is an independent simulation with its own buffers, so its results do not depend
// on what else is resident (tested: alone vs in the mix).  Host-side failures (a request that
// does not fit the budget at all, allocation failure, invalid input) are reported per request.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "../../include/smoke_gb300.h"
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
    float* out = nullptr;                          // caller's host buffer for the final density
    int state = SMK_REQ_QUEUED;
    int steps_issued = 0;
    int steps_done = 0;
    int error = SMK_OK;
    size_t bytes = 0;
    smk_sim* sim = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start[2] = {nullptr, nullptr};
    cudaEvent_t ev_end[2] = {nullptr, nullptr};
    bool pending[2] = {false, false};
    double admit_time = 0.0;
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
    double cell_updates = 0.0;
    long long steps_completed = 0;
    int requests_completed = 0;
};

extern "C" {

const char* smk_server_last_error(void) { return g_srv_err.c_str(); }

int smk_server_create(size_t budget_bytes, int max_active, smk_server** out) {
    if (!out || budget_bytes == 0 || max_active < 1) return sfail(SMK_ERR_INVALID, "bad server limits");
    smk_server* s = new smk_server();
    s->budget = budget_bytes;
    s->max_active = max_active;
    cudaGetDevice(&s->device);
    *out = s;
    return SMK_OK;
}

static void release_request(smk_server* s, Request* r) {
    if (r->sim) {
        smk_destroy(r->sim);
        r->sim = nullptr;
        s->used -= r->bytes;
    }
    for (int k = 0; k < 2; ++k) {
        if (r->ev_start[k]) cudaEventDestroy(r->ev_start[k]);
        if (r->ev_end[k]) cudaEventDestroy(r->ev_end[k]);
        r->ev_start[k] = r->ev_end[k] = nullptr;
    }
    if (r->stream) cudaStreamDestroy(r->stream);
    r->stream = nullptr;
}

int smk_server_destroy(smk_server* s) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    cudaDeviceSynchronize();
    for (Request* r : s->all) {
        release_request(s, r);
        delete r;
    }
    delete s;
    return SMK_OK;
}

int smk_server_submit(smk_server* s, const smk_request_desc* d, int* id) {
    if (!s || !d) return sfail(SMK_ERR_INVALID, "null argument");
    if (d->nx < 3 || d->ny < 3 || d->nz < 3 || d->steps < 1 || !(d->dt > 0.0f))
        return sfail(SMK_ERR_INVALID, "request needs a grid of at least 3^3 cells, steps >= 1, dt > 0");
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
    r->bytes = footprint(d->nx, d->ny, d->nz);
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

// Collect the latency of a finished step (slot k) of request r.
static void collect(smk_server* s, Request* r, int k) {
    if (!r->pending[k]) return;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, r->ev_start[k], r->ev_end[k]) == cudaSuccess) s->latencies_ms.push_back(ms);
    r->pending[k] = false;
    r->steps_done++;
    s->steps_completed++;
    s->cell_updates += (double)r->nx * r->ny * r->nz;
}

static int admit(smk_server* s, Request* r) {
    int rc = smk_create(r->nx, r->ny, r->nz, &r->params, &r->sim);
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
    if (rc == SMK_OK && cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = SMK_ERR_CUDA;
    for (int k = 0; rc == SMK_OK && k < 2; ++k) {
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

int smk_server_tick(smk_server* s, int* n_active, int* n_queued) {
    if (!s) return sfail(SMK_ERR_INVALID, "server is null");
    // (1) collect finished steps and retire finished requests.  A request keeps at most one
    // step in flight while the next is issued: the step issued two ticks ago is waited for,
    // the one issued last tick is collected if it has already finished.
    std::vector<Request*> still;
    for (Request* r : s->active) {
        bool failed = false;
        const int k_old = (r->steps_issued - 2) & 1;
        if (r->steps_issued >= 2 && r->pending[k_old]) {
            if (cudaEventSynchronize(r->ev_end[k_old]) != cudaSuccess) failed = true;
            else collect(s, r, k_old);
        }
        const int k_new = (r->steps_issued - 1) & 1;
        if (!failed && r->steps_issued >= 1 && r->pending[k_new]) {
            const bool last = r->steps_issued >= r->steps;
            const cudaError_t q = last ? cudaEventSynchronize(r->ev_end[k_new]) : cudaEventQuery(r->ev_end[k_new]);
            if (q == cudaSuccess) collect(s, r, k_new);
            else if (q != cudaErrorNotReady) failed = true;
        }
        if (failed) {
            r->error = SMK_ERR_CUDA;
            r->state = SMK_REQ_FAILED;
            release_request(s, r);
            continue;
        }
        if (r->steps_done >= r->steps) {
            int rc = SMK_OK;
            if (r->out) {
                rc = smk_read_density(r->sim, r->out, 0, r->stream);
                if (rc == SMK_OK) rc = smk_sync(r->sim, r->stream);
            }
            r->error = rc;
            r->state = rc == SMK_OK ? SMK_REQ_DONE : SMK_REQ_FAILED;
            s->requests_completed++;
            release_request(s, r);
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
        if (admit(s, r) == SMK_OK) s->active.push_back(r);
    }
    // (3) one step per active request, each on its own stream
    for (Request* r : s->active) {
        if (r->steps_issued >= r->steps) continue;
        const int k = r->steps_issued & 1;
        if (r->pending[k]) {  // its previous use is still in flight (not collected yet)
            if (cudaEventSynchronize(r->ev_end[k]) != cudaSuccess) {
                r->error = SMK_ERR_CUDA;
                r->state = SMK_REQ_FAILED;
                continue;
            }
            collect(s, r, k);
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
    if (n_active) *n_active = (int)s->active.size();
    if (n_queued) *n_queued = (int)s->queue.size();
    return SMK_OK;
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
    if (!s->latencies_ms.empty()) {
        std::vector<float> v = s->latencies_ms;
        auto pct = [&v](double q) {
            size_t i = (size_t)std::min<double>((double)v.size() - 1, q * (double)(v.size() - 1) + 0.5);
            std::nth_element(v.begin(), v.begin() + i, v.end());
            return v[i];
        };
        out->p50_step_ms = pct(0.50);
        out->p99_step_ms = pct(0.99);
        out->max_step_ms = *std::max_element(v.begin(), v.end());
    }
    return SMK_OK;
}

}  // extern "C"
