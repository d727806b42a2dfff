// af_serve.cu -- continuous-batching request loop over a Batch.
//
// Requests (a MIXED config, a step count, a seed) queue in arrival order.
// Each round admits queued requests while a slot and enough of the device
// budget are free -- their state is created and stays resident on the
// device -- then advances every resident request by the same number of
// Steps in one batched graph launch, and retires the ones that finished:
// their max|div| is read back as the result and their slot and memory go to
// the next requests.  Requests that arrive while others are on the GPU join
// at the next round; a request's bits do not depend on what else is resident.
#include "../../include/aeroflux_cuda.h"
#include "af_batch.h"
#include "af_internal.h"

#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <string>
#include <vector>

namespace {

struct Req {
    int64_t id = 0;
    af_config cfg{};
    int64_t steps = 0, done = 0;
    uint64_t seed = 0;
    double arrival = 0, admitted = 0, completed = 0;
    size_t bytes = 0;
    int slot = -1;
    int status = AF_OK;
    double max_div = 0;
    int64_t passes = 0;
    std::string msg;
};

}  // namespace

struct af_server {
    af::Batch* b = nullptr;
    int device = 0;
    size_t budget = 0, used = 0;
    int max_slots = 0;
    int64_t max_resident_cells = 0;  // admission work target (0: none)
    int64_t resident_cells = 0;
    int max_round_steps = 1;
    bool retain = false;
    std::deque<Req> queue;
    std::vector<Req> resident;
    std::vector<Req> done;
    std::vector<Req> retained;
    int64_t next_id = 1;
    int64_t executed_cell_steps = 0;
    std::chrono::steady_clock::time_point t0;
    unsigned long long* mx = nullptr;
    std::string err;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

std::string normalize_copy(af_config* c, af_server* s) {
    char buf[512] = {0};
    if (af_config_normalize(c, buf, sizeof buf) != AF_OK) return buf;
    if (c->precision != AF_PRECISION_MIXED) return "aeroflux: the server steps the mixed-precision form only";
    (void)s;
    return "";
}

int fail(af_server* s, int code, const std::string& m) {
    s->err = m;
    return code;
}

double max_div_of(af_server* s, int slot, const af_config& c) {
    double *u, *v, *w;
    af::batch_field(s->b, slot, AF_FIELD_U, &u);
    af::batch_field(s->b, slot, AF_FIELD_V, &v);
    af::batch_field(s->b, slot, AF_FIELD_W, &w);
    cudaStream_t st = af::batch_stream(s->b);
    cudaMemsetAsync(s->mx, 0, sizeof *s->mx, st);
    af::launch_max_divergence(af::batch_geom(s->b, slot), u, v, w, 1.0 / c.h, s->mx, st);
    unsigned long long bits = 0;
    cudaMemcpyAsync(&bits, s->mx, sizeof bits, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    double d;
    memcpy(&d, &bits, sizeof d);
    return d;
}

}  // namespace

extern "C" {

int af_server_create(int64_t budget_bytes, int64_t max_slots, int64_t max_resident_cells, int32_t device,
                     int32_t max_round_steps, int32_t retain, af_server** out, char* err, size_t errlen) {
    if (!out || budget_bytes <= 0 || max_slots < 1 || max_resident_cells < 0 || device < 0 || max_round_steps < 1)
        return AF_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) {
        if (err && errlen) snprintf(err, errlen, "aeroflux: cuda: no such device");
        return AF_ERR_CUDA;
    }
    std::string m;
    af::Batch* b = af::batch_create((int)max_slots, (size_t)budget_bytes, &m);
    if (!b) {
        if (err && errlen) snprintf(err, errlen, "%s", m.c_str());
        return AF_ERR_NOMEM;
    }
    af_server* s = new af_server();
    s->b = b;
    s->device = device;
    s->budget = (size_t)budget_bytes;
    s->max_slots = (int)max_slots;
    s->max_resident_cells = max_resident_cells;
    s->max_round_steps = max_round_steps;
    s->retain = retain != 0;
    s->t0 = std::chrono::steady_clock::now();
    if (cudaMalloc(&s->mx, sizeof *s->mx) != cudaSuccess) {
        af::batch_destroy(b);
        delete s;
        if (err && errlen) snprintf(err, errlen, "aeroflux: cuda: server result word");
        return AF_ERR_NOMEM;
    }
    *out = s;
    return AF_OK;
}

int af_server_now(af_server* s, double* seconds) {
    if (!s || !seconds) return AF_ERR_ARG;
    *seconds = s->now();
    return AF_OK;
}

int af_server_submit(af_server* s, const af_config* cfg, int64_t steps, uint64_t seed, double arrival_s, int64_t* id) {
    if (!s || !cfg || !id || steps < 1) return AF_ERR_ARG;
    Req r;
    r.cfg = *cfg;
    std::string m = normalize_copy(&r.cfg, s);
    if (!m.empty()) return fail(s, AF_ERR_CONFIG, m);
    r.bytes = af::batch_slot_bytes(r.cfg);
    if (r.bytes > s->budget) return fail(s, AF_ERR_NOMEM, "aeroflux: request exceeds the server's device budget");
    r.id = s->next_id++;
    r.steps = steps;
    r.seed = seed;
    r.arrival = arrival_s < 0 ? s->now() : arrival_s;
    s->queue.push_back(r);
    *id = r.id;
    return AF_OK;
}

// One round: admit, step every resident request, retire the finished ones.
int af_server_round(af_server* s, int64_t* completed_now, int64_t* resident, int64_t* queued) {
    if (!s) return AF_ERR_ARG;
    cudaSetDevice(s->device);
    int64_t fin = 0;
    // Admission in arrival order: the head waits until it fits (no overtaking)
    // in the slots, the device budget and the resident-work target (one
    // request is always admitted when none is running).
    bool admitted_any = false;
    auto cells = [](const Req& r) { return r.cfg.nx * r.cfg.ny * r.cfg.nz; };
    while (!s->queue.empty() && (int)(s->resident.size() + s->retained.size()) < s->max_slots &&
           s->used + s->queue.front().bytes <= s->budget &&
           (s->max_resident_cells == 0 || s->resident.empty() ||
            s->resident_cells + cells(s->queue.front()) <= s->max_resident_cells)) {
        Req r = s->queue.front();
        std::string m;
        const int slot = af::batch_assign(s->b, r.cfg, nullptr, &m);
        if (slot < 0) break;  // pool fragmentation: wait for a release
        s->queue.pop_front();
        r.slot = slot;
        af::batch_seed(s->b, slot, 1.0, 0.01, r.seed, (uint64_t)r.id);
        r.admitted = s->now();
        s->used += r.bytes;
        s->resident_cells += cells(r);
        s->resident.push_back(r);
        admitted_any = true;
    }
    if (admitted_any) {
        // applyVelocityBC is idempotent on requests already stepping.
        cudaError_t rc = af::batch_velocity_bc(s->b);
        if (rc != cudaSuccess) return fail(s, AF_ERR_CUDA, cudaGetErrorString(rc));
    }
    if (!s->resident.empty()) {
        // A round runs up to max_round_steps Steps; a request with fewer left
        // stops after its last one (the batch skips it for the rest of the
        // round), so one request close to done does not shorten the round.
        int64_t k = 0;
        for (const Req& r : s->resident) k = std::max<int64_t>(k, r.steps - r.done);
        k = std::min<int64_t>(k, s->max_round_steps);
        std::vector<int64_t> stop_at(s->max_slots + 1, 0);
        for (const Req& r : s->resident)
            if (r.steps - r.done < k && r.slot < (int)stop_at.size()) stop_at[r.slot] = r.steps - r.done;
        std::string m;
        cudaError_t rc = af::batch_step(s->b, k, &m, &stop_at);
        if (rc != cudaSuccess) return fail(s, AF_ERR_CUDA, m);
        cudaStreamSynchronize(af::batch_stream(s->b));
        if (af::debug_bounds_error(&m)) return fail(s, AF_ERR_CUDA, m);
        if (af::batch_device_error(s->b, &m)) return fail(s, AF_ERR_CUDA, m);
        int first = -1;
        af::batch_collect_faults(s->b, &m, &first);
        const double t = s->now();
        std::vector<Req> keep;
        for (Req& r : s->resident) {
            const int64_t ran = std::min<int64_t>(k, r.steps - r.done);
            r.done += ran;
            s->executed_cell_steps += r.cfg.nx * r.cfg.ny * r.cfg.nz * ran;
            std::string fm;
            const bool faulted = af::batch_slot_faulted(s->b, r.slot, &fm);
            if (faulted || r.done >= r.steps) {
                r.status = faulted ? AF_ERR_FAULT : AF_OK;
                r.msg = fm;
                r.max_div = max_div_of(s, r.slot, r.cfg);
                double est;
                af::batch_slot_projection(s->b, r.slot, &r.passes, &est);
                r.completed = t;
                ++fin;
                s->resident_cells -= cells(r);
                if (s->retain) {
                    af::batch_set_active(s->b, r.slot, false);
                    s->retained.push_back(r);
                } else {
                    af::batch_release(s->b, r.slot);
                    s->used -= r.bytes;
                }
                s->done.push_back(r);
            } else {
                keep.push_back(r);
            }
        }
        s->resident.swap(keep);
    }
    if (completed_now) *completed_now = fin;
    if (resident) *resident = (int64_t)s->resident.size();
    if (queued) *queued = (int64_t)s->queue.size();
    return AF_OK;
}

int af_server_results(af_server* s, af_request_result* out, int64_t cap, int64_t* n) {
    if (!s || !n || (cap > 0 && !out)) return AF_ERR_ARG;
    const int64_t k = std::min<int64_t>(cap, (int64_t)s->done.size());
    for (int64_t i = 0; i < k; ++i) {
        const Req& r = s->done[i];
        af_request_result& o = out[i];
        o.id = r.id;
        o.status = r.status;
        o.reserved = 0;
        o.cells = r.cfg.nx * r.cfg.ny * r.cfg.nz;
        o.steps = r.done;
        o.refinement_passes = r.passes;
        o.arrival_s = r.arrival;
        o.admitted_s = r.admitted;
        o.completed_s = r.completed;
        o.max_divergence = r.max_div;
    }
    s->done.erase(s->done.begin(), s->done.begin() + k);
    *n = k;
    return AF_OK;
}

int af_server_download(af_server* s, int64_t id, int field, double* host, size_t count) {
    if (!s || !host || field < 0 || field > 7) return AF_ERR_ARG;
    for (const Req& r : s->retained) {
        if (r.id != id) continue;
        cudaSetDevice(s->device);
        double* dev = nullptr;
        const af_field_desc d = af::batch_field(s->b, r.slot, field, &dev);
        if ((int64_t)count != d.count) return fail(s, AF_ERR_ARG, "aeroflux: field size mismatch");
        cudaStream_t st = af::batch_stream(s->b);
        cudaMemcpyAsync(host, dev, count * 8, cudaMemcpyDeviceToHost, st);
        return cudaStreamSynchronize(st) == cudaSuccess ? AF_OK : fail(s, AF_ERR_CUDA, "aeroflux: cuda: download");
    }
    return fail(s, AF_ERR_ARG, "aeroflux: no retained result with that id");
}

int af_server_release(af_server* s, int64_t id) {
    if (!s) return AF_ERR_ARG;
    for (size_t i = 0; i < s->retained.size(); ++i) {
        if (s->retained[i].id != id) continue;
        cudaSetDevice(s->device);
        af::batch_release(s->b, s->retained[i].slot);
        s->used -= s->retained[i].bytes;
        s->retained.erase(s->retained.begin() + (long)i);
        return AF_OK;
    }
    return fail(s, AF_ERR_ARG, "aeroflux: no retained result with that id");
}

int af_server_cancel_queued(af_server* s, int64_t* cancelled) {
    if (!s) return AF_ERR_ARG;
    if (cancelled) *cancelled = (int64_t)s->queue.size();
    s->queue.clear();
    return AF_OK;
}

int af_server_get_stats(af_server* s, af_server_stats* out) {
    if (!s || !out) return AF_ERR_ARG;
    out->queued = (int64_t)s->queue.size();
    out->resident = (int64_t)s->resident.size();
    out->retained = (int64_t)s->retained.size();
    out->budget_bytes = (int64_t)s->budget;
    out->used_bytes = (int64_t)s->used;
    out->executed_cell_steps = s->executed_cell_steps;
    out->now_s = s->now();
    return AF_OK;
}

int af_server_tune(af_server* s, int32_t reps, char* report, size_t len) {
    if (!s || reps < 1) return AF_ERR_ARG;
    cudaSetDevice(s->device);
    const std::string r = af::batch_tune(s->b, reps);
    if (report && len) snprintf(report, len, "%s", r.c_str());
    return AF_OK;
}

void af_server_destroy(af_server* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    af::batch_destroy(s->b);
    cudaFree(s->mx);
    delete s;
}

const char* af_server_last_error(const af_server* s) { return s ? s->err.c_str() : ""; }

}  // extern "C"
