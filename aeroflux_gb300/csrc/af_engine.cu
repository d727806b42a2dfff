// af_engine.cu -- the C ABI of libaeroflux_cuda (include/aeroflux_cuda.h):
// configuration, engine lifecycle, field transfer, and the Step driver.
//
// A Step is one CUDA graph: the reference's 6 + 2*(2 + 2*GaussSeidelIters)
// dispatches (layout.go:15-25) plus the boundary-condition passes become
// kernel nodes on the engine's stream, captured once per descriptor parity
// and replayed.  Nothing is allocated per step (engine_test.go:271-288 pins
// zero allocations per Step in the reference).
#include "../../include/aeroflux_cuda.h"
#include "af_debug.cuh"
#include "af_internal.h"
#include "af_batch.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <sched.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <thread>
#include <vector>

using af::Dims;
using af::Fields;
using af::Geom;
using af::Status;

namespace {

constexpr int64_t kCacheLine = 128;  // layout.go:13

// strconv.FormatFloat(v, 'g', -1, 64): fmt's %v and %g for a float64.
std::string go_float(double v) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "+Inf" : "-Inf";
    char buf[64];
    for (int nd = 1; nd <= 17; ++nd) {
        snprintf(buf, sizeof buf, "%.*e", nd - 1, v);
        if (strtod(buf, nullptr) == v) break;
    }
    const char* p = buf;
    bool neg = false;
    if (*p == '-') { neg = true; ++p; }
    std::string digs;
    for (; *p && *p != 'e'; ++p)
        if (*p >= '0' && *p <= '9') digs.push_back(*p);
    int exp10 = atoi(p + 1);
    while (digs.size() > 1 && digs.back() == '0') digs.pop_back();
    if (v == 0) { digs = "0"; exp10 = 0; }
    std::string out = neg ? "-" : "";
    const int n = (int)digs.size();
    if (exp10 < -4 || exp10 >= 6) {  // shortest 'g' switches to %e at exponent 6
        out += digs[0];
        if (n > 1) out += "." + digs.substr(1);
        char e[16];
        snprintf(e, sizeof e, "e%c%02d", exp10 < 0 ? '-' : '+', exp10 < 0 ? -exp10 : exp10);
        out += e;
    } else if (exp10 < 0) {
        out += "0." + std::string(-exp10 - 1, '0') + digs;
    } else {
        const int dp = exp10 + 1;
        for (int i = 0; i < dp; ++i) out += i < n ? digs[i] : '0';
        if (n > dp) out += "." + digs.substr(dp);
    }
    return out;
}

std::string sfmt(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return buf;
}

void put_err(char* err, size_t errlen, const std::string& m) {
    if (err && errlen) snprintf(err, errlen, "%s", m.c_str());
}

// (*Config).Normalize, aeroflux.go:47-113.  Empty string on success.
std::string normalize(af_config* c) {
    if (c->nx <= 0 || c->ny <= 0 || c->nz <= 0)
        return sfmt("aeroflux: interior extents must be positive, got %lldx%lldx%lld", (long long)c->nx,
                    (long long)c->ny, (long long)c->nz);
    if (c->ghost == 0) c->ghost = 1;
    if (c->ghost < 1) return sfmt("aeroflux: ghost thickness must be >= 1, got %lld", (long long)c->ghost);
    if (c->h == 0) c->h = 1.0 / (double)std::max(c->nx, std::max(c->ny, c->nz));
    if (c->h <= 0 || std::isnan(c->h) || std::isinf(c->h))
        return "aeroflux: cell size must be finite and positive, got " + go_float(c->h);
    if (c->density == 0) c->density = 1.0;
    if (c->density <= 0 || std::isnan(c->density) || std::isinf(c->density))
        return "aeroflux: density must be finite and positive, got " + go_float(c->density);
    if (c->viscosity < 0 || std::isnan(c->viscosity) || std::isinf(c->viscosity))
        return "aeroflux: viscosity must be finite and non-negative, got " + go_float(c->viscosity);
    if (c->dt == 0) {
        if (c->viscosity > 0) c->dt = 0.5 * c->h * c->h / (6 * c->viscosity);
        else c->dt = 0.25 * c->h;
    }
    if (c->dt <= 0 || std::isnan(c->dt) || std::isinf(c->dt))
        return "aeroflux: timestep must be finite and positive, got " + go_float(c->dt);
    if (c->workers == 0) {
        // runtime.GOMAXPROCS(0): the CPUs this process may run on.
        cpu_set_t set;
        c->workers = sched_getaffinity(0, sizeof set, &set) == 0
                         ? CPU_COUNT(&set)
                         : (int64_t)std::max(1u, std::thread::hardware_concurrency());
    }
    if (c->workers < 1) return sfmt("aeroflux: worker count must be >= 1, got %lld", (long long)c->workers);
    if (c->workers > c->nz) c->workers = c->nz;
    if (c->gauss_seidel_iters == 0) c->gauss_seidel_iters = 24;
    if (c->gauss_seidel_iters < 1)
        return sfmt("aeroflux: gauss-seidel iterations must be >= 1, got %lld", (long long)c->gauss_seidel_iters);
    if (c->viscosity > 0) {
        const double limit = c->h * c->h / (6 * c->viscosity);
        if (c->dt > limit)
            return "aeroflux: dt " + go_float(c->dt) + " exceeds explicit diffusion stability limit " +
                   go_float(limit) + " (h=" + go_float(c->h) + ", nu=" + go_float(c->viscosity) +
                   "); reduce dt or h";
    }
    // Extensions.
    if (c->precision != AF_PRECISION_FP64 && c->precision != AF_PRECISION_MIXED)
        return sfmt("aeroflux: unknown precision form %d", (int)c->precision);
    if (c->div_tol == 0) c->div_tol = 1e-10;
    if (!(c->div_tol > 0) || std::isinf(c->div_tol))
        return "aeroflux: divergence tolerance must be finite and positive, got " + go_float(c->div_tol);
    if (c->inner_sweeps == 0) c->inner_sweeps = 2;
    if (c->inner_sweeps < 1) return sfmt("aeroflux: inner sweeps must be >= 1, got %lld", (long long)c->inner_sweeps);
    if (c->device < 0) return sfmt("aeroflux: device ordinal must be >= 0, got %d", (int)c->device);
    if (c->max_refine == 0) c->max_refine = 30;
    if (c->max_refine < 1) return sfmt("aeroflux: refinement cap must be >= 1, got %lld", (long long)c->max_refine);
    return "";
}

af_field_desc field_layout(int64_t* off, int64_t nx, int64_t ny, int64_t nz) {
    af_field_desc f;
    f.off = *off;
    f.nx = nx;
    f.ny = ny;
    f.nz = nz;
    f.sy = nx;
    f.sz = nx * ny;
    f.count = nx * ny * nz;
    int64_t sz = f.count * 8;
    if (int64_t r = sz % kCacheLine) sz += kCacheLine - r;
    *off += sz;
    return f;
}

// NewMAC layout, grid.go:101-134.
int64_t mac_layout(int64_t nx, int64_t ny, int64_t nz, int64_t g, af_field_desc f[8]) {
    const int64_t cx = nx + 2 * g, cy = ny + 2 * g, cz = nz + 2 * g;
    int64_t off = 0;
    f[AF_FIELD_P] = field_layout(&off, cx, cy, cz);
    f[AF_FIELD_U] = field_layout(&off, cx + 1, cy, cz);
    f[AF_FIELD_V] = field_layout(&off, cx, cy + 1, cz);
    f[AF_FIELD_W] = field_layout(&off, cx, cy, cz + 1);
    f[AF_FIELD_DIV] = field_layout(&off, cx, cy, cz);
    f[AF_FIELD_TMP0] = field_layout(&off, cx + 1, cy, cz);
    f[AF_FIELD_TMP1] = field_layout(&off, cx, cy + 1, cz);
    f[AF_FIELD_TMP2] = field_layout(&off, cx, cy, cz + 1);
    return off;
}

Dims to_dims(const af_field_desc& d) {
    Dims r;
    r.nx = (int)d.nx;
    r.ny = (int)d.ny;
    r.nz = (int)d.nz;
    r.sy = d.sy;
    r.sz = d.sz;
    r.count = d.count;
    return r;
}

constexpr int kEvStart = 0, kEvEnd = 1, kEvSweep = 2 /* 2 per sweep */, kEvRb = 14 /* 2 per projection */;
constexpr int kNumEvents = 18;

constexpr int kFwd[3] = {0, 1, 2};  // aeroflux.go:373
constexpr int kRev[3] = {2, 1, 0};  // aeroflux.go:390

}  // namespace

struct af_engine {
    af_config cfg{};
    Geom geom{};
    af_field_desc desc[8]{};  // layout slots (never swapped)
    int parity = 0;           // 1 when U/V/W live in the Tmp slots (after a faulted step)
    int64_t bytes = 0;
    char* arena = nullptr;
    double* b = nullptr;      // h2*Div (P-shaped), FP64 form
    Status* st = nullptr;
    double* partials = nullptr;
    double* sum = nullptr;
    unsigned long long* mx = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    af::Batch* batch = nullptr;  // MIXED form: a batch of one over this arena
    // FP64 form with the multigrid projection option: a batch of one over
    // this arena supplies the projection; `st` then points at its status
    // word and `own_st` keeps the engine's own for release.
    af::Batch* mg = nullptr;
    Status* own_st = nullptr;
    // Advection scheme (af_advection); MacCormack keeps its forward step in
    // three face fields shaped like U, V, W.
    int advection = AF_ADVECTION_SEMI_LAGRANGIAN;
    char* mc_scratch = nullptr;
    // Profiling: event nodes at the step's ends, around each sweep and around
    // each projection's red-black loop.
    bool profiling = false;
    cudaEvent_t ev[kNumEvents] = {};
    int64_t launches_per_step = 0;
    int64_t rbgs_launches_per_step = 0;
    bool closed = false;
    std::string err;

    double* slot(int id) const { return (double*)(arena + desc[id].off); }
    // Current descriptor and device pointer of field id.
    af_field_desc current(int id, double** dev) const {
        if (batch) return af::batch_field(batch, 0, id, dev);
        const int c = cur(id);
        if (dev) *dev = slot(c);
        return desc[c];
    }
    // Current descriptor slot of field id (commitVelocity swaps U/V/W with Tmp0..2).
    int cur(int id) const {
        if (!parity) return id;
        switch (id) {
        case AF_FIELD_U: return AF_FIELD_TMP0;
        case AF_FIELD_V: return AF_FIELD_TMP1;
        case AF_FIELD_W: return AF_FIELD_TMP2;
        case AF_FIELD_TMP0: return AF_FIELD_U;
        case AF_FIELD_TMP1: return AF_FIELD_V;
        case AF_FIELD_TMP2: return AF_FIELD_W;
        default: return id;
        }
    }
    Fields fields() const {
        Fields f;
        if (batch) {
            af::batch_field(batch, 0, AF_FIELD_P, &f.p);
            af::batch_field(batch, 0, AF_FIELD_U, &f.u);
            af::batch_field(batch, 0, AF_FIELD_V, &f.v);
            af::batch_field(batch, 0, AF_FIELD_W, &f.w);
            af::batch_field(batch, 0, AF_FIELD_DIV, &f.div);
            af::batch_field(batch, 0, AF_FIELD_TMP0, &f.t0);
            af::batch_field(batch, 0, AF_FIELD_TMP1, &f.t1);
            af::batch_field(batch, 0, AF_FIELD_TMP2, &f.t2);
            return f;
        }
        f.p = slot(AF_FIELD_P);
        f.u = slot(cur(AF_FIELD_U));
        f.v = slot(cur(AF_FIELD_V));
        f.w = slot(cur(AF_FIELD_W));
        f.div = slot(AF_FIELD_DIV);
        f.t0 = slot(cur(AF_FIELD_TMP0));
        f.t1 = slot(cur(AF_FIELD_TMP1));
        f.t2 = slot(cur(AF_FIELD_TMP2));
        return f;
    }
};

namespace {

int cuda_fail(af_engine* e, cudaError_t rc, const char* what) {
    e->err = sfmt("aeroflux: cuda: %s: %s", what, cudaGetErrorString(rc));
    return AF_ERR_CUDA;
}

#define AF_CUDA(e, call)                                   \
    do {                                                   \
        cudaError_t rc__ = (call);                         \
        if (rc__ != cudaSuccess) return cuda_fail(e, rc__, #call); \
    } while (0)

int check_open(af_engine* e) {
    if (!e) return AF_ERR_ARG;
    if (e->closed) {
        e->err = "aeroflux: engine is closed";
        return AF_ERR_CLOSED;
    }
    // The calling thread may have another device current.
    AF_CUDA(e, cudaSetDevice(e->cfg.device));
    return AF_OK;
}

int reset_status(af_engine* e) {
    const Status s{af::kNoFault, 0u, af::kNoKey};
    AF_CUDA(e, cudaMemcpyAsync(e->st, &s, sizeof s, cudaMemcpyHostToDevice, e->stream));
    return AF_OK;
}

void rec(af_engine* e, int idx) {
    if (e->profiling) cudaEventRecordWithFlags(e->ev[idx], e->stream, cudaEventRecordExternal);
}

void swap_fields(Fields& f) {
    std::swap(f.u, f.t0);
    std::swap(f.v, f.t1);
    std::swap(f.w, f.t2);
}

// project, project.go:12-34, FP64 plain form.
void enqueue_project_fp64(af_engine* e, const Fields& f, int gate) {
    const Geom& g = e->geom;
    const af_config& c = e->cfg;
    cudaStream_t s = e->stream;
    af::launch_velocity_bc(g, f.u, f.v, f.w, e->st, gate, s);
    const double scale = c.density / (c.dt * c.h);  // project.go:49
    const double h2 = c.h * c.h;                    // project.go:107
    af::launch_divergence_fp64(g, f, e->b, scale, h2, true, e->st, gate, s);
    rec(e, kEvRb + (gate == 3 ? 0 : 2));
    for (int64_t it = 0; it < c.gauss_seidel_iters; ++it) {
        af::launch_rbgs_fp64(g, f.p, e->b, 0, e->st, gate, s);
        af::launch_rbgs_fp64(g, f.p, e->b, 1, e->st, gate, s);
    }
    rec(e, kEvRb + (gate == 3 ? 1 : 3));
    e->launches_per_step += 5 + 2 * c.gauss_seidel_iters;
    e->rbgs_launches_per_step += 2 * c.gauss_seidel_iters;
    af::launch_pressure_bc_fp64(g, f.p, e->st, gate, s);
    af::launch_gradient_fp64(g, f, c.dt / (c.density * c.h), e->st, gate, s);  // project.go:179
    af::launch_velocity_bc(g, f.u, f.v, f.w, e->st, gate, s);
}

// `parity` is the U/V/W slot parity at this point of the step (the
// multigrid projection addresses fields through the batch's slot table).
void enqueue_project(af_engine* e, const Fields& f, int gate, int parity) {
    if (!e->mg) {
        enqueue_project_fp64(e, f, gate);
        return;
    }
    rec(e, kEvRb + (gate == 3 ? 0 : 2));
    e->launches_per_step += af::batch_enqueue_project(e->mg, parity, gate, e->stream);
    rec(e, kEvRb + (gate == 3 ? 1 : 3));
}

// The sweep kernels of one axis: the reference's semi-Lagrangian sweep, or
// its MacCormack form.  Returns the launches.
int launch_advect(af_engine* e, const Fields& f, int axis, double dt, int phase) {
    const Geom& g = e->geom;
    const double invH = 1.0 / e->cfg.h;
    const double lam = e->cfg.viscosity * dt * invH * invH;  // stencil.go:73
    if (e->advection == AF_ADVECTION_MACCORMACK) {
        Fields fwd = f;
        fwd.t0 = (double*)e->mc_scratch;
        fwd.t1 = fwd.t0 + ((g.u.count + 15) & ~15ll);
        fwd.t2 = fwd.t1 + ((g.v.count + 15) & ~15ll);
        af::launch_maccormack_fp64(g, axis, f, fwd, dt, invH, lam, e->st, phase, e->stream);
        return 2;
    }
    af::launch_sweep_fp64(g, axis, f, dt, invH, lam, e->st, phase, e->stream);
    return 1;
}

void enqueue_sweep(af_engine* e, Fields& f, int axis, double dt, int phase) {
    af::launch_velocity_bc(e->geom, f.u, f.v, f.w, e->st, phase, e->stream);
    rec(e, kEvSweep + 2 * phase);
    e->launches_per_step += 1 + launch_advect(e, f, axis, dt, phase);
    rec(e, kEvSweep + 2 * phase + 1);
    swap_fields(f);  // commitVelocity, stencil.go:230-235
}

// Step, aeroflux.go:348-409.
void enqueue_step(af_engine* e) {
    Fields f = e->fields();
    e->launches_per_step = 1;  // the step tick
    e->rbgs_launches_per_step = 0;
    rec(e, kEvStart);
    const double half = e->cfg.dt * 0.5;  // aeroflux.go:353
    for (int k = 0; k < 3; ++k) enqueue_sweep(e, f, kFwd[k], half, k);
    enqueue_project(e, f, 3, e->parity ^ 1);
    for (int k = 0; k < 3; ++k) enqueue_sweep(e, f, kRev[k], half, 3 + k);
    enqueue_project(e, f, 6, e->parity);
    af::launch_step_tick(e->st, e->stream);
    rec(e, kEvEnd);
}

// Captures `body` on the engine stream and instantiates it.
template <class F>
int capture(af_engine* e, F body, cudaGraphExec_t* out) {
    cudaGraph_t graph = nullptr;
    AF_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    body();
    cudaError_t rc = cudaStreamEndCapture(e->stream, &graph);
    if (rc != cudaSuccess) return cuda_fail(e, rc, "cudaStreamEndCapture");
    rc = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (rc != cudaSuccess) return cuda_fail(e, rc, "cudaGraphInstantiate");
    return AF_OK;
}

// Captures `body`; with the multigrid option the batch's tables are
// prepared first and an error its enqueue recorded fails the capture.
template <class F>
int capture_step(af_engine* e, F body, cudaGraphExec_t* out) {
    if (e->mg) {
        const cudaError_t rc = af::batch_prepare_capture(e->mg);
        if (rc != cudaSuccess) return cuda_fail(e, rc, "preparing the multigrid projection");
    }
    if (int rc = capture(e, body, out)) return rc;
    if (e->mg) {
        const cudaError_t rc = af::batch_capture_error(e->mg);
        if (rc != cudaSuccess) {
            cudaGraphExecDestroy(*out);
            *out = nullptr;
            return cuda_fail(e, rc, "capturing the multigrid projection");
        }
    }
    return AF_OK;
}

int build_graph(af_engine* e) { return capture_step(e, [&] { enqueue_step(e); }, &e->graph[e->parity]); }

std::string fault_message(const af_engine* e, unsigned gate, unsigned long long key) {
    return af::fault_message_for(e->geom, gate, key);
}

void drop_graphs(af_engine* e) {
    for (auto& gexec : e->graph)
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
}

int release(af_engine* e) {
    drop_graphs(e);
    for (auto& ev : e->ev)
        if (ev) { cudaEventDestroy(ev); ev = nullptr; }
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->batch) { af::batch_destroy(e->batch); e->batch = nullptr; }
    if (e->mg) {
        af::batch_destroy(e->mg);
        e->mg = nullptr;
        e->st = e->own_st;
        e->own_st = nullptr;
    }
    cudaFree(e->mc_scratch);
    e->mc_scratch = nullptr;
    cudaFree(e->arena);
    cudaFree(e->b);
    cudaFree(e->st);
    cudaFree(e->partials);
    cudaFree(e->sum);
    cudaFree(e->mx);
    e->arena = nullptr;
    e->b = nullptr;
    e->st = nullptr;
    e->partials = e->sum = nullptr;
    e->mx = nullptr;
    if (e->stream) { cudaStreamDestroy(e->stream); e->stream = nullptr; }
    return AF_OK;
}

// MIXED: wait for the batch stream and turn a slot fault into the error.
int batch_check(af_engine* e, cudaError_t rc, const std::string& what) {
    if (rc != cudaSuccess) {
        e->err = what.empty() ? sfmt("aeroflux: cuda: %s", cudaGetErrorString(rc)) : what;
        return AF_ERR_CUDA;
    }
    if ((rc = cudaStreamSynchronize(af::batch_stream(e->batch))) != cudaSuccess) return cuda_fail(e, rc, "batch");
    std::string msg;
    int first = -1;
    if (af::debug_bounds_error(&msg)) {
        e->err = msg;
        return AF_ERR_CUDA;
    }
    if (af::batch_device_error(e->batch, &msg)) {
        e->err = msg;
        return AF_ERR_CUDA;
    }
    if (af::batch_collect_faults(e->batch, &msg, &first)) {
        e->err = msg;
        return AF_ERR_FAULT;
    }
    return AF_OK;
}

int sync_and_check(af_engine* e) {
    Status s;
    AF_CUDA(e, cudaMemcpyAsync(&s, e->st, sizeof s, cudaMemcpyDeviceToHost, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    if (af::debug_bounds_error(&e->err)) return AF_ERR_CUDA;
    if (s.fault_gate != af::kNoFault) {
        e->err = fault_message(e, s.fault_gate, s.fault_key);
        // The reference returns before commitVelocity of the faulting sweep:
        // `phase` commits happened in the faulting step.
        e->parity ^= (int)((s.fault_gate % 8u) & 1u);
        return AF_ERR_FAULT;
    }
    return AF_OK;
}

}  // namespace

namespace af {

bool debug_bounds_error(std::string* msg) {
    unsigned long long f1 = ~0ull, f2 = ~0ull;
    unsigned n1 = 0, n2 = 0;
    if (!batch_debug_bounds(&f1, &n1, false) || !fp64_debug_bounds(&f2, &n2, false) || n1 + n2 == 0) return false;
    const unsigned long long f = f1 != ~0ull ? f1 : f2;
    *msg = sfmt("aeroflux: debug bounds check: %u out-of-buffer accesses; first in kernel %u, slot %u, at element "
                "offset %lld",
                n1 + n2, (unsigned)(f >> 56), (unsigned)((f >> 40) & 0xFFFF),
                (long long)((f & 0x8000000000ull) ? (long long)(f & 0xFFFFFFFFFFull) - (1ll << 40)
                                                  : (long long)(f & 0xFFFFFFFFFFull)));
    batch_debug_bounds(&f1, &n1, true);
    fp64_debug_bounds(&f2, &n2, true);
    return true;
}

}  // namespace af

extern "C" {

int af_abi_version(void) { return AF_ABI_VERSION; }

int af_debug_bounds(int32_t* enabled, uint64_t* first, uint32_t* violations, int32_t reset) {
    if (!enabled || !first || !violations) return AF_ERR_ARG;
    unsigned long long f1 = ~0ull, f2 = ~0ull;
    unsigned n1 = 0, n2 = 0;
    if (!af::batch_debug_bounds(&f1, &n1, reset != 0) || !af::fp64_debug_bounds(&f2, &n2, reset != 0))
        return AF_ERR_CUDA;
    *enabled = AEROFLUX_DEBUG_BOUNDS;
    *first = f1 != ~0ull ? f1 : f2;
    *violations = n1 + n2;
    return AF_OK;
}

int af_config_normalize(af_config* cfg, char* err, size_t errlen) {
    if (!cfg) return AF_ERR_ARG;
    std::string m = normalize(cfg);
    if (!m.empty()) {
        put_err(err, errlen, m);
        return AF_ERR_CONFIG;
    }
    return AF_OK;
}

int64_t af_mac_bytes(int64_t nx, int64_t ny, int64_t nz, int64_t ghost) {
    if (nx < 1 || ny < 1 || nz < 1 || ghost < 1) return 0;
    af_field_desc f[8];
    return mac_layout(nx, ny, nz, ghost, f);
}

int af_create(const af_config* cin, af_engine** out, char* err, size_t errlen) {
    if (!cin || !out) return AF_ERR_ARG;
    *out = nullptr;
    af_config c = *cin;
    std::string m = normalize(&c);
    if (!m.empty()) {
        put_err(err, errlen, m);
        return AF_ERR_CONFIG;
    }
    af_engine* e = new (std::nothrow) af_engine();
    if (!e) {
        put_err(err, errlen, "aeroflux: out of host memory");
        return AF_ERR_NOMEM;
    }
    e->cfg = c;
    e->bytes = mac_layout(c.nx, c.ny, c.nz, c.ghost, e->desc);
    if (e->desc[AF_FIELD_U].count >= (1ll << 31) || e->desc[AF_FIELD_V].count >= (1ll << 31) ||
        e->desc[AF_FIELD_W].count >= (1ll << 31) || c.nx >= (1 << 20) || c.ny >= (1 << 20) || c.nz >= (1 << 20)) {
        put_err(err, errlen, "aeroflux: grid too large for one device field (2^31 elements per field)");
        delete e;
        return AF_ERR_CONFIG;
    }
    Geom& g = e->geom;
    g.NX = (int)c.nx;
    g.NY = (int)c.ny;
    g.NZ = (int)c.nz;
    g.G = (int)c.ghost;
    g.p = to_dims(e->desc[AF_FIELD_P]);
    g.u = to_dims(e->desc[AF_FIELD_U]);
    g.v = to_dims(e->desc[AF_FIELD_V]);
    g.w = to_dims(e->desc[AF_FIELD_W]);

    int rc = AF_OK;
    auto fail = [&](int code) {
        put_err(err, errlen, e->err);
        release(e);
        delete e;
        return code;
    };
    cudaError_t cr;
    if ((cr = cudaSetDevice(c.device)) != cudaSuccess)
        return (cuda_fail(e, cr, "cudaSetDevice"), fail(AF_ERR_CUDA));
    if ((cr = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return (cuda_fail(e, cr, "cudaStreamCreate"), fail(AF_ERR_CUDA));
    if ((cr = cudaMalloc(&e->arena, (size_t)e->bytes)) != cudaSuccess) {
        e->err = sfmt("aeroflux: device arena of %lld bytes: %s", (long long)e->bytes, cudaGetErrorString(cr));
        return fail(AF_ERR_NOMEM);
    }
    if (c.precision == AF_PRECISION_FP64) {
        if ((cr = cudaMalloc(&e->b, (size_t)e->desc[AF_FIELD_P].count * 8)) != cudaSuccess) {
            e->err = sfmt("aeroflux: device scratch: %s", cudaGetErrorString(cr));
            return fail(AF_ERR_NOMEM);
        }
    }
    if ((cr = cudaMalloc(&e->st, sizeof(Status))) != cudaSuccess ||
        (cr = cudaMalloc(&e->partials, sizeof(double) * (size_t)std::max<int64_t>(c.nz, 1))) != cudaSuccess ||
        (cr = cudaMalloc(&e->sum, sizeof(double))) != cudaSuccess ||
        (cr = cudaMalloc(&e->mx, sizeof(unsigned long long))) != cudaSuccess) {
        e->err = sfmt("aeroflux: device scratch: %s", cudaGetErrorString(cr));
        return fail(AF_ERR_NOMEM);
    }
    // MAC.Zero (grid.go:158-163): every field, ghosts and Tmp included.
    if ((cr = cudaMemsetAsync(e->arena, 0, (size_t)e->bytes, e->stream)) != cudaSuccess)
        return (cuda_fail(e, cr, "cudaMemset"), fail(AF_ERR_CUDA));
    if (c.precision == AF_PRECISION_MIXED) {
        if ((cr = cudaStreamSynchronize(e->stream)) != cudaSuccess)
            return (cuda_fail(e, cr, "cudaStreamSynchronize"), fail(AF_ERR_CUDA));
        std::string merr;
        e->batch = af::batch_create(1, 0, &merr);
        if (!e->batch || af::batch_assign(e->batch, c, e->arena, &merr) != 0) {
            e->err = merr;
            return fail(AF_ERR_NOMEM);
        }
        // Pick launch shapes while every field is still zero (results do not
        // depend on them); AEROFLUX_NO_TUNE=1 keeps the defaults.
        const char* nt = getenv("AEROFLUX_NO_TUNE");
        if (!(nt && nt[0] == '1')) af::batch_tune(e->batch, 2);
    }
    if ((rc = reset_status(e)) != AF_OK) return fail(rc);
    if ((cr = cudaStreamSynchronize(e->stream)) != cudaSuccess)
        return (cuda_fail(e, cr, "cudaStreamSynchronize"), fail(AF_ERR_CUDA));
    *out = e;
    return AF_OK;
}

int af_get_config(const af_engine* e, af_config* out) {
    if (!e || !out) return AF_ERR_ARG;
    *out = e->cfg;
    return AF_OK;
}

int af_field_info(const af_engine* e, int field, af_field_desc* out) {
    if (!e || !out || field < 0 || field > 7) return AF_ERR_ARG;
    *out = e->current(field, nullptr);
    return AF_OK;
}

int af_field_upload(af_engine* e, int field, const double* host, size_t count) {
    if (int rc = check_open(e)) return rc;
    if (field < 0 || field > 7 || !host) {
        e->err = "aeroflux: bad field upload arguments";
        return AF_ERR_ARG;
    }
    double* dev = nullptr;
    const af_field_desc d = e->current(field, &dev);
    if ((int64_t)count != d.count) {
        e->err = sfmt("aeroflux: field upload of %lld values, field holds %lld", (long long)count, (long long)d.count);
        return AF_ERR_ARG;
    }
    AF_CUDA(e, cudaMemcpyAsync(dev, host, count * 8, cudaMemcpyHostToDevice, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    return AF_OK;
}

int af_field_download(af_engine* e, int field, double* host, size_t count) {
    if (int rc = check_open(e)) return rc;
    if (field < 0 || field > 7 || !host) {
        e->err = "aeroflux: bad field download arguments";
        return AF_ERR_ARG;
    }
    double* dev = nullptr;
    const af_field_desc d = e->current(field, &dev);
    if ((int64_t)count != d.count) {
        e->err = sfmt("aeroflux: field download of %lld values, field holds %lld", (long long)count,
                      (long long)d.count);
        return AF_ERR_ARG;
    }
    AF_CUDA(e, cudaMemcpyAsync(host, dev, count * 8, cudaMemcpyDeviceToHost, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    return AF_OK;
}

int af_apply_velocity_bc(af_engine* e) {
    if (int rc = check_open(e)) return rc;
    if (e->batch) return batch_check(e, af::batch_velocity_bc(e->batch), "");
    if (int rc = reset_status(e)) return rc;
    Fields f = e->fields();
    af::launch_velocity_bc(e->geom, f.u, f.v, f.w, e->st, 0, e->stream);
    AF_CUDA(e, cudaGetLastError());
    return sync_and_check(e);
}

int af_step(af_engine* e, int64_t nsteps) {
    if (int rc = check_open(e)) return rc;
    if (nsteps < 0) {
        e->err = "aeroflux: negative step count";
        return AF_ERR_ARG;
    }
    if (nsteps == 0) return AF_OK;
    if (e->batch) {
        std::string err;
        cudaError_t rc = af::batch_step(e->batch, nsteps, &err);
        return batch_check(e, rc, err);
    }
    if (!e->graph[e->parity])
        if (int rc = build_graph(e)) return rc;
    if (int rc = reset_status(e)) return rc;
    for (int64_t i = 0; i < nsteps; ++i) AF_CUDA(e, cudaGraphLaunch(e->graph[e->parity], e->stream));
    return sync_and_check(e);
}

int af_project(af_engine* e) {
    if (int rc = check_open(e)) return rc;
    if (e->batch) {
        std::string err;
        cudaError_t rc = af::batch_project(e->batch, &err);
        return batch_check(e, rc, err);
    }
    if (int rc = reset_status(e)) return rc;
    if (e->mg) {
        // The multigrid projection's refinement loop is a conditional graph
        // node, so even a single projection runs as a captured graph.
        cudaGraphExec_t g = nullptr;
        if (int rc = capture_step(e, [&] { enqueue_project(e, e->fields(), 0, e->parity); }, &g)) return rc;
        const cudaError_t lr = cudaGraphLaunch(g, e->stream);
        cudaStreamSynchronize(e->stream);
        cudaGraphExecDestroy(g);
        AF_CUDA(e, lr);
        return sync_and_check(e);
    }
    enqueue_project(e, e->fields(), 0, e->parity);
    AF_CUDA(e, cudaGetLastError());
    return sync_and_check(e);
}

int af_phase_sweep(af_engine* e, int axis, double dt) {
    if (int rc = check_open(e)) return rc;
    if (axis < 0 || axis > 2) {
        e->err = "aeroflux: axis must be 0, 1 or 2";
        return AF_ERR_ARG;
    }
    if (e->batch) return batch_check(e, af::batch_sweep(e->batch, axis, dt), "");
    if (int rc = reset_status(e)) return rc;
    launch_advect(e, e->fields(), axis, dt, 0);
    AF_CUDA(e, cudaGetLastError());
    Status s;
    AF_CUDA(e, cudaMemcpyAsync(&s, e->st, sizeof s, cudaMemcpyDeviceToHost, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    if (s.fault_gate != af::kNoFault) {
        // fault_message derives the axis from the phase: map axis to a forward phase.
        e->err = fault_message(e, (unsigned)axis, s.fault_key);
        return AF_ERR_FAULT;
    }
    e->parity ^= 1;  // commitVelocity
    return AF_OK;
}

int af_phase_divergence(af_engine* e) {
    if (int rc = check_open(e)) return rc;
    if (e->batch) {
        e->err = "aeroflux: phase hooks of the projection exist for the FP64 form only";
        return AF_ERR_UNSUPPORTED;
    }
    if (int rc = reset_status(e)) return rc;
    const af_config& c = e->cfg;
    af::launch_divergence_fp64(e->geom, e->fields(), e->b, c.density / (c.dt * c.h), c.h * c.h, false, e->st, 0,
                               e->stream);
    AF_CUDA(e, cudaGetLastError());
    return sync_and_check(e);
}

int af_phase_red_black(af_engine* e) {
    if (int rc = check_open(e)) return rc;
    if (e->batch) {
        e->err = "aeroflux: phase hooks of the projection exist for the FP64 form only";
        return AF_ERR_UNSUPPORTED;
    }
    if (int rc = reset_status(e)) return rc;
    // solvePressureRedBlack zeroes P itself (project.go:81-83); the divergence
    // kernel does that zeroing in the fused path, so do it here explicitly.
    Fields f = e->fields();
    AF_CUDA(e, cudaMemsetAsync(f.p, 0, (size_t)e->desc[AF_FIELD_P].count * 8, e->stream));
    // B = h2*Div as the divergence kernel would have left it.
    af::launch_b_from_div(e->geom, f.div, e->b, e->cfg.h * e->cfg.h, e->stream);
    for (int64_t it = 0; it < e->cfg.gauss_seidel_iters; ++it) {
        af::launch_rbgs_fp64(e->geom, f.p, e->b, 0, e->st, 0, e->stream);
        af::launch_rbgs_fp64(e->geom, f.p, e->b, 1, e->st, 0, e->stream);
    }
    af::launch_pressure_bc_fp64(e->geom, f.p, e->st, 0, e->stream);
    AF_CUDA(e, cudaGetLastError());
    return sync_and_check(e);
}

int af_phase_pressure_bc(af_engine* e) {
    if (int rc = check_open(e)) return rc;
    if (int rc = reset_status(e)) return rc;
    af::launch_pressure_bc_fp64(e->geom, e->fields().p, e->st, 0, e->stream);
    AF_CUDA(e, cudaGetLastError());
    return sync_and_check(e);
}

int af_phase_subtract_gradient(af_engine* e) {
    if (int rc = check_open(e)) return rc;
    if (int rc = reset_status(e)) return rc;
    const af_config& c = e->cfg;
    af::launch_gradient_fp64(e->geom, e->fields(), c.dt / (c.density * c.h), e->st, 0, e->stream);
    AF_CUDA(e, cudaGetLastError());
    return sync_and_check(e);
}

int af_max_divergence(af_engine* e, double* out) {
    if (int rc = check_open(e)) return rc;
    if (!out) return AF_ERR_ARG;
    Fields f = e->fields();
    AF_CUDA(e, cudaMemsetAsync(e->mx, 0, sizeof(unsigned long long), e->stream));
    af::launch_max_divergence(e->geom, f.u, f.v, f.w, 1.0 / e->cfg.h, e->mx, e->stream);
    AF_CUDA(e, cudaGetLastError());
    unsigned long long bits = 0;
    AF_CUDA(e, cudaMemcpyAsync(&bits, e->mx, sizeof bits, cudaMemcpyDeviceToHost, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    memcpy(out, &bits, sizeof bits);
    return AF_OK;
}

int af_kinetic_energy(af_engine* e, double* out) {
    if (int rc = check_open(e)) return rc;
    if (!out) return AF_ERR_ARG;
    Fields f = e->fields();
    af::launch_kinetic_energy(e->geom, f.u, f.v, f.w, e->partials, e->sum, e->stream);
    AF_CUDA(e, cudaGetLastError());
    double sum = 0;
    AF_CUDA(e, cudaMemcpyAsync(&sum, e->sum, sizeof sum, cudaMemcpyDeviceToHost, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    const double h = e->cfg.h;
    const double vol = h * h * h;
    *out = 0.5 * sum * vol;  // project.go:244,257
    return AF_OK;
}

int af_max_velocity(af_engine* e, double* out) {
    if (int rc = check_open(e)) return rc;
    if (!out) return AF_ERR_ARG;
    Fields f = e->fields();
    AF_CUDA(e, cudaMemsetAsync(e->mx, 0, sizeof(unsigned long long), e->stream));
    af::launch_max_abs3(f.u, e->geom.u.count, f.v, e->geom.v.count, f.w, e->geom.w.count, e->mx, e->stream);
    AF_CUDA(e, cudaGetLastError());
    unsigned long long bits = 0;
    AF_CUDA(e, cudaMemcpyAsync(&bits, e->mx, sizeof bits, cudaMemcpyDeviceToHost, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    memcpy(out, &bits, sizeof bits);
    return AF_OK;
}

int af_cfl(af_engine* e, double* out) {
    double mv = 0;
    if (int rc = af_max_velocity(e, &mv)) return rc;
    *out = mv * e->cfg.dt / e->cfg.h;  // stencil.go:337
    return AF_OK;
}

int af_enable_sparse_solver(af_engine* e) {
    if (int rc = check_open(e)) return rc;
    e->err =
        "aeroflux: sparse direct solver requires darwin with cgo (Accelerate); the Red-Black iterative solver is "
        "used instead";
    return AF_ERR_UNSUPPORTED;
}

int af_enable_multigrid_solver(af_engine* e, double div_tol) {
    if (int rc = check_open(e)) return rc;
    if (e->batch) {
        e->err = "aeroflux: the mixed-precision form already projects with multigrid";
        return AF_ERR_UNSUPPORTED;
    }
    if (e->mg) return AF_OK;  // EnableSparseSolver is idempotent (sparse_darwin.go:26-29)
    if (div_tol == 0.0) div_tol = 1e-12;
    if (!(div_tol > 0.0) || !std::isfinite(div_tol)) {
        e->err = sfmt("aeroflux: multigrid divergence tolerance must be positive and finite, got %g", div_tol);
        return AF_ERR_ARG;
    }
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    af_config mc = e->cfg;
    mc.precision = AF_PRECISION_MIXED;
    mc.div_tol = div_tol;
    if (mc.inner_sweeps < 1) mc.inner_sweeps = 2;
    if (mc.max_refine < 1) mc.max_refine = 30;
    std::string merr;
    af::Batch* b = af::batch_create(1, 0, &merr);
    if (!b || af::batch_assign(b, mc, e->arena, &merr) != 0) {
        if (b) af::batch_destroy(b);
        e->err = merr.empty() ? "aeroflux: multigrid solver setup failed" : merr;
        return AF_ERR_NOMEM;
    }
    e->mg = b;
    e->own_st = e->st;
    e->st = af::batch_status(b, 0);
    e->cfg.div_tol = div_tol;
    drop_graphs(e);  // recaptured with the multigrid projection and the new status word
    return reset_status(e);
}

int af_set_advection(af_engine* e, int scheme) {
    if (int rc = check_open(e)) return rc;
    if (scheme != AF_ADVECTION_SEMI_LAGRANGIAN && scheme != AF_ADVECTION_MACCORMACK) {
        e->err = sfmt("aeroflux: unknown advection scheme %d", scheme);
        return AF_ERR_ARG;
    }
    if (e->batch) {
        if (scheme == AF_ADVECTION_SEMI_LAGRANGIAN) return AF_OK;
        e->err = "aeroflux: MacCormack advection is available in the FP64 form only";
        return AF_ERR_UNSUPPORTED;
    }
    if (scheme == e->advection) return AF_OK;
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    if (scheme == AF_ADVECTION_MACCORMACK && !e->mc_scratch) {
        const Geom& g = e->geom;
        const size_t n = (size_t)((g.u.count + 15) & ~15ll) + (size_t)((g.v.count + 15) & ~15ll) + (size_t)g.w.count;
        const cudaError_t rc = cudaMalloc(&e->mc_scratch, n * sizeof(double));
        if (rc != cudaSuccess) {
            cudaGetLastError();
            e->mc_scratch = nullptr;
            e->err = sfmt("aeroflux: MacCormack scratch of %zu bytes: %s", n * sizeof(double), cudaGetErrorString(rc));
            return AF_ERR_NOMEM;
        }
    }
    e->advection = scheme;
    drop_graphs(e);
    return AF_OK;
}

int af_last_projection_vcycles(af_engine* e, int64_t* vcycles) {
    if (int rc = check_open(e)) return rc;
    if (!vcycles) return AF_ERR_ARG;
    *vcycles = 0;
    af::Batch* b = e->mg ? e->mg : e->batch;
    if (!b) return AF_OK;
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    int64_t passes = 0;
    double md = 0;
    af::batch_slot_projection(b, 0, &passes, &md, vcycles);
    return AF_OK;
}

int af_last_projection_stats(af_engine* e, int64_t* passes, double* max_div) {
    if (int rc = check_open(e)) return rc;
    if (!passes || !max_div) return AF_ERR_ARG;
    if (e->mg) {
        AF_CUDA(e, cudaStreamSynchronize(e->stream));
        af::batch_slot_projection(e->mg, 0, passes, max_div);
        return AF_OK;
    }
    if (!e->batch) {
        *passes = 0;
        return af_max_divergence(e, max_div);
    }
    af::batch_slot_projection(e->batch, 0, passes, max_div);
    return AF_OK;
}

int af_profile(af_engine* e, int enable) {
    if (int rc = check_open(e)) return rc;
    if (e->batch) {
        AF_CUDA(e, af::batch_profile(e->batch, enable != 0));
        return AF_OK;
    }
    const bool on = enable != 0;
    if (on == e->profiling) return AF_OK;
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    if (on)
        for (auto& ev : e->ev)
            if (!ev) AF_CUDA(e, cudaEventCreate(&ev));
    e->profiling = on;
    drop_graphs(e);
    return AF_OK;
}

int af_last_step_profile(af_engine* e, af_step_profile* out) {
    if (int rc = check_open(e)) return rc;
    if (!out) return AF_ERR_ARG;
    if (e->batch) {
        af_step_profile p{};
        AF_CUDA(e, af::batch_last_profile(e->batch, &p.step_ms, &p.sweep_ms, &p.rbgs_ms, &p.kernel_launches));
        *out = p;
        return AF_OK;
    }
    if (!e->profiling || !e->graph[e->parity]) {
        e->err = "aeroflux: profiling is off or no step has run";
        return AF_ERR_ARG;
    }
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    auto ms = [&](int a, int b, double* acc) -> cudaError_t {
        float t = 0;
        cudaError_t rc = cudaEventElapsedTime(&t, e->ev[a], e->ev[b]);
        if (rc == cudaSuccess) *acc += t;
        return rc;
    };
    af_step_profile p{};
    AF_CUDA(e, ms(kEvStart, kEvEnd, &p.step_ms));
    for (int k = 0; k < 6; ++k) AF_CUDA(e, ms(kEvSweep + 2 * k, kEvSweep + 2 * k + 1, &p.sweep_ms));
    AF_CUDA(e, ms(kEvRb, kEvRb + 1, &p.rbgs_ms));
    AF_CUDA(e, ms(kEvRb + 2, kEvRb + 3, &p.rbgs_ms));
    p.rbgs_launches = e->rbgs_launches_per_step;
    p.kernel_launches = e->launches_per_step;
    *out = p;
    return AF_OK;
}

int af_selftest_div6(int device, int64_t n, uint64_t seed, int64_t* mismatches) {
    if (!mismatches || n < 0 || device < 0) return AF_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return AF_ERR_CUDA;
    unsigned long long bad = 0;
    if (!af::selftest_div6((unsigned long long)n, seed, &bad)) return AF_ERR_CUDA;
    *mismatches = (int64_t)bad;
    return AF_OK;
}

int af_selftest_dadd(int device, int64_t n, uint64_t seed, int64_t* mismatches) {
    if (!mismatches || n < 0 || device < 0) return AF_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return AF_ERR_CUDA;
    unsigned long long bad = 0;
    if (!af::selftest_dadd((unsigned long long)n, seed, &bad)) return AF_ERR_CUDA;
    *mismatches = (int64_t)bad;
    return AF_OK;
}

int af_device_fp64_rate(int device, double* fma_per_s) {
    if (!fma_per_s || device < 0) return AF_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return AF_ERR_CUDA;
    return af::measure_fp64_rate(fma_per_s) ? AF_OK : AF_ERR_CUDA;
}

int af_seed_device(af_engine* e, double amp, double noise, uint64_t seed, uint64_t stream) {
    if (int rc = check_open(e)) return rc;
    Fields f = e->fields();
    double* zero[6] = {f.u, f.v, f.w, f.t0, f.t1, f.t2};
    const int ids[6] = {AF_FIELD_U, AF_FIELD_V, AF_FIELD_W, AF_FIELD_TMP0, AF_FIELD_TMP1, AF_FIELD_TMP2};
    for (int k = 0; k < 6; ++k)
        AF_CUDA(e, cudaMemsetAsync(zero[k], 0, (size_t)e->current(ids[k], nullptr).count * 8, e->stream));
    AF_CUDA(e, af::seed_tg_fields(e->geom, f.u, f.v, f.w, e->cfg.h, amp, noise, seed, stream, e->stream));
    AF_CUDA(e, cudaStreamSynchronize(e->stream));
    return AF_OK;
}

int af_close(af_engine* e) {
    if (!e) return AF_ERR_ARG;
    if (e->closed) return AF_OK;
    release(e);
    e->closed = true;
    return AF_OK;
}

void af_destroy(af_engine* e) {
    if (!e) return;
    af_close(e);
    delete e;
}

const char* af_last_error(const af_engine* e) { return e ? e->err.c_str() : ""; }

// ---------------------------------------------------------------------------
// Batched form
// ---------------------------------------------------------------------------
struct af_batch {
    af::Batch* b = nullptr;
    int device = 0;
    unsigned long long* mx = nullptr;  // MaxDivergence result word
    std::vector<af_config> cfg;
    std::string err;
};

namespace {

int batch_fail(af_batch* h, int code, const std::string& m) {
    h->err = m;
    return code;
}

int batch_slot_ok(const af_batch* h, int64_t slot) {
    return h && slot >= 0 && slot < (int64_t)h->cfg.size() && h->cfg[slot].nx > 0;
}

int batch_wait(af_batch* h) {
    cudaError_t rc = cudaStreamSynchronize(af::batch_stream(h->b));
    if (rc != cudaSuccess) return batch_fail(h, AF_ERR_CUDA, sfmt("aeroflux: cuda: %s", cudaGetErrorString(rc)));
    return AF_OK;
}

}  // namespace

int af_batch_create(int64_t capacity, int64_t pool_bytes, int32_t device, af_batch** out, char* err, size_t errlen) {
    if (!out || capacity < 1 || pool_bytes < 0 || device < 0) return AF_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) {
        put_err(err, errlen, "aeroflux: cuda: no such device");
        return AF_ERR_CUDA;
    }
    std::string m;
    af::Batch* b = af::batch_create((int)capacity, (size_t)pool_bytes, &m);
    if (!b) {
        put_err(err, errlen, m);
        return AF_ERR_NOMEM;
    }
    af_batch* h = new af_batch();
    h->b = b;
    h->device = device;
    if (cudaMalloc(&h->mx, sizeof *h->mx) != cudaSuccess) {
        af::batch_destroy(b);
        delete h;
        put_err(err, errlen, "aeroflux: cuda: batch result word");
        return AF_ERR_NOMEM;
    }
    h->cfg.assign((size_t)capacity, af_config{});
    *out = h;
    return AF_OK;
}

int af_batch_slot_bytes(const af_config* cfg, int64_t* bytes) {
    if (!cfg || !bytes) return AF_ERR_ARG;
    af_config c = *cfg;
    if (!normalize(&c).empty()) return AF_ERR_CONFIG;
    if (!af::batch_config_fits(c, nullptr)) return AF_ERR_CONFIG;
    *bytes = (int64_t)af::batch_slot_bytes(c);
    return AF_OK;
}

int af_batch_assign(af_batch* h, const af_config* cfg, int64_t* slot) {
    if (!h || !cfg || !slot) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    af_config c = *cfg;
    std::string m = normalize(&c);
    if (!m.empty()) return batch_fail(h, AF_ERR_CONFIG, m);
    if (c.precision != AF_PRECISION_MIXED)
        return batch_fail(h, AF_ERR_CONFIG, "aeroflux: batches step the mixed-precision form only");
    const int s = af::batch_assign(h->b, c, nullptr, &m);
    if (s < 0) return batch_fail(h, AF_ERR_NOMEM, m);
    h->cfg[s] = c;
    *slot = s;
    return batch_wait(h);
}

int af_batch_release(af_batch* h, int64_t slot) {
    if (!batch_slot_ok(h, slot)) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    af::batch_release(h->b, (int)slot);
    h->cfg[slot] = af_config{};
    return AF_OK;
}

int af_batch_set_active(af_batch* h, int64_t slot, int active) {
    if (!batch_slot_ok(h, slot)) return AF_ERR_ARG;
    af::batch_set_active(h->b, (int)slot, active != 0);
    return AF_OK;
}

int af_batch_get_config(const af_batch* h, int64_t slot, af_config* out) {
    if (!batch_slot_ok(h, slot) || !out) return AF_ERR_ARG;
    *out = h->cfg[slot];
    return AF_OK;
}

int af_batch_field_info(const af_batch* h, int64_t slot, int field, af_field_desc* out) {
    if (!batch_slot_ok(h, slot) || !out || field < 0 || field > 7) return AF_ERR_ARG;
    *out = af::batch_field(h->b, (int)slot, field, nullptr);
    return AF_OK;
}

static int batch_copy(af_batch* h, int64_t slot, int field, void* host, size_t count, bool up) {
    if (!batch_slot_ok(h, slot) || !host || field < 0 || field > 7) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    double* dev = nullptr;
    const af_field_desc d = af::batch_field(h->b, (int)slot, field, &dev);
    if ((int64_t)count != d.count)
        return batch_fail(h, AF_ERR_ARG, sfmt("aeroflux: field copy of %lld values, field holds %lld",
                                              (long long)count, (long long)d.count));
    cudaStream_t s = af::batch_stream(h->b);
    cudaError_t rc = up ? cudaMemcpyAsync(dev, host, count * 8, cudaMemcpyHostToDevice, s)
                        : cudaMemcpyAsync(host, dev, count * 8, cudaMemcpyDeviceToHost, s);
    if (rc != cudaSuccess) return batch_fail(h, AF_ERR_CUDA, sfmt("aeroflux: cuda: %s", cudaGetErrorString(rc)));
    return batch_wait(h);
}

int af_batch_field_upload(af_batch* h, int64_t slot, int field, const double* host, size_t count) {
    return batch_copy(h, slot, field, const_cast<double*>(host), count, true);
}

int af_batch_field_download(af_batch* h, int64_t slot, int field, double* host, size_t count) {
    return batch_copy(h, slot, field, host, count, false);
}

int af_batch_apply_velocity_bc(af_batch* h) {
    if (!h) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    cudaError_t rc = af::batch_velocity_bc(h->b);
    if (rc != cudaSuccess) return batch_fail(h, AF_ERR_CUDA, sfmt("aeroflux: cuda: %s", cudaGetErrorString(rc)));
    return batch_wait(h);
}

int af_batch_step(af_batch* h, int64_t nsteps) {
    if (!h || nsteps < 0) return AF_ERR_ARG;
    if (nsteps == 0) return AF_OK;
    cudaSetDevice(h->device);
    std::string m;
    cudaError_t rc = af::batch_step(h->b, nsteps, &m);
    if (rc != cudaSuccess) return batch_fail(h, AF_ERR_CUDA, m);
    if (int r = batch_wait(h)) return r;
    if (af::debug_bounds_error(&m)) return batch_fail(h, AF_ERR_CUDA, m);
    if (af::batch_device_error(h->b, &m)) return batch_fail(h, AF_ERR_CUDA, m);
    int first = -1;
    af::batch_collect_faults(h->b, &m, &first);
    return AF_OK;
}

int af_batch_slot_status(af_batch* h, int64_t slot, int32_t* faulted, char* msg, size_t msglen) {
    if (!batch_slot_ok(h, slot) || !faulted) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    std::string m;
    *faulted = af::batch_slot_faulted(h->b, (int)slot, &m) ? 1 : 0;
    put_err(msg, msglen, *faulted ? m : "");
    return AF_OK;
}

int af_batch_max_divergence(af_batch* h, int64_t slot, double* out) {
    if (!batch_slot_ok(h, slot) || !out) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    double *u, *v, *w;
    af::batch_field(h->b, (int)slot, AF_FIELD_U, &u);
    af::batch_field(h->b, (int)slot, AF_FIELD_V, &v);
    af::batch_field(h->b, (int)slot, AF_FIELD_W, &w);
    cudaStream_t s = af::batch_stream(h->b);
    cudaMemsetAsync(h->mx, 0, sizeof *h->mx, s);
    af::launch_max_divergence(af::batch_geom(h->b, (int)slot), u, v, w, 1.0 / h->cfg[slot].h, h->mx, s);
    unsigned long long bits = 0;
    cudaMemcpyAsync(&bits, h->mx, sizeof bits, cudaMemcpyDeviceToHost, s);
    if (int r = batch_wait(h)) return r;
    memcpy(out, &bits, sizeof bits);
    return AF_OK;
}

int af_batch_projection_stats(af_batch* h, int64_t slot, int64_t* passes, double* max_div) {
    if (!batch_slot_ok(h, slot) || !passes || !max_div) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    af::batch_slot_projection(h->b, (int)slot, passes, max_div);
    return AF_OK;
}

int af_batch_tune(af_batch* h, int32_t reps, char* report, size_t len) {
    if (!h || reps < 1) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    const std::string r = af::batch_tune(h->b, reps);
    put_err(report, len, r);
    return AF_OK;
}

int af_batch_profile(af_batch* h, int enable) {
    if (!h) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    cudaError_t rc = af::batch_profile(h->b, enable != 0);
    return rc == cudaSuccess ? AF_OK : batch_fail(h, AF_ERR_CUDA, cudaGetErrorString(rc));
}

int af_batch_last_step_profile(af_batch* h, af_step_profile* out) {
    if (!h || !out) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    af_step_profile p{};
    cudaError_t rc = af::batch_last_profile(h->b, &p.step_ms, &p.sweep_ms, &p.rbgs_ms, &p.kernel_launches);
    if (rc != cudaSuccess) return batch_fail(h, AF_ERR_CUDA, "aeroflux: profiling is off or no step has run");
    *out = p;
    return AF_OK;
}

int af_batch_seed(af_batch* h, int64_t slot, double amp, double noise, uint64_t seed, uint64_t stream) {
    if (!batch_slot_ok(h, slot)) return AF_ERR_ARG;
    cudaSetDevice(h->device);
    cudaError_t rc = af::batch_seed(h->b, (int)slot, amp, noise, seed, stream);
    if (rc != cudaSuccess) return batch_fail(h, AF_ERR_CUDA, sfmt("aeroflux: cuda: %s", cudaGetErrorString(rc)));
    return batch_wait(h);
}

void af_batch_destroy(af_batch* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    af::batch_destroy(h->b);
    cudaFree(h->mx);
    delete h;
}

const char* af_batch_last_error(const af_batch* h) { return h ? h->err.c_str() : ""; }

}  // extern "C"
