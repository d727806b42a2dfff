/*
 * aeroflux_oracle.c -- CPU restatement of AeroFlux's fractional-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity oracle for the CUDA path.  Only the
 * test suite, the smoke check and the benchmark's CPU-baseline leg load it.
 *
 * Parity pin status: UNPINNED at the bit level (the reference ships no golden
 * vectors and Go is not available to run it).  The restatement is checked
 * against the properties the reference's tests assert and against the
 * divergence magnitudes published in the reference README.
 *
 * Arithmetic contract (must be compiled with -ffp-contract=off, no fast-math):
 *   - every expression is evaluated left to right exactly as the Go source
 *     writes it; Go on amd64 never contracts x*y+z into an FMA;
 *   - float64 -> int conversion follows amd64 CVTTSD2SQ: truncation toward
 *     zero, NaN -> INT64_MIN, and the index arithmetic that follows wraps
 *     modulo 2^64, so a NaN backtrace faults (or not) exactly where Go's
 *     slice bounds check would;
 *   - a contained fault aborts the faulting worker's shard for that dispatch,
 *     as RecoverFault (arena.go:230-243) does for a panicking goroutine.
 *
 * Threading mirrors the reference's worker pool: a static Z-slab partition
 * (aeroflux.go:218-232), one persistent thread per shard, and a join after
 * every phase (aeroflux.go:313-324).  Results do not depend on the worker
 * count, as in the reference.
 */
#define _GNU_SOURCE
#include "aeroflux_oracle.h"

#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <unistd.h>

#define CACHE_LINE_SIZE 128 /* layout.go:13 */

enum { AXIS_X = 0, AXIS_Y = 1, AXIS_Z = 2 };         /* stencil.go:5-11 */
enum { COMP_U = 0, COMP_V = 1, COMP_W = 2 };         /* stencil.go:27-33 */
enum { COLOR_RED = 0, COLOR_BLACK = 1 };             /* layout.go:27-33 */

typedef struct shard {
    int64_t z0, z1; /* half-open padded z-range, aeroflux.go:126-130 */
    int id;
} shard;

struct orc_engine;
typedef int (*shard_fn)(struct orc_engine*, const shard*, char* msg, size_t msglen);

typedef struct worker_slot {
    int faulted;
    char msg[256];
} worker_slot;

struct orc_engine {
    orc_config cfg;
    int64_t NX, NY, NZ, G;
    double H;
    orc_field f[ORC_NFIELDS];
    int64_t bytes;
    unsigned char* arena;
    size_t arena_len;
    int locked;

    shard* shards;
    int nw;
    worker_slot* slots;

    /* persistent pool: one thread per shard except shard 0 (run by the caller) */
    pthread_t* threads;
    pthread_mutex_t mu;
    pthread_cond_t cv_work, cv_done;
    uint64_t gen;
    int pending;
    int quit;
    shard_fn fn;
    int started;

    /* phase parameters, aeroflux.go:152-158 */
    int cur_axis;
    double cur_dt;
    int cur_color;

    /* MacCormack advection (orc_set_advection): scheme and the forward
     * step's three scratch fields, laid out as U, V, W. */
    int advection;
    double* mc[3];
};

/* ------------------------------------------------------------------------ */
/* Go formatting helpers                                                     */
/* ------------------------------------------------------------------------ */

/* strconv.FormatFloat(v, 'g', -1, 64): shortest round-trip digits, %e form
 * when the decimal exponent is < -4 or >= 6 (strconv/ftoa.go, 'g' with
 * shortest precision), "+Inf"/"-Inf"/"NaN" for the specials. */
void orc_go_format_float(double v, char* out, size_t outlen) {
    if (isnan(v)) { snprintf(out, outlen, "NaN"); return; }
    if (isinf(v)) { snprintf(out, outlen, v > 0 ? "+Inf" : "-Inf"); return; }
    char buf[64];
    int nd = 1;
    for (nd = 1; nd <= 17; ++nd) {
        snprintf(buf, sizeof buf, "%.*e", nd - 1, v);
        if (strtod(buf, NULL) == v) break;
    }
    /* buf = [-]d[.ddd]e[+-]XX ; pull the digits and the exponent out */
    const char* p = buf;
    int neg = 0;
    if (*p == '-') { neg = 1; ++p; }
    char digs[32];
    int n = 0;
    for (; *p && *p != 'e'; ++p)
        if (*p >= '0' && *p <= '9') digs[n++] = *p;
    digs[n] = 0;
    int exp10 = atoi(p + 1);
    /* strip trailing zeros (shortest digits never need them, except "0") */
    while (n > 1 && digs[n - 1] == '0') digs[--n] = 0;
    if (v == 0) { n = 1; digs[0] = '0'; digs[1] = 0; exp10 = 0; }
    char res[96];
    size_t k = 0;
    if (neg) res[k++] = '-';
    if (exp10 < -4 || exp10 >= 6) {
        res[k++] = digs[0];
        if (n > 1) {
            res[k++] = '.';
            for (int i = 1; i < n; ++i) res[k++] = digs[i];
        }
        k += (size_t)snprintf(res + k, sizeof res - k, "e%c%02d", exp10 < 0 ? '-' : '+', exp10 < 0 ? -exp10 : exp10);
    } else if (exp10 < 0) {
        res[k++] = '0';
        res[k++] = '.';
        for (int i = 0; i < -exp10 - 1; ++i) res[k++] = '0';
        for (int i = 0; i < n; ++i) res[k++] = digs[i];
        res[k] = 0;
    } else {
        int dp = exp10 + 1; /* digits before the decimal point */
        for (int i = 0; i < dp; ++i) res[k++] = i < n ? digs[i] : '0';
        if (n > dp) {
            res[k++] = '.';
            for (int i = dp; i < n; ++i) res[k++] = digs[i];
        }
        res[k] = 0;
    }
    snprintf(out, outlen, "%s", res);
}

static int fail(char* err, size_t errlen, const char* fmt, ...) {
    if (err && errlen) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, errlen, fmt, ap);
        va_end(ap);
    }
    return -1;
}

/* ------------------------------------------------------------------------ */
/* Config                                                                    */
/* ------------------------------------------------------------------------ */

static int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

/* (*Config).Normalize, aeroflux.go:47-113. */
int orc_normalize(orc_config* c, char* err, size_t errlen) {
    char a[48], b[48], d[48], e[48];
    if (c->nx <= 0 || c->ny <= 0 || c->nz <= 0)
        return fail(err, errlen, "aeroflux: interior extents must be positive, got %lldx%lldx%lld",
                    (long long)c->nx, (long long)c->ny, (long long)c->nz);
    if (c->ghost == 0) c->ghost = 1;
    if (c->ghost < 1)
        return fail(err, errlen, "aeroflux: ghost thickness must be >= 1, got %lld", (long long)c->ghost);
    if (c->h == 0) c->h = 1.0 / (double)max64(c->nx, max64(c->ny, c->nz));
    if (c->h <= 0 || isnan(c->h) || isinf(c->h)) {
        orc_go_format_float(c->h, a, sizeof a);
        return fail(err, errlen, "aeroflux: cell size must be finite and positive, got %s", a);
    }
    if (c->density == 0) c->density = 1.0;
    if (c->density <= 0 || isnan(c->density) || isinf(c->density)) {
        orc_go_format_float(c->density, a, sizeof a);
        return fail(err, errlen, "aeroflux: density must be finite and positive, got %s", a);
    }
    if (c->viscosity < 0 || isnan(c->viscosity) || isinf(c->viscosity)) {
        orc_go_format_float(c->viscosity, a, sizeof a);
        return fail(err, errlen, "aeroflux: viscosity must be finite and non-negative, got %s", a);
    }
    if (c->dt == 0) {
        if (c->viscosity > 0)
            c->dt = 0.5 * c->h * c->h / (6 * c->viscosity); /* ((0.5*h)*h)/(6*nu) */
        else
            c->dt = 0.25 * c->h;
    }
    if (c->dt <= 0 || isnan(c->dt) || isinf(c->dt)) {
        orc_go_format_float(c->dt, a, sizeof a);
        return fail(err, errlen, "aeroflux: timestep must be finite and positive, got %s", a);
    }
    if (c->workers == 0) {
        /* runtime.GOMAXPROCS(0) defaults to the CPUs this process may run on */
        cpu_set_t set;
        c->workers = sched_getaffinity(0, sizeof set, &set) == 0 ? CPU_COUNT(&set)
                                                                 : (int64_t)sysconf(_SC_NPROCESSORS_ONLN);
    }
    if (c->workers < 1)
        return fail(err, errlen, "aeroflux: worker count must be >= 1, got %lld", (long long)c->workers);
    if (c->workers > c->nz) c->workers = c->nz;
    if (c->gauss_seidel_iters == 0) c->gauss_seidel_iters = 24;
    if (c->gauss_seidel_iters < 1)
        return fail(err, errlen, "aeroflux: gauss-seidel iterations must be >= 1, got %lld",
                    (long long)c->gauss_seidel_iters);
    if (c->viscosity > 0) {
        double limit = c->h * c->h / (6 * c->viscosity);
        if (c->dt > limit) {
            orc_go_format_float(c->dt, a, sizeof a);
            orc_go_format_float(limit, b, sizeof b);
            orc_go_format_float(c->h, d, sizeof d);
            orc_go_format_float(c->viscosity, e, sizeof e);
            return fail(err, errlen,
                        "aeroflux: dt %s exceeds explicit diffusion stability limit %s (h=%s, nu=%s); reduce dt or h",
                        a, b, d, e);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Layout, grid.go:79-144                                                    */
/* ------------------------------------------------------------------------ */

static orc_field field_layout(int64_t* off, int64_t nx, int64_t ny, int64_t nz) {
    orc_field f;
    f.off = *off;
    f.nx = nx;
    f.ny = ny;
    f.nz = nz;
    f.sy = nx;
    f.sz = nx * ny;
    f.count = nx * ny * nz;
    int64_t sz = f.count * 8;
    int64_t r = sz % CACHE_LINE_SIZE;
    if (r != 0) sz += CACHE_LINE_SIZE - r;
    *off += sz;
    return f;
}

static int64_t mac_layout(int64_t nx, int64_t ny, int64_t nz, int64_t g, orc_field f[ORC_NFIELDS]) {
    int64_t cx = nx + 2 * g, cy = ny + 2 * g, cz = nz + 2 * g;
    int64_t off = 0;
    f[ORC_P] = field_layout(&off, cx, cy, cz);
    f[ORC_U] = field_layout(&off, cx + 1, cy, cz);
    f[ORC_V] = field_layout(&off, cx, cy + 1, cz);
    f[ORC_W] = field_layout(&off, cx, cy, cz + 1);
    f[ORC_DIV] = field_layout(&off, cx, cy, cz);
    f[ORC_TMP0] = field_layout(&off, cx + 1, cy, cz);
    f[ORC_TMP1] = field_layout(&off, cx, cy + 1, cz);
    f[ORC_TMP2] = field_layout(&off, cx, cy, cz + 1);
    return off;
}

int64_t orc_mac_bytes(int64_t nx, int64_t ny, int64_t nz, int64_t ghost) {
    if (nx < 1 || ny < 1 || nz < 1 || ghost < 1) return 0;
    orc_field f[ORC_NFIELDS];
    return mac_layout(nx, ny, nz, ghost, f);
}

/* Planted mistakes for the oracle's self-checks (0: none); see the header. */
static int g_orc_mut = 0;
void orc_set_mutation(int m) { g_orc_mut = m; }

static inline double* D(orc_engine* e, int id) { return (double*)(e->arena + e->f[id].off); }
static inline int64_t IX(const orc_field* f, int64_t x, int64_t y, int64_t z) { return x + y * f->sy + z * f->sz; }

/* ------------------------------------------------------------------------ */
/* Worker pool and dispatch, aeroflux.go:218-324                             */
/* ------------------------------------------------------------------------ */

typedef struct { orc_engine* e; int id; } thread_arg;

static void run_shard(orc_engine* e, int id) {
    worker_slot* s = &e->slots[id];
    s->faulted = e->fn(e, &e->shards[id], s->msg, sizeof s->msg) != 0;
}

static void* worker_main(void* p) {
    thread_arg* ta = (thread_arg*)p;
    orc_engine* e = ta->e;
    int id = ta->id;
    free(ta);
    uint64_t seen = 0;
    for (;;) {
        pthread_mutex_lock(&e->mu);
        while (e->gen == seen && !e->quit) pthread_cond_wait(&e->cv_work, &e->mu);
        if (e->quit) { pthread_mutex_unlock(&e->mu); return NULL; }
        seen = e->gen;
        pthread_mutex_unlock(&e->mu);
        run_shard(e, id);
        pthread_mutex_lock(&e->mu);
        if (--e->pending == 0) pthread_cond_signal(&e->cv_done);
        pthread_mutex_unlock(&e->mu);
    }
}

/* dispatch: run fn on every shard, join, and return the error of the
 * lowest-numbered worker that faulted (aeroflux.go:313-324 drains the done
 * channels in worker order and keeps the first non-nil). */
static int dispatch(orc_engine* e, shard_fn fn, char* err, size_t errlen) {
    e->fn = fn;
    if (e->nw == 1) {
        run_shard(e, 0);
    } else {
        pthread_mutex_lock(&e->mu);
        e->pending = e->nw - 1;
        e->gen++;
        pthread_cond_broadcast(&e->cv_work);
        pthread_mutex_unlock(&e->mu);
        run_shard(e, 0);
        pthread_mutex_lock(&e->mu);
        while (e->pending) pthread_cond_wait(&e->cv_done, &e->mu);
        pthread_mutex_unlock(&e->mu);
    }
    for (int i = 0; i < e->nw; ++i)
        if (e->slots[i].faulted) return fail(err, errlen, "%s", e->slots[i].msg);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Advection + diffusion, stencil.go:21-225                                  */
/* ------------------------------------------------------------------------ */

/* amd64 CVTTSD2SQ: truncate toward zero; NaN and out-of-range give INT64_MIN. */
static inline int64_t go_float_to_int(double v) {
    if (isnan(v) || v >= 9223372036854775808.0 || v < -9223372036854775808.0) return INT64_MIN;
    return (int64_t)v;
}

/* Go int arithmetic wraps modulo 2^64. */
static inline int64_t wadd(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
static inline int64_t wmul(int64_t a, int64_t b) { return (int64_t)((uint64_t)a * (uint64_t)b); }

/* Go's slice bounds check: returns nonzero and fills the runtime error text
 * (runtime/error.go boundsError, boundsIndex) when idx is out of [0,len). */
static int bounds_fault(int64_t idx, int64_t len, char* msg, size_t msglen) {
    if (idx >= 0 && idx < len) return 0;
    if (idx < 0)
        snprintf(msg, msglen, "aeroflux: guard-page fault contained: runtime error: index out of range [%lld]",
                 (long long)idx);
    else
        snprintf(msg, msglen,
                 "aeroflux: guard-page fault contained: runtime error: index out of range [%lld] with length %lld",
                 (long long)idx, (long long)len);
    return 1;
}

/* faceVelocity, stencil.go:128-155: only the component along the active axis
 * feeds the backtrace, and computing the others has no side effects. */
static inline double face_velocity_axis(orc_engine* e, int c, int ax, int64_t x, int64_t y, int64_t z) {
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    const double* u = D(e, ORC_U);
    const double* v = D(e, ORC_V);
    const double* w = D(e, ORC_W);
    switch (c) {
    case COMP_U:
        if (ax == AXIS_X) return u[IX(fu, x, y, z)];
        if (ax == AXIS_Y)
            return 0.25 * (v[IX(fv, x - 1, y, z)] + v[IX(fv, x, y, z)] + v[IX(fv, x - 1, y + 1, z)] +
                           v[IX(fv, x, y + 1, z)]);
        return 0.25 * (w[IX(fw, x - 1, y, z)] + w[IX(fw, x, y, z)] + w[IX(fw, x - 1, y, z + 1)] +
                       w[IX(fw, x, y, z + 1)]);
    case COMP_V:
        if (ax == AXIS_X)
            return 0.25 * (u[IX(fu, x, y - 1, z)] + u[IX(fu, x + 1, y - 1, z)] + u[IX(fu, x, y, z)] +
                           u[IX(fu, x + 1, y, z)]);
        if (ax == AXIS_Y) return v[IX(fv, x, y, z)];
        return 0.25 * (w[IX(fw, x, y - 1, z)] + w[IX(fw, x, y, z)] + w[IX(fw, x, y - 1, z + 1)] +
                       w[IX(fw, x, y, z + 1)]);
    default:
        if (ax == AXIS_X)
            return 0.25 * (u[IX(fu, x, y, z - 1)] + u[IX(fu, x + 1, y, z - 1)] + u[IX(fu, x, y, z)] +
                           u[IX(fu, x + 1, y, z)]);
        if (ax == AXIS_Y)
            return 0.25 * (v[IX(fv, x, y, z - 1)] + v[IX(fv, x, y + 1, z - 1)] + v[IX(fv, x, y, z)] +
                           v[IX(fv, x, y + 1, z)]);
        return w[IX(fw, x, y, z)];
    }
}

/* sampleTrilinear, stencil.go:169-225.  Returns nonzero on a contained fault. */
static inline int sample_trilinear(const orc_field* f, const double* d, double px, double py, double pz,
                                   double* out, char* msg, size_t msglen) {
    double maxX = (double)(f->nx - 1);
    double maxY = (double)(f->ny - 1);
    double maxZ = (double)(f->nz - 1);
    if (px < 0) px = 0; else if (px > maxX) px = maxX;
    if (py < 0) py = 0; else if (py > maxY) py = maxY;
    if (pz < 0) pz = 0; else if (pz > maxZ) pz = maxZ;
    int64_t x0 = go_float_to_int(px);
    int64_t y0 = go_float_to_int(py);
    int64_t z0 = go_float_to_int(pz);
    if (x0 >= f->nx - 1) x0 = f->nx - 2;
    if (y0 >= f->ny - 1) y0 = f->ny - 2;
    if (z0 >= f->nz - 1) z0 = f->nz - 2;
    double tx = px - (double)x0;
    double ty = py - (double)y0;
    double tz = pz - (double)z0;
    int64_t i000 = wadd(wadd(x0, wmul(y0, f->sy)), wmul(z0, f->sz));
    int64_t i100 = wadd(i000, 1);
    int64_t i010 = wadd(i000, f->sy);
    int64_t i110 = wadd(i010, 1);
    int64_t i001 = wadd(i000, f->sz);
    int64_t i101 = wadd(i001, 1);
    int64_t i011 = wadd(i001, f->sy);
    int64_t i111 = wadd(i011, 1);
    /* Go evaluates (and bounds-checks) the taps in source order. */
    const int64_t order[8] = {i000, i100, i010, i110, i001, i101, i011, i111};
    for (int k = 0; k < 8; ++k)
        if (bounds_fault(order[k], f->count, msg, msglen)) return 1;
    double c00 = d[i000] * (1 - tx) + d[i100] * tx;
    double c10 = d[i010] * (1 - tx) + d[i110] * tx;
    double c01 = d[i001] * (1 - tx) + d[i101] * tx;
    double c11 = d[i011] * (1 - tx) + d[i111] * tx;
    if (g_orc_mut == 2) { /* a contracting compiler's x * y + z */
        c00 = fma(d[i100], tx, d[i000] * (1 - tx));
        c10 = fma(d[i110], tx, d[i010] * (1 - tx));
        c01 = fma(d[i101], tx, d[i001] * (1 - tx));
        c11 = fma(d[i111], tx, d[i011] * (1 - tx));
    }
    double c0 = c00 * (1 - ty) + c10 * ty;
    double c1 = c01 * (1 - ty) + c11 * ty;
    *out = c0 * (1 - tz) + c1 * tz;
    return 0;
}

/* advectComponent, stencil.go:44-119, into dd (laid out as dst); with
 * diffuse = 0 the diffusion term is skipped (lam = 0: the MacCormack forward
 * step). */
static int advect_component_into(orc_engine* e, const shard* s, int src_id, double* dd, const orc_field* dst,
                                 int c, int ax, double dt, int diffuse, char* msg, size_t msglen) {
    const orc_field* src = &e->f[src_id];
    double h = e->H;
    double invH = 1.0 / h;
    double nu = e->cfg.viscosity;
    const double* sd = D(e, src_id);
    int64_t g = e->G;
    int64_t x0 = g, x1 = g + e->NX;
    int64_t y0 = g, y1 = g + e->NY;
    int64_t z0 = s->z0, z1 = s->z1;
    switch (c) {
    case COMP_U: x1++; break;
    case COMP_V: y1++; break;
    default:
        if (s->z1 == g + e->NZ) z1++;
    }
    double lam = diffuse ? nu * dt * invH * invH : 0.0;
    for (int64_t z = z0; z < z1; ++z) {
        for (int64_t y = y0; y < y1; ++y) {
            int64_t base = IX(src, 0, y, z);
            int64_t dbase = IX(dst, 0, y, z);
            for (int64_t x = x0; x < x1; ++x) {
                int64_t i = base + x;
                double vel = face_velocity_axis(e, c, ax, x, y, z);
                double px = (double)x, py = (double)y, pz = (double)z;
                switch (ax) {
                case AXIS_X: px -= dt * vel * invH; break;
                case AXIS_Y: py -= dt * vel * invH; break;
                default: pz -= dt * vel * invH; break;
                }
                double adv;
                if (sample_trilinear(src, sd, px, py, pz, &adv, msg, msglen)) return 1;
                double lap = 0;
                if (lam != 0) {
                    int64_t im, ip;
                    switch (ax) {
                    case AXIS_X: im = i - 1; ip = i + 1; break;
                    case AXIS_Y: im = i - src->sy; ip = i + src->sy; break;
                    default: im = i - src->sz; ip = i + src->sz; break;
                    }
                    lap = lam * (sd[im] - 2 * sd[i] + sd[ip]);
                }
                dd[dbase + x] = adv + lap;
            }
        }
    }
    return 0;
}

static int advect_component(orc_engine* e, const shard* s, int src_id, int dst_id, int c, int ax, double dt,
                            char* msg, size_t msglen) {
    return advect_component_into(e, s, src_id, D(e, dst_id), &e->f[dst_id], c, ax, dt, 1, msg, msglen);
}

/* advectDiffuseAxis, stencil.go:21-25: a fault in one component aborts the
 * rest of the shard's work, as the panic would. */
static int sweep_fn(orc_engine* e, const shard* s, char* msg, size_t msglen) {
    if (advect_component(e, s, ORC_U, ORC_TMP0, COMP_U, e->cur_axis, e->cur_dt, msg, msglen)) return 1;
    if (advect_component(e, s, ORC_V, ORC_TMP1, COMP_V, e->cur_axis, e->cur_dt, msg, msglen)) return 1;
    if (advect_component(e, s, ORC_W, ORC_TMP2, COMP_W, e->cur_axis, e->cur_dt, msg, msglen)) return 1;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MacCormack advection: the engine's optional higher-order sweep (Selle,    */
/* Fedkiw, Kim, Liu, Rossignac, J. Sci. Comput. 2008), restated in the       */
/* binary64 operation order of the engine's kernel, one sweep axis at a time: */
/* the forward step is the reference sweep without diffusion into scratch    */
/* (phi^); each face then traces its velocity forward through phi^ (taps     */
/* outside the faces the sweep writes read phi), forms phi^ + (phi - phi~)/2, */
/* falls back to phi^ outside the range of the two source values the forward */
/* step interpolated, and adds the reference's diffusion of phi.             */
/* ------------------------------------------------------------------------ */
static int mc_forward_fn(orc_engine* e, const shard* s, char* msg, size_t msglen) {
    for (int c = 0; c < 3; ++c)
        if (advect_component_into(e, s, ORC_U + c, e->mc[c], &e->f[ORC_U + c], c, e->cur_axis, e->cur_dt, 0, msg,
                                  msglen))
            return 1;
    return 0;
}

static void maccormack_component(orc_engine* e, const shard* s, int c, int ax, double dt) {
    const orc_field* src = &e->f[ORC_U + c];
    const orc_field* dst = &e->f[ORC_TMP0 + c];
    const double* sd = D(e, ORC_U + c);
    const double* fd = e->mc[c];
    double* dd = D(e, ORC_TMP0 + c);
    double invH = 1.0 / e->H;
    double lam = e->cfg.viscosity * dt * invH * invH;
    int64_t g = e->G;
    int64_t x1 = g + e->NX + (c == COMP_U), y1 = g + e->NY + (c == COMP_V);
    int64_t z0 = s->z0, z1 = s->z1;
    if (c == COMP_W && s->z1 == g + e->NZ) z1++;
    /* the faces the sweep writes along the axis: lo .. hi */
    int64_t lo = g, hi = ax == AXIS_X ? x1 - 1 : (ax == AXIS_Y ? y1 - 1 : g + e->NZ + (c == COMP_W) - 1);
    int64_t step = ax == AXIS_X ? 1 : (ax == AXIS_Y ? src->sy : src->sz);
    int64_t na = ax == AXIS_X ? src->nx : (ax == AXIS_Y ? src->ny : src->nz);
    double maxA = (double)(na - 1);
    for (int64_t z = z0; z < z1; ++z)
        for (int64_t y = g; y < y1; ++y)
            for (int64_t x = g; x < x1; ++x) {
                int64_t i = IX(src, x, y, z);
                double fwd = fd[i];
                double lap = 0.0;
                if (lam != 0) lap = lam * (sd[i - step] - 2 * sd[i] + sd[i + step]);
                double shift = dt * face_velocity_axis(e, c, ax, x, y, z) * invH;
                int64_t ca = ax == AXIS_X ? x : (ax == AXIS_Y ? y : z);
                double pf = (double)ca - shift, pb = (double)ca + shift;
                if (isnan(pf) || isnan(pb)) {
                    dd[IX(dst, x, y, z)] = fwd + lap;
                    continue;
                }
                pf = fmin(fmax(pf, 0.0), maxA);
                pb = fmin(fmax(pb, 0.0), maxA);
                int64_t f0 = (int64_t)pf, b0 = (int64_t)pb;
                if (f0 >= na - 1) f0 = na - 2;
                if (b0 >= na - 1) b0 = na - 2;
                int64_t base = i - ca * step;
                double s0 = sd[base + f0 * step], s1 = sd[base + (f0 + 1) * step];
                double mn = fmin(s0, s1), mx = fmax(s0, s1);
                double h0 = (b0 >= lo && b0 <= hi) ? fd[base + b0 * step] : sd[base + b0 * step];
                double h1 = (b0 + 1 >= lo && b0 + 1 <= hi) ? fd[base + (b0 + 1) * step] : sd[base + (b0 + 1) * step];
                double tb = pb - (double)b0;
                double back = h0 * (1.0 - tb) + h1 * tb;
                double out = fwd + 0.5 * (sd[i] - back);
                if (!(out >= mn && out <= mx)) out = fwd;
                dd[IX(dst, x, y, z)] = out + lap;
            }
}

static int mc_correct_fn(orc_engine* e, const shard* s, char* msg, size_t msglen) {
    (void)msg;
    (void)msglen;
    for (int c = 0; c < 3; ++c) maccormack_component(e, s, c, e->cur_axis, e->cur_dt);
    return 0;
}

int orc_set_advection(orc_engine* e, int scheme) {
    if (scheme != ORC_ADVECTION_SEMI_LAGRANGIAN && scheme != ORC_ADVECTION_MACCORMACK) return -1;
    if (scheme == ORC_ADVECTION_MACCORMACK && !e->mc[0])
        for (int c = 0; c < 3; ++c) {
            e->mc[c] = (double*)calloc((size_t)e->f[ORC_U + c].count, sizeof(double));
            if (!e->mc[c]) return -1;
        }
    e->advection = scheme;
    return 0;
}

/* One axis sweep of the current scheme into Tmp (before commitVelocity). */
static int sweep_phase(orc_engine* e, char* err, size_t errlen) {
    if (e->advection == ORC_ADVECTION_MACCORMACK) {
        if (dispatch(e, mc_forward_fn, err, errlen)) return -1;
        return dispatch(e, mc_correct_fn, err, errlen);
    }
    return dispatch(e, sweep_fn, err, errlen);
}

/* commitVelocity, stencil.go:230-235: descriptor swap. */
static void commit_velocity(orc_engine* e) {
    orc_field t;
    t = e->f[ORC_U]; e->f[ORC_U] = e->f[ORC_TMP0]; e->f[ORC_TMP0] = t;
    t = e->f[ORC_V]; e->f[ORC_V] = e->f[ORC_TMP1]; e->f[ORC_TMP1] = t;
    t = e->f[ORC_W]; e->f[ORC_W] = e->f[ORC_TMP2]; e->f[ORC_TMP2] = t;
}

void orc_commit_velocity(orc_engine* e) { commit_velocity(e); }

/* applyVelocityBC, stencil.go:246-315 (serial, in the reference's loop order). */
void orc_apply_velocity_bc(orc_engine* e) {
    int64_t g = e->G;
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    double* u = D(e, ORC_U);
    double* v = D(e, ORC_V);
    double* w = D(e, ORC_W);
    int64_t ux0 = g, ux1 = g + e->NX;
    int64_t y0 = g, y1 = g + e->NY;
    int64_t z0 = g, z1 = g + e->NZ;
    int64_t NX = e->NX;
    for (int64_t z = z0; z < z1; ++z)
        for (int64_t y = y0; y < y1; ++y) {
            u[IX(fu, ux0, y, z)] = 0;
            u[IX(fu, ux1, y, z)] = 0;
        }
    for (int64_t z = z0; z < z1; ++z)
        for (int64_t x = g; x < g + NX; ++x) {
            v[IX(fv, x, y0, z)] = 0;
            v[IX(fv, x, y1, z)] = 0;
        }
    for (int64_t y = y0; y < y1; ++y)
        for (int64_t x = g; x < g + NX; ++x) {
            w[IX(fw, x, y, z0)] = 0;
            w[IX(fw, x, y, z1)] = 0;
        }
    for (int pass = 0; pass < 2; ++pass) {
        /* stencil.go:279-284 then 285-290; mutation 1 swaps them. */
        if ((pass == 0) == (g_orc_mut != 1)) {
            for (int64_t z = z0; z < z1; ++z)
                for (int64_t x = ux0; x <= ux1; ++x) {
                    u[IX(fu, x, y0 - 1, z)] = -u[IX(fu, x, y0, z)];
                    u[IX(fu, x, y1, z)] = -u[IX(fu, x, y1 - 1, z)];
                }
        } else {
            for (int64_t y = y0 - 1; y <= y1; ++y)
                for (int64_t x = ux0; x <= ux1; ++x) {
                    u[IX(fu, x, y, z0 - 1)] = -u[IX(fu, x, y, z0)];
                    u[IX(fu, x, y, z1)] = -u[IX(fu, x, y, z1 - 1)];
                }
        }
    }
    for (int64_t z = z0; z < z1; ++z)
        for (int64_t y = y0; y <= y1; ++y) {
            v[IX(fv, g - 1, y, z)] = -v[IX(fv, g, y, z)];
            v[IX(fv, g + NX, y, z)] = -v[IX(fv, g + NX - 1, y, z)];
        }
    for (int64_t y = y0; y <= y1; ++y)
        for (int64_t x = g - 1; x <= g + NX; ++x) {
            v[IX(fv, x, y, z0 - 1)] = -v[IX(fv, x, y, z0)];
            v[IX(fv, x, y, z1)] = -v[IX(fv, x, y, z1 - 1)];
        }
    for (int64_t z = z0; z <= z1; ++z)
        for (int64_t y = y0; y < y1; ++y) {
            w[IX(fw, g - 1, y, z)] = -w[IX(fw, g, y, z)];
            w[IX(fw, g + NX, y, z)] = -w[IX(fw, g + NX - 1, y, z)];
        }
    for (int64_t z = z0; z <= z1; ++z)
        for (int64_t x = g - 1; x <= g + NX; ++x) {
            w[IX(fw, x, y0 - 1, z)] = -w[IX(fw, x, y0, z)];
            w[IX(fw, x, y1, z)] = -w[IX(fw, x, y1 - 1, z)];
        }
}

/* ------------------------------------------------------------------------ */
/* Projection, project.go:12-205                                             */
/* ------------------------------------------------------------------------ */

/* computeDivergence, project.go:42-62. */
static int div_fn(orc_engine* e, const shard* s, char* msg, size_t msglen) {
    (void)msg; (void)msglen;
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    const orc_field* fd = &e->f[ORC_DIV];
    const double* u = D(e, ORC_U);
    const double* v = D(e, ORC_V);
    const double* w = D(e, ORC_W);
    double* dv = D(e, ORC_DIV);
    double scale = e->cfg.density / (e->cfg.dt * e->H);
    int64_t g = e->G;
    for (int64_t z = s->z0; z < s->z1; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x) {
                double du = u[IX(fu, x + 1, y, z)] - u[IX(fu, x, y, z)];
                double dvv = v[IX(fv, x, y + 1, z)] - v[IX(fv, x, y, z)];
                double dw = w[IX(fw, x, y, z + 1)] - w[IX(fw, x, y, z)];
                dv[IX(fd, x, y, z)] = scale * (du + dvv + dw);
            }
    return 0;
}

/* gaussSeidelSweep, project.go:103-130. */
static int gs_fn(orc_engine* e, const shard* s, char* msg, size_t msglen) {
    (void)msg; (void)msglen;
    const orc_field* fp = &e->f[ORC_P];
    const orc_field* fd = &e->f[ORC_DIV];
    double* p = D(e, ORC_P);
    const double* dv = D(e, ORC_DIV);
    double h2 = e->H * e->H;
    int64_t g = e->G;
    int64_t sy = fp->sy, sz = fp->sz;
    int col = e->cur_color;
    for (int64_t z = s->z0; z < s->z1; ++z)
        for (int64_t y = g; y < g + e->NY; ++y) {
            int64_t start = g;
            if (((start + y + z) & 1) != col) start++;
            int64_t base = IX(fp, 0, y, z);
            for (int64_t x = start; x < g + e->NX; x += 2) {
                int64_t i = base + x;
                double sum = p[i - 1] + p[i + 1] + p[i - sy] + p[i + sy] + p[i - sz] + p[i + sz];
                if (g_orc_mut == 5) sum = (p[i - 1] + p[i + 1]) + (p[i - sy] + p[i + sy]) + (p[i - sz] + p[i + sz]);
                p[i] = (sum - h2 * dv[IX(fd, x, y, z)]) / 6.0;
            }
        }
    return 0;
}

/* applyPressureBC, project.go:139-163. */
void orc_apply_pressure_bc(orc_engine* e) {
    const orc_field* fp = &e->f[ORC_P];
    double* p = D(e, ORC_P);
    int64_t g = e->G;
    int64_t x1 = g + e->NX, y1 = g + e->NY, z1 = g + e->NZ;
    if (g_orc_mut == 4) /* z-ghosts first: edges and corners read stale ghosts */
        for (int64_t y = g - 1; y <= y1; ++y)
            for (int64_t x = g - 1; x <= x1; ++x) {
                p[IX(fp, x, y, g - 1)] = p[IX(fp, x, y, g)];
                p[IX(fp, x, y, z1)] = p[IX(fp, x, y, z1 - 1)];
            }
    for (int64_t z = g; z < z1; ++z)
        for (int64_t y = g; y < y1; ++y) {
            p[IX(fp, g - 1, y, z)] = p[IX(fp, g, y, z)];
            p[IX(fp, x1, y, z)] = p[IX(fp, x1 - 1, y, z)];
        }
    for (int64_t z = g; z < z1; ++z)
        for (int64_t x = g - 1; x <= x1; ++x) {
            p[IX(fp, x, g - 1, z)] = p[IX(fp, x, g, z)];
            p[IX(fp, x, y1, z)] = p[IX(fp, x, y1 - 1, z)];
        }
    if (g_orc_mut == 4) return;
    for (int64_t y = g - 1; y <= y1; ++y)
        for (int64_t x = g - 1; x <= x1; ++x) {
            p[IX(fp, x, y, g - 1)] = p[IX(fp, x, y, g)];
            p[IX(fp, x, y, z1)] = p[IX(fp, x, y, z1 - 1)];
        }
}

/* solvePressureRedBlack, project.go:73-100. */
void orc_solve_pressure_red_black(orc_engine* e) {
    double* p = D(e, ORC_P);
    int64_t n = e->f[ORC_P].count;
    for (int64_t i = 0; i < n; ++i) p[i] = 0;
    for (int64_t it = 0; it < e->cfg.gauss_seidel_iters; ++it) {
        orc_apply_pressure_bc(e);
        e->cur_color = g_orc_mut == 3 ? COLOR_BLACK : COLOR_RED;
        dispatch(e, gs_fn, NULL, 0);
        orc_apply_pressure_bc(e);
        e->cur_color = g_orc_mut == 3 ? COLOR_RED : COLOR_BLACK;
        dispatch(e, gs_fn, NULL, 0);
    }
    orc_apply_pressure_bc(e);
}

/* subtractGradient, project.go:172-205. */
static int grad_fn(orc_engine* e, const shard* s, char* msg, size_t msglen) {
    (void)msg; (void)msglen;
    const orc_field* fp = &e->f[ORC_P];
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    const double* p = D(e, ORC_P);
    double* u = D(e, ORC_U);
    double* v = D(e, ORC_V);
    double* w = D(e, ORC_W);
    double scale = e->cfg.dt / (e->cfg.density * e->H);
    int64_t g = e->G;
    for (int64_t z = s->z0; z < s->z1; ++z) {
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x <= g + e->NX; ++x)
                u[IX(fu, x, y, z)] -= scale * (p[IX(fp, x, y, z)] - p[IX(fp, x - 1, y, z)]);
        for (int64_t y = g; y <= g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x)
                v[IX(fv, x, y, z)] -= scale * (p[IX(fp, x, y, z)] - p[IX(fp, x, y - 1, z)]);
    }
    int64_t zhi = s->z1;
    if (s->z1 == g + e->NZ) zhi++;
    for (int64_t z = s->z0; z < zhi; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x)
                w[IX(fw, x, y, z)] -= scale * (p[IX(fp, x, y, z)] - p[IX(fp, x, y, z - 1)]);
    return 0;
}

void orc_compute_divergence(orc_engine* e) { dispatch(e, div_fn, NULL, 0); }
void orc_subtract_gradient(orc_engine* e) { dispatch(e, grad_fn, NULL, 0); }

/* project, project.go:12-34 (the Darwin-only direct solve is never enabled). */
int orc_project(orc_engine* e, char* err, size_t errlen) {
    orc_apply_velocity_bc(e);
    if (dispatch(e, div_fn, err, errlen)) return -1;
    orc_solve_pressure_red_black(e);
    if (dispatch(e, grad_fn, err, errlen)) return -1;
    orc_apply_velocity_bc(e);
    return 0;
}

int orc_sweep(orc_engine* e, int axis, double dt, char* err, size_t errlen) {
    e->cur_axis = axis;
    e->cur_dt = dt;
    if (sweep_phase(e, err, errlen)) return -1;
    commit_velocity(e);
    return 0;
}

/* Step, aeroflux.go:348-409: X, Y, Z half-sweeps, project, Z, Y, X, project. */
int orc_step(orc_engine* e, char* err, size_t errlen) {
    static const int fwd[3] = {AXIS_X, AXIS_Y, AXIS_Z};
    static const int rev[3] = {AXIS_Z, AXIS_Y, AXIS_X};
    e->cur_dt = e->cfg.dt * 0.5;
    for (int k = 0; k < 3; ++k) {
        orc_apply_velocity_bc(e);
        e->cur_axis = fwd[k];
        if (sweep_phase(e, err, errlen)) return -1;
        commit_velocity(e);
    }
    if (orc_project(e, err, errlen)) return -1;
    for (int k = 0; k < 3; ++k) {
        orc_apply_velocity_bc(e);
        e->cur_axis = rev[k];
        if (sweep_phase(e, err, errlen)) return -1;
        commit_velocity(e);
    }
    if (orc_project(e, err, errlen)) return -1;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Diagnostics                                                               */
/* ------------------------------------------------------------------------ */

double orc_max_divergence(orc_engine* e) {
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    const double* u = D(e, ORC_U);
    const double* v = D(e, ORC_V);
    const double* w = D(e, ORC_W);
    int64_t g = e->G;
    double invH = 1.0 / e->H;
    double mx = 0;
    for (int64_t z = g; z < g + e->NZ; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x) {
                double d = invH * ((u[IX(fu, x + 1, y, z)] - u[IX(fu, x, y, z)]) +
                                   (v[IX(fv, x, y + 1, z)] - v[IX(fv, x, y, z)]) +
                                   (w[IX(fw, x, y, z + 1)] - w[IX(fw, x, y, z)]));
                double a = fabs(d);
                if (a > mx) mx = a;
            }
    return mx;
}

double orc_kinetic_energy(orc_engine* e) {
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    const double* u = D(e, ORC_U);
    const double* v = D(e, ORC_V);
    const double* w = D(e, ORC_W);
    int64_t g = e->G;
    double vol = e->H * e->H * e->H;
    double sum = 0;
    for (int64_t z = g; z < g + e->NZ; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x) {
                double uc = 0.5 * (u[IX(fu, x, y, z)] + u[IX(fu, x + 1, y, z)]);
                double vc = 0.5 * (v[IX(fv, x, y, z)] + v[IX(fv, x, y + 1, z)]);
                double wc = 0.5 * (w[IX(fw, x, y, z)] + w[IX(fw, x, y, z + 1)]);
                sum += uc * uc + vc * vc + wc * wc;
            }
    return 0.5 * sum * vol;
}

double orc_max_velocity(orc_engine* e) {
    double mx = 0;
    const int ids[3] = {ORC_U, ORC_V, ORC_W};
    for (int k = 0; k < 3; ++k) {
        const double* d = D(e, ids[k]);
        int64_t n = e->f[ids[k]].count;
        for (int64_t i = 0; i < n; ++i) {
            double a = fabs(d[i]);
            if (a > mx) mx = a;
        }
    }
    return mx;
}

double orc_cfl(orc_engine* e) { return orc_max_velocity(e) * e->cfg.dt / e->cfg.h; }

/* ------------------------------------------------------------------------ */
/* The reference's test inputs                                               */
/* ------------------------------------------------------------------------ */

/* seedVortex, engine_test.go:302-335. */
void orc_seed_vortex(orc_engine* e, double amp) {
    int64_t g = e->G;
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    double* u = D(e, ORC_U);
    double* v = D(e, ORC_V);
    double* w = D(e, ORC_W);
    double pi = 3.14159265358979323846;
    double fx = 2 * pi / (double)e->NX;
    double fy = 2 * pi / (double)e->NY;
    double fz = 2 * pi / (double)e->NZ;
    for (int64_t z = g; z < g + e->NZ; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x <= g + e->NX; ++x)
                u[IX(fu, x, y, z)] = amp * sin(fx * (double)(x - g)) * cos(fy * (double)(y - g));
    for (int64_t z = g; z < g + e->NZ; ++z)
        for (int64_t y = g; y <= g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x)
                v[IX(fv, x, y, z)] = -amp * cos(fx * (double)(x - g)) * sin(fy * (double)(y - g));
    for (int64_t z = g; z <= g + e->NZ; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x)
                w[IX(fw, x, y, z)] = 0.25 * amp * sin(fz * (double)(z - g));
    orc_apply_velocity_bc(e);
}

/* PCG32, XSH-RR 64/32 (O'Neill 2014), pcg32_srandom_r seeding; a 53-bit
 * uniform double in [0, 1) from two outputs. */
typedef struct { uint64_t state, inc; } orc_pcg32;
static uint32_t orc_pcg_next(orc_pcg32* r) {
    uint64_t old = r->state;
    r->state = old * 6364136223846793005ull + r->inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
static double orc_pcg_uniform(orc_pcg32* r) {
    uint32_t a = orc_pcg_next(r) >> 5, b = orc_pcg_next(r) >> 6;
    return ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
}

/* The benchmark's synthetic field: Taylor-Green of amplitude amp at the
 * staggered face positions plus uniform [-noise, noise] noise, over
 * seedVortex's index ranges (engine_test.go:313-333) in U, V, W and z, y, x
 * order.  U, V, W are zeroed first; no BC is applied. */
void orc_seed_taylor_green(orc_engine* e, double amp, double noise, uint64_t seed, uint64_t stream) {
    int64_t g = e->G;
    const orc_field* fu = &e->f[ORC_U];
    const orc_field* fv = &e->f[ORC_V];
    const orc_field* fw = &e->f[ORC_W];
    double* u = D(e, ORC_U);
    double* v = D(e, ORC_V);
    double* w = D(e, ORC_W);
    memset(u, 0, sizeof(double) * (size_t)fu->count);
    memset(v, 0, sizeof(double) * (size_t)fv->count);
    memset(w, 0, sizeof(double) * (size_t)fw->count);
    double h = e->cfg.h, twopi = 6.283185307179586;
    orc_pcg32 r = {0u, (stream << 1u) | 1u};
    orc_pcg_next(&r);
    r.state += seed;
    orc_pcg_next(&r);
    for (int64_t z = g; z < g + e->NZ; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x <= g + e->NX; ++x) {
                double X = (double)(x - g) * h, Y = ((double)(y - g) + 0.5) * h, Z = ((double)(z - g) + 0.5) * h;
                u[IX(fu, x, y, z)] = amp * sin(twopi * X) * cos(twopi * Y) * cos(twopi * Z) +
                                     noise * (2.0 * orc_pcg_uniform(&r) - 1.0);
            }
    for (int64_t z = g; z < g + e->NZ; ++z)
        for (int64_t y = g; y <= g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x) {
                double X = ((double)(x - g) + 0.5) * h, Y = (double)(y - g) * h, Z = ((double)(z - g) + 0.5) * h;
                v[IX(fv, x, y, z)] = -amp * cos(twopi * X) * sin(twopi * Y) * cos(twopi * Z) +
                                     noise * (2.0 * orc_pcg_uniform(&r) - 1.0);
            }
    for (int64_t z = g; z <= g + e->NZ; ++z)
        for (int64_t y = g; y < g + e->NY; ++y)
            for (int64_t x = g; x < g + e->NX; ++x) w[IX(fw, x, y, z)] = 0.0 + noise * (2.0 * orc_pcg_uniform(&r) - 1.0);
}

/* Example's shear layer, example_test.go:34-47 (no BC: Step applies it). */
void orc_seed_shear_layer(orc_engine* e) {
    int64_t g = e->G;
    const orc_field* fu = &e->f[ORC_U];
    double* u = D(e, ORC_U);
    for (int64_t z = g; z < g + e->NZ; ++z)
        for (int64_t y = g; y < g + e->NY; ++y) {
            double val = 1.0;
            if (y < g + e->NY / 2) val = -1.0;
            for (int64_t x = g; x <= g + e->NX; ++x) u[IX(fu, x, y, z)] = val;
        }
}

/* ------------------------------------------------------------------------ */
/* Lifecycle, aeroflux.go:176-264,419-439                                    */
/* ------------------------------------------------------------------------ */

orc_engine* orc_new(const orc_config* cin, char* err, size_t errlen) {
    orc_config c = *cin;
    if (orc_normalize(&c, err, errlen)) return NULL;
    int64_t need = orc_mac_bytes(c.nx, c.ny, c.nz, c.ghost);
    if (need <= 0) {
        fail(err, errlen, "aeroflux: could not size grid");
        return NULL;
    }
    orc_engine* e = (orc_engine*)calloc(1, sizeof *e);
    if (!e) { fail(err, errlen, "aeroflux: out of memory"); return NULL; }
    e->cfg = c;
    e->NX = c.nx; e->NY = c.ny; e->NZ = c.nz; e->G = c.ghost; e->H = c.h;
    e->bytes = mac_layout(c.nx, c.ny, c.nz, c.ghost, e->f);
    size_t len = (size_t)need;
    size_t huge = 2u << 20;
    len = (len + huge - 1) / huge * huge;
    void* mem = mmap(NULL, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (mem == MAP_FAILED) {
        free(e);
        fail(err, errlen, "aeroflux: mmap reserve %lld bytes: out of memory", (long long)len);
        return NULL;
    }
    e->arena = (unsigned char*)mem;
    e->arena_len = len;
    e->locked = mlock(mem, len) == 0;
    if (c.lock && !e->locked) {
        munmap(mem, len);
        free(e);
        fail(err, errlen, "aeroflux: mlock requested but unavailable (raise RLIMIT_MEMLOCK)");
        return NULL;
    }
    memset(e->arena, 0, (size_t)e->bytes); /* MAC.Zero, grid.go:158-163 */

    /* partition, aeroflux.go:218-232 */
    e->nw = (int)c.workers;
    e->shards = (shard*)calloc((size_t)e->nw, sizeof(shard));
    e->slots = (worker_slot*)calloc((size_t)e->nw, sizeof(worker_slot));
    int64_t base = c.nz / c.workers, rem = c.nz % c.workers, z = c.ghost;
    for (int i = 0; i < e->nw; ++i) {
        int64_t cnt = base + (i < rem ? 1 : 0);
        e->shards[i].z0 = z;
        e->shards[i].z1 = z + cnt;
        e->shards[i].id = i;
        z += cnt;
    }
    /* start, aeroflux.go:244-264 */
    pthread_mutex_init(&e->mu, NULL);
    pthread_cond_init(&e->cv_work, NULL);
    pthread_cond_init(&e->cv_done, NULL);
    if (e->nw > 1) {
        e->threads = (pthread_t*)calloc((size_t)e->nw, sizeof(pthread_t));
        for (int i = 1; i < e->nw; ++i) {
            thread_arg* ta = (thread_arg*)malloc(sizeof *ta);
            ta->e = e;
            ta->id = i;
            pthread_create(&e->threads[i], NULL, worker_main, ta);
        }
    }
    e->started = 1;
    return e;
}

void orc_close(orc_engine* e) {
    if (!e) return;
    if (e->started && e->nw > 1) {
        pthread_mutex_lock(&e->mu);
        e->quit = 1;
        pthread_cond_broadcast(&e->cv_work);
        pthread_mutex_unlock(&e->mu);
        for (int i = 1; i < e->nw; ++i) pthread_join(e->threads[i], NULL);
    }
    e->started = 0;
    pthread_mutex_destroy(&e->mu);
    pthread_cond_destroy(&e->cv_work);
    pthread_cond_destroy(&e->cv_done);
    if (e->locked) munlock(e->arena, e->arena_len);
    munmap(e->arena, e->arena_len);
    free(e->threads);
    free(e->shards);
    free(e->slots);
    for (int c = 0; c < 3; ++c) free(e->mc[c]);
    free(e);
}

void orc_get_config(const orc_engine* e, orc_config* out) { *out = e->cfg; }

double* orc_field_data(orc_engine* e, int id, orc_field* desc) {
    if (id < 0 || id >= ORC_NFIELDS) return NULL;
    if (desc) *desc = e->f[id];
    return D(e, id);
}

unsigned char* orc_arena(orc_engine* e, int64_t* bytes) {
    if (bytes) *bytes = e->bytes;
    return e->arena;
}
