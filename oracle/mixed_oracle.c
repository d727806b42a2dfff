/*
 * mixed_oracle.c -- CPU restatement of the mixed-precision form.
 *
 * TEST INFRASTRUCTURE ONLY (see mixed_oracle.h).  Build with
 * -ffp-contract=off: every binary32 and binary64 operation below is one IEEE
 * rounding, fused multiply-adds are written as fmaf/fma, and the evaluation
 * order is the CUDA kernels' (aeroflux_gb300/csrc/af_cells.cuh mx_face_vel4,
 * mx_face_update, f64_to_f32; af_batch.cu kb_residual, kb_correct, kb_check,
 * mg_relax, mg_res, mg_interp, kb_vtail).  Which thread computes a cell never
 * matters to those kernels (colour sweeps are order independent within a
 * colour, every other stage writes each cell from values nobody writes in
 * that stage), so plain loops restate them; the two reductions whose order
 * does matter -- the tail V-cycle's means over the coarsest level -- are
 * restated with the kernel's 512-thread partial sums and shuffle trees.
 */
#include "mixed_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int g_mut = 0;
void mxo_set_mutation(int m) { g_mut = m; }

/* ------------------------------------------------------------------------ */
/* Conversions                                                               */
/* ------------------------------------------------------------------------ */

static inline uint64_t dbits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }
static inline double dfrom(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static inline uint32_t fbits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }
static inline float ffrom(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }

float mxo_f64_to_f32(double d) {
    uint64_t b = dbits(d);
    uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    uint32_t sign = hi & 0x80000000u;
    int e = (int)((hi >> 20) & 0x7FF);
    if (e == 0x7FF) return ffrom(sign | 0x7F800000u | (((hi & 0xFFFFFu) | lo) ? 0x400000u : 0u));
    int ef = e - 1023 + 127;
    if (ef <= 0) return ffrom(sign);
    if (ef >= 255) return ffrom(sign | 0x7F800000u);
    uint32_t mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    uint32_t rnd = (lo >> 28) & 1u;
    return ffrom(sign | (((uint32_t)ef << 23) + mant + rnd)); /* a carry rounds into the exponent */
}

double mxo_f32_to_f64(float f) {
    uint32_t u = fbits(f);
    uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xFFu, mant = u & 0x7FFFFFu;
    uint32_t hi, lo = mant << 29;
    if (e == 0) { hi = sign; lo = 0u; }
    else if (e == 0xFF) hi = sign | 0x7FF00000u | (mant >> 3) | (mant ? 0x80000u : 0u);
    else hi = sign | ((e - 127u + 1023u) << 20) | (mant >> 3);
    return dfrom(((uint64_t)hi << 32) | lo);
}

/* ------------------------------------------------------------------------ */
/* The binary32 sweep (stencil.go:44-225 in binary32)                        */
/* ------------------------------------------------------------------------ */

typedef struct { int64_t nx, ny, nz, sy, sz, count; } dims;

static dims field_dims(int comp, int64_t cx, int64_t cy, int64_t cz) {
    dims d;
    d.nx = cx + (comp == 0);
    d.ny = cy + (comp == 1);
    d.nz = cz + (comp == 2);
    d.sy = d.nx;
    d.sz = d.nx * d.ny;
    d.count = d.sz * d.nz;
    return d;
}

/* 0.25 * (((t0 + t1) + t2) + t3). */
static inline float face_vel4(float t0, float t1, float t2, float t3) {
    if (g_mut == 3) return 0.25f * (((t3 + t2) + t1) + t0);
    return 0.25f * (((t0 + t1) + t2) + t3);
}

/* New value of the face at f[0] (neighbours along the axis at f[-s], f[s]):
 * backtrace relative to the face, clamp into the padded field as
 * stencil.go:174-188 clamps, linear interpolation, plus lam times the second
 * difference.  0 on a NaN backtrace. */
static int face_update(const float* f, int64_t s, float vel, int ca, int na, float dt_invh, float lam, float* out) {
    float off = -(vel * dt_invh);
    if (isnan(off)) return 0;
    float fl = floorf(off);
    float pos = (float)ca + off;
    int i0;
    float t;
    if (!(pos > 0.0f)) {
        i0 = 0;
        t = 0.0f;
    } else if (pos >= (float)(na - 1)) {
        i0 = na - 2;
        t = 1.0f;
    } else {
        i0 = ca + (int)fl;
        t = off - fl;
        if (i0 >= na - 1) {
            i0 = na - 2;
            t = 1.0f;
        }
    }
    const float* p0 = f + (int64_t)(i0 - ca) * s;
    float d0 = p0[0], d1 = p0[s];
    float adv = fmaf(t, d1 - d0, d0);
    if (lam != 0.0f) *out = fmaf(lam, (f[-s] - 2.0f * f[0]) + f[s], adv);
    else *out = adv + 0.0f;
    return 1;
}

int64_t mxo_sweep(int64_t NX, int64_t NY, int64_t NZ, int64_t G, int axis, float dt_invh, float lam,
                  const double* u, const double* v, const double* w, double* tu, double* tv, double* tw) {
    const int64_t cx = NX + 2 * G, cy = NY + 2 * G, cz = NZ + 2 * G;
    dims d[3];
    float* sh[3];
    const double* src[3] = {u, v, w};
    double* dst[3] = {tu, tv, tw};
    for (int c = 0; c < 3; ++c) {
        d[c] = field_dims(c, cx, cy, cz);
        sh[c] = (float*)malloc(sizeof(float) * (size_t)d[c].count);
        for (int64_t j = 0; j < d[c].count; ++j) sh[c][j] = mxo_f64_to_f32(src[c][j]);
    }
    int64_t faults = 0;
    const dims a = d[axis];
    for (int c = 0; c < 3; ++c) {
        const dims dc = d[c];
        const int64_t s = axis == 0 ? 1 : (axis == 1 ? dc.sy : dc.sz);
        const int na = (int)(axis == 0 ? dc.nx : (axis == 1 ? dc.ny : dc.nz));
        const float* f = sh[c];
        const float* va = sh[axis];
        for (int64_t z = G; z < G + NZ + (c == 2); ++z)
            for (int64_t y = G; y < G + NY + (c == 1); ++y)
                for (int64_t x = G; x < G + NX + (c == 0); ++x) {
                    const int64_t i = x + y * dc.sy + z * dc.sz;
                    float vel;
                    if (c == axis) {
                        vel = f[i];
                    } else {
#define A(X, Y, Z) va[(X) + (Y) * a.sy + (Z) * a.sz]
                        if (c == 0 && axis == 1) vel = face_vel4(A(x - 1, y, z), A(x, y, z), A(x - 1, y + 1, z), A(x, y + 1, z));
                        else if (c == 0 && axis == 2) vel = face_vel4(A(x - 1, y, z), A(x, y, z), A(x - 1, y, z + 1), A(x, y, z + 1));
                        else if (c == 1 && axis == 0) vel = face_vel4(A(x, y - 1, z), A(x + 1, y - 1, z), A(x, y, z), A(x + 1, y, z));
                        else if (c == 1 && axis == 2) vel = face_vel4(A(x, y - 1, z), A(x, y, z), A(x, y - 1, z + 1), A(x, y, z + 1));
                        else if (c == 2 && axis == 0) vel = face_vel4(A(x, y, z - 1), A(x + 1, y, z - 1), A(x, y, z), A(x + 1, y, z));
                        else vel = face_vel4(A(x, y, z - 1), A(x, y + 1, z - 1), A(x, y, z), A(x, y + 1, z));
#undef A
                    }
                    const int ca = (int)(axis == 0 ? x : (axis == 1 ? y : z));
                    float res;
                    if (!face_update(f + i, s, vel, ca, na, dt_invh, lam, &res)) {
                        ++faults;
                        continue;
                    }
                    dst[c][i] = (double)res; /* widening is exact */
                }
    }
    for (int c = 0; c < 3; ++c) free(sh[c]);
    return faults;
}

/* ------------------------------------------------------------------------ */
/* Multigrid                                                                 */
/* ------------------------------------------------------------------------ */

#define MXO_MAX_LEV 16
#define MXO_TAIL_MAX 4096  /* cells of a level the one-block tail holds */
#define MXO_TAIL_THREADS 512
#define MXO_COARSEST 8

typedef struct {
    int nx, ny, nz;
    float wx, wy, wz;
    int cx, cy, cz;
} lvl;

struct mxo_solver {
    int64_t NX, NY, NZ;
    int nlev, tail, coarse_sweeps;
    lvl L[MXO_MAX_LEV];
    float* e[MXO_MAX_LEV];
    float* r[MXO_MAX_LEV];
    float* rc;  /* the coarsest level's right-hand side as the tail modifies it */
    float* e0;  /* level 0, owned */
    float* r0;
    int nu, max_refine, vcycles;
    double thresh, res_scale, pass_floor;
    /* refinement control (af_batch.cu Ctl) */
    uint64_t maxr_bits;
    unsigned passes, stopped, nv, vtotal;
    double last_div, vfac; /* vfac is kept across projections */
};

static inline int64_t cells(const lvl* L) { return (int64_t)L->nx * L->ny * L->nz; }

/* Coarsen every axis whose extent is even and >= 4 until at most 8 cells
 * remain or no axis halves; an axis of extent 1 has weight 0 unless all do. */
static int plan_levels(int nx, int ny, int nz, lvl* lev, int* coarse_sweeps) {
    int n = 0;
    float wx = 1.0f, wy = 1.0f, wz = 1.0f;
    for (;;) {
        lvl* L = &lev[n++];
        L->nx = nx; L->ny = ny; L->nz = nz;
        L->wx = wx; L->wy = wy; L->wz = wz;
        L->cx = L->cy = L->cz = 0;
        if (g_mut != 4 && (nx > 1 || ny > 1 || nz > 1)) {
            if (nx == 1) L->wx = 0.0f;
            if (ny == 1) L->wy = 0.0f;
            if (nz == 1) L->wz = 0.0f;
        }
        int64_t c = (int64_t)nx * ny * nz;
        int cx = nx % 2 == 0 && nx >= 4, cy = ny % 2 == 0 && ny >= 4, cz = nz % 2 == 0 && nz >= 4;
        if (c <= MXO_COARSEST || !(cx || cy || cz) || n == MXO_MAX_LEV) break;
        L->cx = cx; L->cy = cy; L->cz = cz;
        if (cx) { nx /= 2; wx *= 0.25f; }
        if (cy) { ny /= 2; wy *= 0.25f; }
        if (cz) { nz /= 2; wz *= 0.25f; }
    }
    const lvl* last = &lev[n - 1];
    int nmax = last->nx > last->ny ? last->nx : last->ny;
    if (last->nz > nmax) nmax = last->nz;
    int cs = 2 * nmax * nmax;
    if (cs < 8) cs = 8;
    if (cs > 1000) cs = 1000;
    *coarse_sweeps = cs;
    return n;
}

static int plan_tail(const lvl* lev, int n) {
    if (cells(&lev[n - 1]) > MXO_TAIL_MAX) return -1;
    int t = n - 1;
    while (t > 0 && cells(&lev[t - 1]) <= MXO_TAIL_MAX) --t;
    return t;
}

static inline float inv_diag(const lvl* L) { return 1.0f / (2.0f * (L->wx + L->wy + L->wz)); }

/* c + 1.5 ((wx sx + wy sy + wz sz - r) / (2 (wx + wy + wz)) - c). */
static inline float relax(const lvl* L, float sx, float sy, float sz, float r, float inv, float c) {
    const float v = (fmaf(L->wz, sz, fmaf(L->wy, sy, L->wx * sx)) - r) * inv;
    if (g_mut == 2) return 1.5f * (v - c) + c;
    return fmaf(1.5f, v - c, c);
}

/* r - (wx dxx + wy dyy + wz dzz) of one cell, d** the second differences. */
static inline float cell_res(const lvl* L, float sx, float sy, float sz, float c, float r) {
    const float c2 = 2.0f * c;
    return r - fmaf(L->wz, sz - c2, fmaf(L->wy, sy - c2, L->wx * (sx - c2)));
}

/* Neighbour sums with the Neumann reflection (the cell itself across a wall). */
static inline void nsums(const lvl* L, const float* e, int x, int y, int z, float* sx, float* sy, float* sz) {
    const int64_t nxy = (int64_t)L->nx * L->ny;
    const int64_t i = x + (int64_t)L->nx * y + nxy * z;
    const float c = e[i];
    *sx = (x > 0 ? e[i - 1] : c) + (x < L->nx - 1 ? e[i + 1] : c);
    *sy = (y > 0 ? e[i - L->nx] : c) + (y < L->ny - 1 ? e[i + L->nx] : c);
    *sz = (z > 0 ? e[i - nxy] : c) + (z < L->nz - 1 ? e[i + nxy] : c);
}

/* One colour sweep in place: cells with (x + y + z) & 1 == color. */
static void colour_sweep(const lvl* L, float* e, const float* r, int color) {
    const float inv = inv_diag(L);
    for (int z = 0; z < L->nz; ++z)
        for (int y = 0; y < L->ny; ++y)
            for (int x = ((y + z) & 1) != color ? 1 : 0; x < L->nx; x += 2) {
                const int64_t i = x + (int64_t)L->nx * (y + (int64_t)L->ny * z);
                float sx, sy, sz;
                nsums(L, e, x, y, z, &sx, &sy, &sz);
                e[i] = relax(L, sx, sy, sz, r[i], inv, e[i]);
            }
}

/* `pairs` red-black pairs (red = even x + y + z first). */
static void smooth(const lvl* L, float* e, const float* r, int pairs) {
    for (int k = 0; k < pairs; ++k) {
        colour_sweep(L, e, r, g_mut == 1 ? 1 : 0);
        colour_sweep(L, e, r, g_mut == 1 ? 0 : 1);
    }
}

/* Coarse rhs = mean of the children's residuals, coarse e = 0. */
static void restrict_level(const lvl* F, const lvl* C, const float* ef, const float* rf, float* ec, float* rcs) {
    const int ex = F->cx ? 2 : 1, ey = F->cy ? 2 : 1, ez = F->cz ? 2 : 1;
    const float inv = 1.0f / (float)(ex * ey * ez);
    for (int Z = 0; Z < C->nz; ++Z)
        for (int Y = 0; Y < C->ny; ++Y)
            for (int X = 0; X < C->nx; ++X) {
                float sum = 0.0f;
                for (int dz = 0; dz < ez; ++dz)
                    for (int dy = 0; dy < ey; ++dy)
                        for (int dx = 0; dx < ex; ++dx) {
                            const int x = X * ex + dx, y = Y * ey + dy, z = Z * ez + dz;
                            const int64_t i = x + (int64_t)F->nx * (y + (int64_t)F->ny * z);
                            float sx, sy, sz;
                            nsums(F, ef, x, y, z, &sx, &sy, &sz);
                            sum += cell_res(F, sx, sy, sz, ef[i], rf[i]);
                        }
                const int64_t j = X + (int64_t)C->nx * (Y + (int64_t)C->ny * Z);
                rcs[j] = sum * inv;
                ec[j] = 0.0f;
            }
}

/* Cell-centred trilinear weights: a* on the parent, 1 - a* on its neighbour. */
static inline float interp(float ax, float ay, float az, float e000, float e100, float e010, float e110, float e001,
                           float e101, float e011, float e111) {
    const float bx = 1.0f - ax, by = 1.0f - ay, bz = 1.0f - az;
#define LX(p, q) fmaf(bx, (q), ax * (p))
#define LY(p, q) fmaf(by, (q), ay * (p))
    const float z0 = LY(LX(e000, e100), LX(e010, e110)), z1 = LY(LX(e001, e101), LX(e011, e111));
#undef LX
#undef LY
    return fmaf(bz, z1, az * z0);
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* e_fine += prolongation of e_coarse. */
static void prolong_level(const lvl* F, const lvl* C, float* ef, const float* ec) {
    for (int z = 0; z < F->nz; ++z)
        for (int y = 0; y < F->ny; ++y)
            for (int x = 0; x < F->nx; ++x) {
                int X0 = x, X1 = x, Y0 = y, Y1 = y, Z0 = z, Z1 = z;
                float ax = 1.0f, ay = 1.0f, az = 1.0f;
                if (F->cx) { X0 = x >> 1; X1 = clampi(X0 + ((x & 1) ? 1 : -1), 0, C->nx - 1); ax = 0.75f; }
                if (F->cy) { Y0 = y >> 1; Y1 = clampi(Y0 + ((y & 1) ? 1 : -1), 0, C->ny - 1); ay = 0.75f; }
                if (F->cz) { Z0 = z >> 1; Z1 = clampi(Z0 + ((z & 1) ? 1 : -1), 0, C->nz - 1); az = 0.75f; }
#define E(a, b, c) ec[(a) + (int64_t)C->nx * ((b) + (int64_t)C->ny * (c))]
                const int64_t i = x + (int64_t)F->nx * (y + (int64_t)F->ny * z);
                ef[i] = ef[i] + interp(ax, ay, az, E(X0, Y0, Z0), E(X1, Y0, Z0), E(X0, Y1, Z0), E(X1, Y1, Z0),
                                       E(X0, Y0, Z1), E(X1, Y0, Z1), E(X0, Y1, Z1), E(X1, Y1, Z1));
#undef E
            }
}

/* The tail kernel's block sum: 512 threads, each summing its strided cells
 * in increasing order; xor-shuffle trees per warp, then over the 16 warp
 * sums padded to 32 lanes with zeros. */
static float block_sum512(const float* a, int64_t n) {
    float part[MXO_TAIL_THREADS];
    for (int t = 0; t < MXO_TAIL_THREADS; ++t) {
        float s = 0.0f;
        for (int64_t i = t; i < n; i += MXO_TAIL_THREADS) s += a[i];
        part[t] = s;
    }
    float lanes[32], warp[32];
    for (int w = 0; w < 32; ++w) {
        if (w < MXO_TAIL_THREADS / 32) {
            for (int l = 0; l < 32; ++l) lanes[l] = part[32 * w + l];
            for (int o = 16; o > 0; o >>= 1) {
                float nxt[32];
                for (int l = 0; l < 32; ++l) nxt[l] = lanes[l] + lanes[l ^ o];
                memcpy(lanes, nxt, sizeof lanes);
            }
            warp[w] = lanes[0];
        } else {
            warp[w] = 0.0f;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        float nxt[32];
        for (int l = 0; l < 32; ++l) nxt[l] = warp[l] + warp[l ^ o];
        memcpy(warp, nxt, sizeof warp);
    }
    return warp[0];
}

/* The coarsest level's solve. */
static void coarse_solve(mxo_solver* s, float* e, const float* r) {
    const lvl* C = &s->L[s->nlev - 1];
    const int64_t n = cells(C);
    if (s->tail < 0) {
        /* Too large for one block: smoothed in place, 8 nu pairs. */
        smooth(C, e, r, 8 * s->nu);
        return;
    }
    float* rc = s->rc;
    const float mean_r = block_sum512(r, n) / (float)n;
    for (int64_t i = 0; i < n; ++i) {
        rc[i] = r[i] - mean_r;
        e[i] = 0.0f;
    }
    for (int k = 0; k < s->coarse_sweeps; ++k) {
        colour_sweep(C, e, rc, 0);
        colour_sweep(C, e, rc, 1);
    }
    const float mean_e = block_sum512(e, n) / (float)n;
    for (int64_t i = 0; i < n; ++i) e[i] = e[i] - mean_e;
}

void mxo_vcycle(mxo_solver* s, float* e0, const float* r0) {
    float* e[MXO_MAX_LEV];
    const float* r[MXO_MAX_LEV];
    for (int l = 0; l < s->nlev; ++l) {
        e[l] = l ? s->e[l] : e0;
        r[l] = l ? s->r[l] : r0;
    }
    for (int l = 0; l + 1 < s->nlev; ++l) {
        smooth(&s->L[l], e[l], r[l], s->nu);
        restrict_level(&s->L[l], &s->L[l + 1], e[l], r[l], e[l + 1], s->r[l + 1]);
    }
    coarse_solve(s, e[s->nlev - 1], r[s->nlev - 1]);
    for (int l = s->nlev - 2; l >= 0; --l) {
        prolong_level(&s->L[l], &s->L[l + 1], e[l], e[l + 1]);
        smooth(&s->L[l], e[l], r[l], s->nu);
    }
}

mxo_solver* mxo_solver_new(int64_t NX, int64_t NY, int64_t NZ, int64_t nu, int64_t max_refine, int64_t vcycles,
                           double div_tol, double dt, double density, double h, double pass_floor) {
    mxo_solver* s = (mxo_solver*)calloc(1, sizeof(mxo_solver));
    s->NX = NX; s->NY = NY; s->NZ = NZ;
    s->nlev = plan_levels((int)NX, (int)NY, (int)NZ, s->L, &s->coarse_sweeps);
    s->tail = plan_tail(s->L, s->nlev);
    for (int l = 0; l < s->nlev; ++l) {
        const int64_t n = cells(&s->L[l]);
        s->e[l] = (float*)calloc((size_t)n, sizeof(float));
        s->r[l] = (float*)calloc((size_t)n, sizeof(float));
    }
    s->rc = (float*)calloc((size_t)cells(&s->L[s->nlev - 1]), sizeof(float));
    s->e0 = s->e[0];
    s->r0 = s->r[0];
    s->nu = (int)nu;
    s->max_refine = (int)max_refine;
    s->vcycles = (int)vcycles;
    s->thresh = 0.5 * div_tol;
    s->res_scale = dt / (density * h * h);
    s->pass_floor = pass_floor;
    return s;
}

void mxo_solver_free(mxo_solver* s) {
    if (!s) return;
    for (int l = 0; l < s->nlev; ++l) {
        free(s->e[l]);
        free(s->r[l]);
    }
    free(s->rc);
    free(s);
}

int mxo_solver_levels(const mxo_solver* s, int32_t* nx, int32_t* ny, int32_t* nz, int32_t* cx, int32_t* cy,
                      int32_t* cz, float* wx, float* wy, float* wz, int32_t* tail, int32_t* coarse_sweeps) {
    for (int l = 0; l < s->nlev; ++l) {
        const lvl* L = &s->L[l];
        nx[l] = L->nx; ny[l] = L->ny; nz[l] = L->nz;
        cx[l] = L->cx; cy[l] = L->cy; cz[l] = L->cz;
        wx[l] = L->wx; wy[l] = L->wy; wz[l] = L->wz;
    }
    *tail = s->tail;
    *coarse_sweeps = s->coarse_sweeps;
    return s->nlev;
}

/* ------------------------------------------------------------------------ */
/* Binary64 refinement (kb_residual, kb_correct, kb_check)                   */
/* ------------------------------------------------------------------------ */

/* r = b - L p over the interior (Neumann: the cell itself across a wall),
 * r32 = its binary32 conversion, e = 0, max|r| (NaN counts as +Inf). */
static void residual(mxo_solver* s, int64_t G, const double* p, const double* b) {
    const int64_t NX = s->NX, NY = s->NY, NZ = s->NZ;
    const int64_t sy = NX + 2 * G, sz = sy * (NY + 2 * G);
    uint64_t m = s->maxr_bits;
    for (int64_t z = 0; z < NZ; ++z)
        for (int64_t y = 0; y < NY; ++y)
            for (int64_t x = 0; x < NX; ++x) {
                const int64_t el = x + NX * (y + NY * z);
                const int64_t i = (G + x) + (G + y) * sy + (G + z) * sz;
                const double pc = p[i];
                const double xm = x > 0 ? p[i - 1] : pc;
                const double xp = x < NX - 1 ? p[i + 1] : pc;
                const double ym = y > 0 ? p[i - sy] : pc;
                const double yp = y < NY - 1 ? p[i + sy] : pc;
                const double zm = z > 0 ? p[i - sz] : pc;
                const double zp = z < NZ - 1 ? p[i + sz] : pc;
                const double res = b[i] - fma(-6.0, pc, ((xm + xp) + (ym + yp)) + (zm + zp));
                s->r0[el] = mxo_f64_to_f32(res);
                s->e0[el] = 0.0f;
                const uint64_t a = dbits(res) & ~(1ull << 63);
                const uint64_t v = a > 0x7FF0000000000000ull ? 0x7FF0000000000000ull : a;
                if (v > m) m = v;
            }
    s->maxr_bits = m;
}

static void correct(mxo_solver* s, int64_t G, double* p) {
    const int64_t NX = s->NX, NY = s->NY, NZ = s->NZ;
    const int64_t sy = NX + 2 * G, sz = sy * (NY + 2 * G);
    for (int64_t z = 0; z < NZ; ++z)
        for (int64_t y = 0; y < NY; ++y)
            for (int64_t x = 0; x < NX; ++x) {
                const int64_t i = (G + x) + (G + y) * sy + (G + z) * sz;
                p[i] = p[i] + mxo_f32_to_f64(s->e0[x + NX * (y + NY * z)]);
            }
}

/* Whether another pass runs, and how many V-cycles it needs (kb_check). */
static void check(mxo_solver* s, int count_pass) {
    const double r = dfrom(s->maxr_bits);
    s->maxr_bits = 0;
    if (s->stopped) return;
    const double div = s->res_scale * r;
    const int stalled = count_pass && div > 0.9 * s->last_div;
    const double prev = s->last_div;
    s->last_div = div;
    if (count_pass) s->passes += 1;
    const int more = div > s->thresh && !isinf(div) && !stalled && s->passes < (unsigned)s->max_refine;
    if (count_pass) s->vtotal += s->nv ? s->nv : (unsigned)s->vcycles;
    if (count_pass && prev > 0.0) {
        const double ran = s->nv ? (double)s->nv : (double)s->vcycles;
        const double f = pow(div / prev, 1.0 / ran);
        if (f < 1.0) s->vfac = f;
    }
    unsigned nv = 0u;
    if (more && s->vfac > 0.0 && s->vfac < 1.0) {
        double k = ceil(log(0.5 * s->thresh / div) / log(s->vfac));
        if (s->pass_floor > 0.0) k = fmin(k, ceil(log(s->pass_floor) / log(s->vfac)));
        if (k < 1.0) k = 1.0;
        if (k < (double)s->vcycles) nv = (unsigned)k;
    }
    s->nv = nv;
    if (!more) s->stopped = 1;
}

static void run_pass(mxo_solver* s, int64_t G, double* p, const double* b) {
    for (int vc = 0; vc < s->vcycles; ++vc)
        if (!(s->stopped || (s->nv && (unsigned)vc >= s->nv))) mxo_vcycle(s, s->e0, s->r0);
    if (!s->stopped) {
        correct(s, G, p);
        residual(s, G, p, b);
    }
    check(s, 1);
}

int64_t mxo_refine(mxo_solver* s, int64_t G, double* p, const double* b, int64_t fixed_passes, int64_t* vcycles,
                   double* last_div) {
    s->maxr_bits = 0;
    s->passes = 0;
    s->stopped = 0;
    s->nv = 0;
    s->vtotal = 0;
    s->last_div = 0.0;
    residual(s, G, p, b);
    check(s, 0);
    if (fixed_passes > 0) {
        for (int64_t k = 0; k < fixed_passes; ++k) run_pass(s, G, p, b);
    } else {
        while (!s->stopped) run_pass(s, G, p, b);
    }
    if (vcycles) *vcycles = s->vtotal;
    if (last_div) *last_div = s->last_div;
    return s->passes;
}
