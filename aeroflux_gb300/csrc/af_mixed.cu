// af_mixed.cu -- mixed-precision form of the fractional step for sm_103a.
//
// The velocity state, divergence, pressure accumulator and residual stay in
// binary64; advection/diffusion and the inner pressure solves run in
// binary32:
//
//   sweeps       binary32 arithmetic on binary64 fields.  GB300 issues about
//                two binary64 operations per SM per clock, so every
//                binary64<->binary32 conversion here is done with integer
//                instructions instead of the (FP64-pipe) F2F conversion.
//   projection   p = 0;  r = h^2 Div - L(p) (binary64);  while max|div| >
//                tol/2 and passes < max_refine: e = V-cycles(L e = r) in
//                binary32, p += e (binary64), r = h^2 Div - L(p) (binary64).
//                L is the reference's 7-point operator with the Neumann walls
//                of applyPressureBC (project.go:139-163): a missing
//                neighbour reads the cell itself.  max|div| after the
//                gradient equals dt/(rho h^2) * max|r| (project.go:42-62 and
//                172-205 are adjoint), so the loop tests the residual.
//
// The refinement loop is a WHILE conditional node of the step graph: a
// one-thread kernel sets the condition from the residual and a pass counter,
// so the loop is bounded by max_refine and needs no host round trip.
//
// The inner solver is a geometric multigrid V-cycle whose smoother is the
// reference's red-black Gauss-Seidel update.  A red-black sweep alone damps
// the smooth error modes by ~1-O(h^2) per sweep, so reaching 1e-10 at 256^3
// and above needs the coarse grids; every level coarsens each axis whose
// extent is even and >= 4 (semi-coarsening keeps odd extents), with the
// operator weights (h0/h_axis)^2 carried per level.
#include "af_mixed.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace af {
namespace {

__device__ __forceinline__ bool gated(const Status* st, int gate) {
    return st->fault_gate < st->step * 8u + (unsigned)gate;
}

// binary64 -> binary32 with integer instructions: round half away from zero
// on the magnitude, flush below FLT_MIN to zero, Inf/NaN kept.
__device__ __forceinline__ float f64_to_f32(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FF);
    if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (((hi & 0xFFFFFu) | lo) ? 0x400000u : 0u));
    const int ef = e - 1023 + 127;
    if (ef <= 0) return __uint_as_float(sign);
    if (ef >= 255) return __uint_as_float(sign | 0x7F800000u);
    const unsigned mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned rnd = (lo >> 28) & 1u;
    return __uint_as_float(sign | (((unsigned)ef << 23) + mant + rnd));  // carry may round up into the exponent
}

// binary32 -> binary64 exactly, with integer instructions (subnormal floats
// flush to zero).
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u;
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned mant = u & 0x7FFFFFu;
    unsigned hi, lo = mant << 29;
    if (e == 0) { hi = sign; lo = 0u; }
    else if (e == 0xFF) hi = sign | 0x7FF00000u | (mant >> 3) | (mant ? 0x80000u : 0u);
    else hi = sign | ((e - 127u + 1023u) << 20) | (mant >> 3);
    return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

struct Lvl {
    int nx, ny, nz;
    float wx, wy, wz;   // (h0 / h_axis)^2
    int cx, cy, cz;     // 1 when the axis coarsens into the next level
    float* e;
    float* r;
};

struct Ctl {
    unsigned long long maxr_bits;  // max |r| of the current pass, binary64 bits
    unsigned int passes;
    unsigned int stopped;
    double last_div;               // dt/(rho h^2) * max|r| at the last check
};

// ---------------------------------------------------------------------------
// binary32 sweep (advectDiffuseAxis, stencil.go:21-225, in binary32)
// ---------------------------------------------------------------------------
struct MxSweepArgs {
    const double* u;
    const double* v;
    const double* w;
    double* tu;
    double* tv;
    double* tw;
    Dims du, dv, dw;
    int NX, NY, NZ, G;
    float dt_invh;   // dt / h
    float lam;
    Status* st;
    int phase;
};

template <int AX>
__device__ __forceinline__ float mx_face_vel(const MxSweepArgs& a, int c, int x, int y, int z) {
    auto U = [&](int i, int j, int k) { return f64_to_f32(a.u[i + j * a.du.sy + k * a.du.sz]); };
    auto V = [&](int i, int j, int k) { return f64_to_f32(a.v[i + j * a.dv.sy + k * a.dv.sz]); };
    auto W = [&](int i, int j, int k) { return f64_to_f32(a.w[i + j * a.dw.sy + k * a.dw.sz]); };
    if (c == 0) {
        if (AX == 0) return U(x, y, z);
        if (AX == 1) return 0.25f * (V(x - 1, y, z) + V(x, y, z) + V(x - 1, y + 1, z) + V(x, y + 1, z));
        return 0.25f * (W(x - 1, y, z) + W(x, y, z) + W(x - 1, y, z + 1) + W(x, y, z + 1));
    } else if (c == 1) {
        if (AX == 0) return 0.25f * (U(x, y - 1, z) + U(x + 1, y - 1, z) + U(x, y, z) + U(x + 1, y, z));
        if (AX == 1) return V(x, y, z);
        return 0.25f * (W(x, y - 1, z) + W(x, y, z) + W(x, y - 1, z + 1) + W(x, y, z + 1));
    } else {
        if (AX == 0) return 0.25f * (U(x, y, z - 1) + U(x + 1, y, z - 1) + U(x, y, z) + U(x + 1, y, z));
        if (AX == 1) return 0.25f * (V(x, y, z - 1) + V(x, y + 1, z - 1) + V(x, y, z) + V(x, y + 1, z));
        return W(x, y, z);
    }
}

template <int AX>
__global__ void k_mx_sweep(MxSweepArgs a) {
    if (gated(a.st, a.phase)) return;
    const int zr = a.NZ + 1;
    const int c = blockIdx.z / zr;
    const int z = a.G + (int)(blockIdx.z % zr);
    const int x = a.G + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = a.G + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int x1 = a.G + a.NX + (c == 0), y1 = a.G + a.NY + (c == 1), z1 = a.G + a.NZ + (c == 2);
    if (x >= x1 || y >= y1 || z >= z1) return;
    const Dims& d = c == 0 ? a.du : (c == 1 ? a.dv : a.dw);
    const double* sd = c == 0 ? a.u : (c == 1 ? a.v : a.w);
    double* dd = c == 0 ? a.tu : (c == 1 ? a.tv : a.tw);
    const float vel = mx_face_vel<AX>(a, c, x, y, z);
    // Backtrace relative to the face so binary32 keeps the fraction exact-ish
    // at any grid size: departure = face + off, off = -dt*v/h.
    const int ca = AX == 0 ? x : (AX == 1 ? y : z);
    const int na = AX == 0 ? d.nx : (AX == 1 ? d.ny : d.nz);
    const float off = -(vel * a.dt_invh);
    if (isnan(off)) {
        atomicMin(&a.st->fault_gate, a.st->step * 8u + (unsigned)a.phase);
        atomicMin(&a.st->fault_key, fault_key(c, x, y, z));
        return;
    }
    const float fl = floorf(off);
    int i0;
    float t;
    const float pos = (float)ca + off;
    if (!(pos > 0.0f)) {  // clamp to the padded field (stencil.go:174-188)
        i0 = 0;
        t = 0.0f;
    } else if (pos >= (float)(na - 1)) {
        i0 = na - 2;
        t = 1.0f;
    } else {
        i0 = ca + (int)fl;
        t = off - fl;
        if (i0 >= na - 1) { i0 = na - 2; t = 1.0f; }
    }
    const long long s = AX == 0 ? 1 : (AX == 1 ? d.sy : d.sz);
    const long long base = (long long)x + (long long)y * d.sy + (long long)z * d.sz;
    const long long j0 = base + (long long)(i0 - ca) * s;
    const float d0 = f64_to_f32(sd[j0]), d1 = f64_to_f32(sd[j0 + s]);
    const float adv = fmaf(t, d1 - d0, d0);
    float lap = 0.0f;
    if (a.lam != 0.0f) {
        const float c0 = f64_to_f32(sd[base]);
        lap = a.lam * ((f64_to_f32(sd[base - s]) - 2.0f * c0) + f64_to_f32(sd[base + s]));
    }
    dd[base] = f32_to_f64(adv + lap);
}

// ---------------------------------------------------------------------------
// Refinement: binary64 residual, correction, loop control
// ---------------------------------------------------------------------------
__global__ void k_mx_init(Ctl* ctl) {
    ctl->maxr_bits = 0;
    ctl->passes = 0;
    ctl->stopped = 0;
    ctl->last_div = 0;
}

__device__ __forceinline__ void max_commit(unsigned long long m, unsigned long long* out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// r = b - L(p) over the interior, binary64; stores r (binary32) for the inner
// solve, zeroes the inner solution and reduces max|r|.  A NaN residual is
// recorded as +Inf so the loop stops.
__global__ void k_mx_residual(Geom g, const double* __restrict__ p, const double* __restrict__ b,
                              float* __restrict__ r0, float* __restrict__ e0, Ctl* ctl, Status* st, int gate) {
    if (gated(st, gate)) return;
    const int G = g.G;
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int yi = blockIdx.y;
    const int zi = blockIdx.z;
    unsigned long long m = 0;
    if (xi < g.NX) {
        const int x = G + xi, y = G + yi, z = G + zi;
        const long long sy = g.p.sy, sz = g.p.sz;
        const long long i = x + y * sy + z * sz;
        const double pc = p[i];
        const double xm = xi > 0 ? p[i - 1] : pc;
        const double xp = xi < g.NX - 1 ? p[i + 1] : pc;
        const double ym = yi > 0 ? p[i - sy] : pc;
        const double yp = yi < g.NY - 1 ? p[i + sy] : pc;
        const double zm = zi > 0 ? p[i - sz] : pc;
        const double zp = zi < g.NZ - 1 ? p[i + sz] : pc;
        const double lap = fma(-6.0, pc, ((xm + xp) + (ym + yp)) + (zm + zp));
        const double res = b[i] - lap;
        const long long j = xi + (long long)g.NX * (yi + (long long)g.NY * zi);
        r0[j] = f64_to_f32(res);
        e0[j] = 0.0f;
        const double a = fabs(res);
        m = isnan(a) ? 0x7FF0000000000000ull : (unsigned long long)__double_as_longlong(a);
    }
    max_commit(m, &ctl->maxr_bits);
}

// p += e over the interior (binary64 accumulator).
__global__ void k_mx_correct(Geom g, double* __restrict__ p, const float* __restrict__ e0, Status* st, int gate) {
    if (gated(st, gate)) return;
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    if (xi >= g.NX) return;
    const int yi = blockIdx.y, zi = blockIdx.z;
    const long long i = (g.G + xi) + (g.G + yi) * g.p.sy + (g.G + zi) * g.p.sz;
    const long long j = xi + (long long)g.NX * (yi + (long long)g.NY * zi);
    p[i] += f32_to_f64(e0[j]);
}

// One thread: decide whether another refinement pass runs.  Bounded by
// max_refine, so the WHILE node always terminates.
__global__ void k_mx_check(Ctl* ctl, cudaGraphConditionalHandle h, int use_cond, double scale, double thresh,
                           unsigned max_refine, unsigned count_pass, Status* st, int gate) {
    const double r = __longlong_as_double((long long)ctl->maxr_bits);
    const double div = scale * r;
    ctl->last_div = div;
    ctl->maxr_bits = 0;
    if (count_pass) ctl->passes += 1;
    const bool more = !gated(st, gate) && div > thresh && !isinf(div) && ctl->passes < max_refine;
    if (!more) ctl->stopped = 1;
    if (use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// binary32 multigrid
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long lidx(int x, int y, int z, int nx, int ny) {
    return x + (long long)nx * (y + (long long)ny * z);
}

// Red-black update of L e = r: e = (sum_w neighbours - r) / (2 sum_w), a
// missing neighbour reading the centre (Neumann).
__global__ void k_mg_smooth(Lvl L, int color) {
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (y >= L.ny) return;
    const int x = (((y + z) & 1) != color ? 1 : 0) + 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (x >= L.nx) return;
    const long long nxy = (long long)L.nx * L.ny;
    const long long i = lidx(x, y, z, L.nx, L.ny);
    const float c = L.e[i];
    const float sx = (x > 0 ? L.e[i - 1] : c) + (x < L.nx - 1 ? L.e[i + 1] : c);
    const float sy = (y > 0 ? L.e[i - L.nx] : c) + (y < L.ny - 1 ? L.e[i + L.nx] : c);
    const float sz = (z > 0 ? L.e[i - nxy] : c) + (z < L.nz - 1 ? L.e[i + nxy] : c);
    const float diag = 2.0f * (L.wx + L.wy + L.wz);
    L.e[i] = (L.wx * sx + L.wy * sy + L.wz * sz - L.r[i]) / diag;
}

__device__ __forceinline__ float mg_residual(const Lvl& L, int x, int y, int z) {
    const long long nxy = (long long)L.nx * L.ny;
    const long long i = lidx(x, y, z, L.nx, L.ny);
    const float c = L.e[i];
    const float sx = (x > 0 ? L.e[i - 1] : c) + (x < L.nx - 1 ? L.e[i + 1] : c) - 2.0f * c;
    const float sy = (y > 0 ? L.e[i - L.nx] : c) + (y < L.ny - 1 ? L.e[i + L.nx] : c) - 2.0f * c;
    const float sz = (z > 0 ? L.e[i - nxy] : c) + (z < L.nz - 1 ? L.e[i + nxy] : c) - 2.0f * c;
    return L.r[i] - (L.wx * sx + L.wy * sy + L.wz * sz);
}

// Coarse rhs = mean of the children's residuals; coarse solution = 0.
__global__ void k_mg_restrict(Lvl F, Lvl C) {
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int Y = blockIdx.y, Z = blockIdx.z;
    if (X >= C.nx) return;
    float s = 0.0f;
    const int ex = F.cx ? 2 : 1, ey = F.cy ? 2 : 1, ez = F.cz ? 2 : 1;
    for (int dz = 0; dz < ez; ++dz)
        for (int dy = 0; dy < ey; ++dy)
            for (int dx = 0; dx < ex; ++dx)
                s += mg_residual(F, X * ex + dx, Y * ey + dy, Z * ez + dz);
    const long long j = lidx(X, Y, Z, C.nx, C.ny);
    C.r[j] = s / (float)(ex * ey * ez);
    C.e[j] = 0.0f;
}

// e_fine += trilinear (cell-centred) interpolation of e_coarse; per
// coarsened axis the parent weighs 3/4 and the next coarse cell toward the
// fine cell 1/4 (clamped at the walls).
__global__ void k_mg_prolong(Lvl F, Lvl C) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= F.nx) return;
    int X0 = x, X1 = x, Y0 = y, Y1 = y, Z0 = z, Z1 = z;
    float ax = 1.0f, ay = 1.0f, az = 1.0f;
    if (F.cx) { X0 = x >> 1; X1 = min(max(X0 + ((x & 1) ? 1 : -1), 0), C.nx - 1); ax = 0.75f; }
    if (F.cy) { Y0 = y >> 1; Y1 = min(max(Y0 + ((y & 1) ? 1 : -1), 0), C.ny - 1); ay = 0.75f; }
    if (F.cz) { Z0 = z >> 1; Z1 = min(max(Z0 + ((z & 1) ? 1 : -1), 0), C.nz - 1); az = 0.75f; }
    auto E = [&](int i, int j, int k) { return C.e[lidx(i, j, k, C.nx, C.ny)]; };
    const float bx = 1.0f - ax, by = 1.0f - ay, bz = 1.0f - az;
    const float v = az * (ay * (ax * E(X0, Y0, Z0) + bx * E(X1, Y0, Z0)) + by * (ax * E(X0, Y1, Z0) + bx * E(X1, Y1, Z0))) +
                    bz * (ay * (ax * E(X0, Y0, Z1) + bx * E(X1, Y0, Z1)) + by * (ax * E(X0, Y1, Z1) + bx * E(X1, Y1, Z1)));
    F.e[lidx(x, y, z, F.nx, F.ny)] += v;
}

// Coarsest level in one block: remove the mean of r (the Neumann problem is
// solvable only for zero-mean data), red-black sweeps from zero in shared
// memory, remove the mean of e.  Sums use a fixed tree.
constexpr int kCoarseThreads = 512;
constexpr int kCoarseMax = 4096;

__device__ float block_sum(float v, float* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float s = 0.0f;
    if (threadIdx.x < 32) {
        s = threadIdx.x < kCoarseThreads / 32 ? red[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) red[0] = s;
    }
    __syncthreads();
    s = red[0];
    __syncthreads();
    return s;
}

__global__ void __launch_bounds__(kCoarseThreads) k_mg_coarse(Lvl L, int sweeps) {
    __shared__ float se[kCoarseMax];
    __shared__ float sr[kCoarseMax];
    __shared__ float red[32];
    const int n = L.nx * L.ny * L.nz;
    float part = 0.0f;
    for (int i = threadIdx.x; i < n; i += kCoarseThreads) {
        sr[i] = L.r[i];
        se[i] = 0.0f;
        part += sr[i];
    }
    const float mean_r = block_sum(part, red) / (float)n;
    for (int i = threadIdx.x; i < n; i += kCoarseThreads) sr[i] -= mean_r;
    __syncthreads();
    const float diag = 2.0f * (L.wx + L.wy + L.wz);
    const int nxy = L.nx * L.ny;
    for (int s = 0; s < 2 * sweeps; ++s) {
        const int color = s & 1;
        for (int i = threadIdx.x; i < n; i += kCoarseThreads) {
            const int x = i % L.nx, y = (i / L.nx) % L.ny, z = i / nxy;
            if (((x + y + z) & 1) != color) continue;
            const float c = se[i];
            const float sx = (x > 0 ? se[i - 1] : c) + (x < L.nx - 1 ? se[i + 1] : c);
            const float sy = (y > 0 ? se[i - L.nx] : c) + (y < L.ny - 1 ? se[i + L.nx] : c);
            const float sz = (z > 0 ? se[i - nxy] : c) + (z < L.nz - 1 ? se[i + nxy] : c);
            se[i] = (L.wx * sx + L.wy * sy + L.wz * sz - sr[i]) / diag;
        }
        __syncthreads();
    }
    part = 0.0f;
    for (int i = threadIdx.x; i < n; i += kCoarseThreads) part += se[i];
    const float mean_e = block_sum(part, red) / (float)n;
    for (int i = threadIdx.x; i < n; i += kCoarseThreads) L.e[i] = se[i] - mean_e;
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
// State and host driver
// ---------------------------------------------------------------------------
struct MixedState {
    int nlev = 0;
    Lvl lev[32];
    float* pool = nullptr;
    double* b = nullptr;
    Ctl* ctl = nullptr;
    cudaStream_t body = nullptr;
    int nu = 2;             // red-black pairs before and after each coarse correction
    int vcycles = 2;        // V-cycles per refinement pass
    int coarse_sweeps = 64;
    unsigned max_refine = 30;
    double div_tol = 1e-10;
    int fixed_passes = 0;   // > 0: unrolled loop of exactly this many passes
    cudaError_t capture_err = cudaSuccess;
};

MixedState* mixed_create(const Geom& g, const af_config& c, cudaStream_t s, std::string* err) {
    MixedState* m = new MixedState();
    m->nu = (int)c.inner_sweeps;
    m->max_refine = (unsigned)c.max_refine;
    m->div_tol = c.div_tol;
    // AEROFLUX_FIXED_REFINEMENT_PASSES=n replaces the WHILE node with n
    // unrolled passes (for profilers and drivers without conditional nodes).
    if (const char* fp = getenv("AEROFLUX_FIXED_REFINEMENT_PASSES")) m->fixed_passes = std::max(0, atoi(fp));
    // Levels: coarsen every axis that is even and >= 4 until none is or the
    // grid fits the one-block coarse solver.
    int nx = g.NX, ny = g.NY, nz = g.NZ;
    float wx = 1.0f, wy = 1.0f, wz = 1.0f;
    size_t total = 0;
    while (true) {
        Lvl& L = m->lev[m->nlev++];
        L.nx = nx; L.ny = ny; L.nz = nz;
        L.wx = wx; L.wy = wy; L.wz = wz;
        total += 2 * (size_t)nx * ny * nz;
        const long long cells = (long long)nx * ny * nz;
        L.cx = (nx % 2 == 0 && nx >= 4);
        L.cy = (ny % 2 == 0 && ny >= 4);
        L.cz = (nz % 2 == 0 && nz >= 4);
        if (cells <= kCoarseMax && (cells <= 64 || !(L.cx || L.cy || L.cz))) { L.cx = L.cy = L.cz = 0; break; }
        if (!(L.cx || L.cy || L.cz) || m->nlev == 32) { L.cx = L.cy = L.cz = 0; break; }
        if (L.cx) { nx /= 2; wx *= 0.25f; }
        if (L.cy) { ny /= 2; wy *= 0.25f; }
        if (L.cz) { nz /= 2; wz *= 0.25f; }
    }
    const Lvl& last = m->lev[m->nlev - 1];
    const long long coarsest = (long long)last.nx * last.ny * last.nz;
    if (coarsest > kCoarseMax) {
        // Extents that never halve to a small grid: smooth the last level
        // many times in place of a coarse solve.
        m->coarse_sweeps = 0;
    } else {
        const int nmax = std::max(last.nx, std::max(last.ny, last.nz));
        m->coarse_sweeps = std::min(1000, std::max(8, 2 * nmax * nmax));
    }
    cudaError_t rc;
    if ((rc = cudaMalloc(&m->pool, total * sizeof(float))) != cudaSuccess ||
        (rc = cudaMalloc(&m->b, (size_t)g.p.count * sizeof(double))) != cudaSuccess ||
        (rc = cudaMalloc(&m->ctl, sizeof(Ctl))) != cudaSuccess ||
        (rc = cudaStreamCreateWithFlags(&m->body, cudaStreamNonBlocking)) != cudaSuccess) {
        *err = std::string("aeroflux: mixed-precision scratch: ") + cudaGetErrorString(rc);
        mixed_destroy(m);
        return nullptr;
    }
    float* p = m->pool;
    for (int l = 0; l < m->nlev; ++l) {
        const size_t n = (size_t)m->lev[l].nx * m->lev[l].ny * m->lev[l].nz;
        m->lev[l].e = p;
        m->lev[l].r = p + n;
        p += 2 * n;
    }
    cudaMemsetAsync(m->pool, 0, total * sizeof(float), s);
    cudaMemsetAsync(m->ctl, 0, sizeof(Ctl), s);
    return m;
}

void mixed_destroy(MixedState* m) {
    if (!m) return;
    if (m->body) cudaStreamDestroy(m->body);
    cudaFree(m->pool);
    cudaFree(m->b);
    cudaFree(m->ctl);
    delete m;
}

void launch_sweep_mixed(MixedState* m, const Geom& g, int axis, const Fields& f, double dt, double invH, double lam,
                        Status* st, int phase, cudaStream_t s) {
    (void)m;
    MxSweepArgs a;
    a.u = f.u; a.v = f.v; a.w = f.w;
    a.tu = f.t0; a.tv = f.t1; a.tw = f.t2;
    a.du = g.u; a.dv = g.v; a.dw = g.w;
    a.NX = g.NX; a.NY = g.NY; a.NZ = g.NZ; a.G = g.G;
    a.dt_invh = (float)(dt * invH);
    a.lam = (float)lam;
    a.st = st;
    a.phase = phase;
    dim3 block(64, 4);
    dim3 grid(cdiv(g.NX + 1, 64), cdiv(g.NY + 1, 4), 3 * (g.NZ + 1));
    if (axis == 0) k_mx_sweep<0><<<grid, block, 0, s>>>(a);
    else if (axis == 1) k_mx_sweep<1><<<grid, block, 0, s>>>(a);
    else k_mx_sweep<2><<<grid, block, 0, s>>>(a);
}

namespace {

void smooth(const Lvl& L, int pairs, cudaStream_t s) {
    dim3 block(32, 4);
    dim3 grid(cdiv((L.nx + 1) / 2, 32), cdiv(L.ny, 4), L.nz);
    for (int k = 0; k < pairs; ++k) {
        k_mg_smooth<<<grid, block, 0, s>>>(L, 0);
        k_mg_smooth<<<grid, block, 0, s>>>(L, 1);
    }
}

void vcycle(MixedState* m, cudaStream_t s) {
    for (int l = 0; l + 1 < m->nlev; ++l) {
        smooth(m->lev[l], m->nu, s);
        const Lvl& C = m->lev[l + 1];
        k_mg_restrict<<<dim3(cdiv(C.nx, 128), C.ny, C.nz), 128, 0, s>>>(m->lev[l], C);
    }
    const Lvl& last = m->lev[m->nlev - 1];
    if (m->coarse_sweeps > 0) k_mg_coarse<<<1, kCoarseThreads, 0, s>>>(last, m->coarse_sweeps);
    else smooth(last, 8 * m->nu, s);
    for (int l = m->nlev - 2; l >= 0; --l) {
        const Lvl& F = m->lev[l];
        k_mg_prolong<<<dim3(cdiv(F.nx, 128), F.ny, F.nz), 128, 0, s>>>(F, m->lev[l + 1]);
        smooth(F, m->nu, s);
    }
}

}  // namespace

// projection with binary64 refinement; the enclosing stream must be capturing.
void enqueue_project_mixed(MixedState* m, const Geom& g, const af_config& c, const Fields& f, Status* st, int gate,
                           cudaStream_t s) {
    launch_velocity_bc(g, f.u, f.v, f.w, st, gate, s);
    launch_divergence_fp64(g, f, m->b, c.density / (c.dt * c.h), c.h * c.h, true, st, gate, s);
    const Lvl& L0 = m->lev[0];
    const dim3 rgrid(cdiv(g.NX, 128), g.NY, g.NZ);
    const double scale = c.dt / (c.density * c.h * c.h);
    const double thresh = 0.5 * m->div_tol;
    k_mx_init<<<1, 1, 0, s>>>(m->ctl);
    k_mx_residual<<<rgrid, 128, 0, s>>>(g, f.p, m->b, L0.r, L0.e, m->ctl, st, gate);

    auto pass_body = [&](cudaStream_t bs, cudaGraphConditionalHandle h, int use_cond) {
        // Later cycles continue from the current e0: their restriction takes
        // the residual r0 - L(e0).
        for (int k = 0; k < m->vcycles; ++k) vcycle(m, bs);
        k_mx_correct<<<rgrid, 128, 0, bs>>>(g, f.p, L0.e, st, gate);
        k_mx_residual<<<rgrid, 128, 0, bs>>>(g, f.p, m->b, L0.r, L0.e, m->ctl, st, gate);
        k_mx_check<<<1, 1, 0, bs>>>(m->ctl, h, use_cond, scale, thresh, m->max_refine, 1u, st, gate);
    };
    auto finish = [&]() {
        launch_pressure_bc_fp64(g, f.p, st, gate, s);
        launch_gradient_fp64(g, f, c.dt / (c.density * c.h), st, gate, s);
        launch_velocity_bc(g, f.u, f.v, f.w, st, gate, s);
    };
    if (m->fixed_passes > 0) {
        cudaGraphConditionalHandle none = 0;
        k_mx_check<<<1, 1, 0, s>>>(m->ctl, none, 0, scale, thresh, m->max_refine, 0u, st, gate);
        for (int k = 0; k < m->fixed_passes; ++k) pass_body(s, none, 0);
        finish();
        return;
    }

    // The WHILE node: add it to the capturing graph after the nodes so far.
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaError_t rc = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
    if (rc != cudaSuccess || cs != cudaStreamCaptureStatusActive) {
        m->capture_err = rc != cudaSuccess ? rc : cudaErrorStreamCaptureUnsupported;
        return;
    }
    cudaGraphConditionalHandle h;
    if ((rc = cudaGraphConditionalHandleCreate(&h, graph, 0, cudaGraphCondAssignDefault)) != cudaSuccess) {
        m->capture_err = rc;
        return;
    }
    k_mx_check<<<1, 1, 0, s>>>(m->ctl, h, 1, scale, thresh, m->max_refine, 0u, st, gate);
    rc = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
    if (rc != cudaSuccess) {
        m->capture_err = rc;
        return;
    }
    cudaGraphNodeParams params{cudaGraphNodeTypeConditional};
    params.type = cudaGraphNodeTypeConditional;
    params.conditional.handle = h;
    params.conditional.type = cudaGraphCondTypeWhile;
    params.conditional.size = 1;
    cudaGraphNode_t node;
    if ((rc = cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &params)) != cudaSuccess) {
        m->capture_err = rc;
        return;
    }
    cudaGraph_t body = params.conditional.phGraph_out[0];
    if ((rc = cudaStreamBeginCaptureToGraph(m->body, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess) {
        m->capture_err = rc;
        return;
    }
    pass_body(m->body, h, 1);
    cudaGraph_t body_out = nullptr;
    if ((rc = cudaStreamEndCapture(m->body, &body_out)) != cudaSuccess) {
        m->capture_err = rc;
        return;
    }
    if ((rc = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
        cudaSuccess) {
        m->capture_err = rc;
        return;
    }
    finish();
}

void mixed_stats(MixedState* m, int64_t* passes, double* max_div) {
    Ctl c;
    cudaMemcpy(&c, m->ctl, sizeof c, cudaMemcpyDeviceToHost);
    *passes = c.passes;
    *max_div = c.last_div;
}

cudaError_t mixed_capture_error(MixedState* m) {
    cudaError_t rc = m->capture_err;
    m->capture_err = cudaSuccess;
    return rc;
}

}  // namespace af
