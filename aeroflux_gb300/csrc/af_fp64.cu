// af_fp64.cu -- FP64 plain form of AeroFlux's fractional-step stages for
// sm_103a.  Every kernel reproduces the reference's binary64 arithmetic bit
// for bit: explicit round-to-nearest intrinsics (never contracted into FMA,
// as Go on amd64 never contracts), the reference's left-to-right evaluation
// order, and sign flips done on the sign bit as Go's unary minus does.
//
// The reference runs each stage as a loop nest over Z-slabs with a join
// between phases; here each stage is one grid-wide kernel and the join is the
// kernel boundary.  Every stage is per-cell independent, so results do not
// depend on the launch shape.
#include "../../include/aeroflux_cuda.h"
#include "af_cells.cuh"
#include "af_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <cmath>
#include <mutex>

namespace af {
namespace {

using namespace cells;

// applyVelocityBC, stencil.go:246-315: 3 components x 3 write sets, each cell
// written once (see bc_cell).
__global__ void k_velocity_bc(Geom g, double* u, double* v, double* w, Status* st, int gate) {
    if (gated(st, gate)) return;
    const int comp = blockIdx.y / 3, set = blockIdx.y % 3;
    const BcComp c = bc_comp(g, comp, view(u, g.u.count, DK_F64_BC, 0), view(v, g.v.count, DK_F64_BC, 0),
                             view(w, g.w.count, DK_F64_BC, 0));
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bc_set_count(c, set)) return;
    bc_cell(c, g.G, set, i);
}

// ---------------------------------------------------------------------------
// advectDiffuseAxis / advectComponent / faceVelocity / sampleTrilinear,
// stencil.go:21-225.
// ---------------------------------------------------------------------------
struct SweepArgs {
    AF_PTR(const double) u;
    AF_PTR(const double) v;
    AF_PTR(const double) w;
    AF_PTR(double) tu;
    AF_PTR(double) tv;
    AF_PTR(double) tw;
    Dims du, dv, dw;
    int NX, NY, NZ, G;
    double dt, invH, lam;
    Status* st;
    int phase;
};

// faceVelocity (stencil.go:128-155), only the component on the active axis:
// the other two feed nothing and have no side effects.
template <int AX>
__device__ __forceinline__ double face_vel(const SweepArgs& a, int c, int x, int y, int z) {
    AF_PTR(const double) u = a.u;
    AF_PTR(const double) v = a.v;
    AF_PTR(const double) w = a.w;
    auto U = [&](int i, int j, int k) { return u[i + j * a.du.sy + k * a.du.sz]; };
    auto V = [&](int i, int j, int k) { return v[i + j * a.dv.sy + k * a.dv.sz]; };
    auto W = [&](int i, int j, int k) { return w[i + j * a.dw.sy + k * a.dw.sz]; };
    if (c == 0) {
        if (AX == 0) return U(x, y, z);
        if (AX == 1)
            return quarter(dadd(dadd(dadd(V(x - 1, y, z), V(x, y, z)), V(x - 1, y + 1, z)), V(x, y + 1, z)));
        return quarter(dadd(dadd(dadd(W(x - 1, y, z), W(x, y, z)), W(x - 1, y, z + 1)), W(x, y, z + 1)));
    } else if (c == 1) {
        if (AX == 0)
            return quarter(dadd(dadd(dadd(U(x, y - 1, z), U(x + 1, y - 1, z)), U(x, y, z)), U(x + 1, y, z)));
        if (AX == 1) return V(x, y, z);
        return quarter(dadd(dadd(dadd(W(x, y - 1, z), W(x, y, z)), W(x, y - 1, z + 1)), W(x, y, z + 1)));
    } else {
        if (AX == 0)
            return quarter(dadd(dadd(dadd(U(x, y, z - 1), U(x + 1, y, z - 1)), U(x, y, z)), U(x + 1, y, z)));
        if (AX == 1)
            return quarter(dadd(dadd(dadd(V(x, y, z - 1), V(x, y + 1, z - 1)), V(x, y, z)), V(x, y + 1, z)));
        return W(x, y, z);
    }
}

__device__ __forceinline__ double lerp(double a, double b, double t, double omt) {
    // a*(1-t) + b*t as the reference writes it; omt = 1-t, the same bits the
    // reference recomputes for every lerp
    return dadd(dmul(a, omt), dmul(b, t));
}

// a*(1-t) + b*t for t = +0, with integer instructions: 1-t = 1 exactly, a*1
// is a (NaN stays NaN), b*0 is a zero carrying b's sign when b is finite and
// NaN otherwise, and a + (+-0) is a except that -0 + +0 = +0.
__device__ __forceinline__ double lerp_t0(double a, double b) {
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    const bool b_nonfinite = (ub & 0x7FF0000000000000ull) == 0x7FF0000000000000ull;
    const bool a_nan = (ua & ~kSign) > 0x7FF0000000000000ull;
    if (b_nonfinite || a_nan) return __longlong_as_double(0x7FFFFFFFFFFFFFFFll);
    if ((ua & ~kSign) == 0ull) return __longlong_as_double((long long)(ua & ub & kSign));
    return a;
}

// |v| < 2^1023 on the bit pattern: a lerp of two such values with weights in
// [0, 1] is finite (the result is bounded by the larger magnitude times
// (1-t) + t <= 1 + 2^-53), so it adds as an exact zero when its weight is +0.
__device__ __forceinline__ bool below_2p1023(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7FF0000000000000ull) < 0x7FE0000000000000ull;
}
// Finite and nonzero: x + (+-0) == x and x * 1 == x exactly.
__device__ __forceinline__ bool finite_nonzero(double v) {
    const unsigned long long m = (unsigned long long)__double_as_longlong(v) & ~kSign;
    return m != 0ull && m < 0x7FF0000000000000ull;
}

template <int AX>
__global__ void k_sweep_fp64(SweepArgs a) {
    if (gated(a.st, a.phase)) return;
    const int zr = a.NZ + 1;
    const int c = blockIdx.z / zr;
    const int z = a.G + (int)(blockIdx.z % zr);
    const int x = a.G + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = a.G + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    // Face-count extents of this component (stencil.go:53-68).
    const int x1 = a.G + a.NX + (c == 0), y1 = a.G + a.NY + (c == 1), z1 = a.G + a.NZ + (c == 2);
    if (x >= x1 || y >= y1 || z >= z1) return;

    const Dims& d = c == 0 ? a.du : (c == 1 ? a.dv : a.dw);
    AF_PTR(const double) sd = c == 0 ? a.u : (c == 1 ? a.v : a.w);
    AF_PTR(double) dd = c == 0 ? a.tu : (c == 1 ? a.tv : a.tw);

    const double vel = face_vel<AX>(a, c, x, y, z);
    // Backtrace along the active axis only: p -= dt*v*invH.
    const int ca = AX == 0 ? x : (AX == 1 ? y : z);
    const int na = AX == 0 ? d.nx : (AX == 1 ? d.ny : d.nz);
    double pa = dsub(i2d_small(ca), dmul(dmul(a.dt, vel), a.invH));
    // Clamp to [0, na-1] (pa < 0 and pa > maxA on the bit patterns: -0 and
    // NaN pass through unchanged, as the comparisons leave them).
    const unsigned long long pab = dbits(pa);
    const bool pnan = (pab & ~kSign) > 0x7FF0000000000000ull;
    if (!pnan) {
        if ((pab & kSign) && (pab & ~kSign)) pa = 0.0;
        else if (!(pab & kSign) && pab > dbits(i2d_small(na - 1))) pa = i2d_small(na - 1);
    }

    // Truncation toward zero as amd64 CVTTSD2SQ does (NaN -> INT64_MIN).  The
    // two other coordinates are integer faces strictly inside the padded
    // field, so their floor is the face itself and their weight is +0.
    long long a0 = pnan ? (long long)0x8000000000000000ull : d2i_trunc_small(pa);
    if (a0 >= na - 1) a0 = na - 2;
    const double ta = pnan ? dsub(pa, (double)a0) : frac_sub(pa, a0);
    long long x0 = x, y0 = y, z0 = z;
    double tx = 0.0, ty = 0.0, tz = 0.0;
    if (AX == 0) { x0 = a0; tx = ta; }
    if (AX == 1) { y0 = a0; ty = ta; }
    if (AX == 2) { z0 = a0; tz = ta; }
    // Index arithmetic wraps modulo 2^64, as Go's int does.
    const unsigned long long i000 =
        (unsigned long long)x0 + (unsigned long long)y0 * (unsigned long long)d.sy +
        (unsigned long long)z0 * (unsigned long long)d.sz;
    if (pnan) {
        // Only a NaN coordinate can leave the field; Go bounds-checks the taps
        // in source order and panics at the first out-of-range one.
        const unsigned long long sy = d.sy, sz = d.sz, n = d.count;
        const unsigned long long taps[8] = {i000, i000 + 1, i000 + sy, i000 + sy + 1,
                                            i000 + sz, i000 + sz + 1, i000 + sz + sy, i000 + sz + sy + 1};
        bool oob = false;
#pragma unroll
        for (int k = 0; k < 8; ++k) oob |= (long long)taps[k] < 0 || taps[k] >= n;
        if (oob) {
            atomicMin(&a.st->fault_gate, a.st->step * 8u + (unsigned)a.phase);
            atomicMin(&a.st->fault_key, fault_key(c, x, y, z));
            return;  // the faulting face is not written, as the panic leaves it
        }
    }
    const long long sy = d.sy, sz = d.sz;
    const long long b = (long long)i000;
    // Only the active axis has a nonzero weight; the lerps along the other
    // two (weight exactly +0) run on the integer pipe with identical bits.
    // The zero-weight lerps only matter when their operands are not finite
    // (NaN propagates, Inf * 0 is NaN) or when the kept value is a zero
    // (-0 + +0 = +0): otherwise the kept value passes through exactly, and
    // the FP64 work of the discarded lerps is skipped.
    double adv;
    if (AX == 0) {
        const double omt = dsub(1.0, tx);
        const double c00 = lerp(sd[b], sd[b + 1], tx, omt);
        const double t1 = sd[b + sy], t2 = sd[b + sy + 1], t3 = sd[b + sz], t4 = sd[b + sz + 1];
        const double t5 = sd[b + sz + sy], t6 = sd[b + sz + sy + 1];
        if (finite_nonzero(c00) && below_2p1023(t1) && below_2p1023(t2) && below_2p1023(t3) && below_2p1023(t4) &&
            below_2p1023(t5) && below_2p1023(t6)) {
            adv = c00;
        } else {
            const double c10 = lerp(t1, t2, tx, omt);
            const double c01 = lerp(t3, t4, tx, omt);
            const double c11 = lerp(t5, t6, tx, omt);
            adv = lerp_t0(lerp_t0(c00, c10), lerp_t0(c01, c11));
        }
    } else if (AX == 1) {
        const double omt = dsub(1.0, ty);
        const double c00 = lerp_t0(sd[b], sd[b + 1]);
        const double c10 = lerp_t0(sd[b + sy], sd[b + sy + 1]);
        const double y0 = lerp(c00, c10, ty, omt);
        const double t3 = sd[b + sz], t4 = sd[b + sz + 1], t5 = sd[b + sz + sy], t6 = sd[b + sz + sy + 1];
        // lerp_t0 of values below 2^1023 is one of them or a zero: below too.
        if (finite_nonzero(y0) && below_2p1023(t3) && below_2p1023(t4) && below_2p1023(t5) && below_2p1023(t6)) {
            adv = y0;
        } else {
            const double c01 = lerp_t0(t3, t4);
            const double c11 = lerp_t0(t5, t6);
            adv = lerp_t0(y0, lerp(c01, c11, ty, omt));
        }
    } else {
        const double c00 = lerp_t0(sd[b], sd[b + 1]);
        const double c10 = lerp_t0(sd[b + sy], sd[b + sy + 1]);
        const double c01 = lerp_t0(sd[b + sz], sd[b + sz + 1]);
        const double c11 = lerp_t0(sd[b + sz + sy], sd[b + sz + sy + 1]);
        adv = lerp(lerp_t0(c00, c10), lerp_t0(c01, c11), tz, dsub(1.0, tz));
    }

    const long long i = (long long)x + (long long)y * sy + (long long)z * sz;
    double lap = 0.0;
    if (a.lam != 0) {
        const long long s = AX == 0 ? 1 : (AX == 1 ? sy : sz);
        lap = dmul(a.lam, dadd(dsub(sd[i - s], twice(sd[i])), sd[i + s]));
    }
    dd[i] = dadd(adv, lap);
}

// ---------------------------------------------------------------------------
// MacCormack correction of one axis sweep (Selle, Fedkiw, Kim, Liu, Rossignac,
// "An Unconditionally Stable MacCormack Method", J. Sci. Comput. 2008), the
// higher-order advection the reference lists as its missing remedy for
// semi-Lagrangian dissipation (README "Known limitations").  The forward
// step is the reference sweep itself run with lam = 0 into `fwd` (phi^ =
// semi-Lagrangian advection of the component, faults and all); this kernel
// traces the same face velocity forward (x + dt*v*invH) through phi^ to get
// phi~, forms phi^ + (phi - phi~)/2, falls back to phi^ where that leaves the
// range of the two source values the forward step interpolated (the limiter
// that keeps the scheme unconditionally stable), and adds the reference's
// directional diffusion of phi.  Along the sweep axis only: the tangential
// weights are zero, as in the forward step.  Taps of phi^ outside the faces
// the sweep writes read phi (the boundary-conditioned field) instead.
template <int AX>
__global__ void k_maccormack_fp64(SweepArgs a, const double* fu, const double* fv, const double* fw) {
    if (gated(a.st, a.phase)) return;
    const int zr = a.NZ + 1;
    const int c = blockIdx.z / zr;
    const int z = a.G + (int)(blockIdx.z % zr);
    const int x = a.G + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = a.G + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int x1 = a.G + a.NX + (c == 0), y1 = a.G + a.NY + (c == 1), z1 = a.G + a.NZ + (c == 2);
    if (x >= x1 || y >= y1 || z >= z1) return;

    const Dims& d = c == 0 ? a.du : (c == 1 ? a.dv : a.dw);
    AF_PTR(const double) sd = c == 0 ? a.u : (c == 1 ? a.v : a.w);
    AF_PTR(const double) fd = view(c == 0 ? fu : (c == 1 ? fv : fw), d.count, DK_F64_MACCORMACK, 0);
    AF_PTR(double) dd = c == 0 ? a.tu : (c == 1 ? a.tv : a.tw);
    const long long sy = d.sy, sz = d.sz;
    const long long step = AX == 0 ? 1 : (AX == 1 ? sy : sz);
    const long long i = (long long)x + (long long)y * sy + (long long)z * sz;
    const int ca = AX == 0 ? x : (AX == 1 ? y : z);
    const int na = AX == 0 ? d.nx : (AX == 1 ? d.ny : d.nz);
    const int lo = a.G, hi = AX == 0 ? x1 - 1 : (AX == 1 ? y1 - 1 : z1 - 1);  // written faces on the axis
    const double fwd = fd[i];

    double lap = 0.0;
    if (a.lam != 0) lap = dmul(a.lam, dadd(dsub(sd[i - step], dmul(2.0, sd[i])), sd[i + step]));

    const double shift = dmul(dmul(a.dt, face_vel<AX>(a, c, x, y, z)), a.invH);
    const double maxA = (double)(na - 1);
    // Forward foot (the one the forward step sampled) and backward foot.
    double pf = dsub((double)ca, shift), pb = dadd((double)ca, shift);
    if (isnan(pf) || isnan(pb)) {  // the forward step has dealt with it
        dd[i] = dadd(fwd, lap);
        return;
    }
    pf = fmin(fmax(pf, 0.0), maxA);
    pb = fmin(fmax(pb, 0.0), maxA);
    long long f0 = (long long)pf, b0 = (long long)pb;
    if (f0 >= na - 1) f0 = na - 2;
    if (b0 >= na - 1) b0 = na - 2;
    const long long base = i - (long long)ca * step;  // the face's row at axis coordinate 0
    const double s0 = sd[base + f0 * step], s1 = sd[base + (f0 + 1) * step];
    const double mn = fmin(s0, s1), mx = fmax(s0, s1);
    auto phi_hat = [&](long long k) { return (k >= lo && k <= hi) ? fd[base + k * step] : sd[base + k * step]; };
    const double tb = dsub(pb, (double)b0);
    const double back = dadd(dmul(phi_hat(b0), dsub(1.0, tb)), dmul(phi_hat(b0 + 1), tb));
    double out = dadd(fwd, dmul(0.5, dsub(sd[i], back)));
    if (!(out >= mn && out <= mx)) out = fwd;
    dd[i] = dadd(out, lap);
}


// ---------------------------------------------------------------------------
// solvePressureRedBlack's zeroing (project.go:81-83) fused with
// computeDivergence (project.go:42-62).  Also stores B = h2*Div, the product
// every red-black update recomputes (project.go:126), so the sweeps read it
// instead of multiplying again: same bits, one FP64 multiply fewer per update.
// ---------------------------------------------------------------------------
__global__ void k_divergence_fp64(Geom g, const double* __restrict__ u, const double* __restrict__ v,
                                  const double* __restrict__ w, double* __restrict__ p, double* __restrict__ dv,
                                  double* __restrict__ bb, double scale, double h2, int zero_p, Status* st,
                                  int gate) {
    if (gated(st, gate)) return;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= g.p.nx || y >= g.p.ny) return;
    div_cell(g, view(u, g.u.count, DK_F64_DIV, 0), view(v, g.v.count, DK_F64_DIV, 0),
             view(w, g.w.count, DK_F64_DIV, 0), view(p, g.p.count, DK_F64_DIV, 0),
             view(dv, g.p.count, DK_F64_DIV, 0), view(bb, g.p.count, DK_F64_DIV, 0), scale, h2, zero_p != 0, x,
             y, z);
}

// ---------------------------------------------------------------------------
// gaussSeidelSweep, project.go:103-130, with applyPressureBC folded in.
// Before each colour the reference mirrors the interior into the ghosts
// (project.go:89,93); a face ghost of a cell being updated then holds that
// cell's own pre-update value, so the sweep reads the centre instead and the
// ghosts are materialised once, after the last sweep (k_pressure_bc).
// ---------------------------------------------------------------------------
// EMU selects which of the update's six binary64 add/subtracts run on the
// integer pipe (bit k: operation k of the chain, the subtraction last); the
// others issue on the FP64 pipe.  Every choice computes the same bits.
template <int EMU>
__device__ __forceinline__ double chain_add(int k, double a, double b) {
    return ((EMU >> k) & 1) ? dadd_int(a, b) : dadd(a, b);
}

template <int EMU>
__global__ void k_rbgs_fp64(Geom g, double* __restrict__ p_, const double* __restrict__ bb_, int color,
                            Status* st, int gate) {
    if (gated(st, gate)) return;
    AF_PTR(double) AF_RESTRICT p = view(p_, g.p.count, DK_F64_RBGS, 0);
    AF_PTR(const double) AF_RESTRICT bb = view(bb_, g.p.count, DK_F64_RBGS, 0);
    const int G = g.G;
    const int y = G + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int z = G + (int)blockIdx.z;
    if (y >= G + g.NY) return;
    const int start = (((G + y + z) & 1) != color) ? G + 1 : G;
    const int x = start + 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (x >= G + g.NX) return;
    const long long sy = g.p.sy, sz = g.p.sz;
    const long long i = x + y * sy + z * sz;
    const double pc = p[i];
    const double xm = x > G ? p[i - 1] : pc;
    const double xp = x < G + g.NX - 1 ? p[i + 1] : pc;
    const double ym = y > G ? p[i - sy] : pc;
    const double yp = y < G + g.NY - 1 ? p[i + sy] : pc;
    const double zm = z > G ? p[i - sz] : pc;
    const double zp = z < G + g.NZ - 1 ? p[i + sz] : pc;
    double sum = chain_add<EMU>(0, xm, xp);
    sum = chain_add<EMU>(1, sum, ym);
    sum = chain_add<EMU>(2, sum, yp);
    sum = chain_add<EMU>(3, sum, zm);
    sum = chain_add<EMU>(4, sum, zp);
    const double r = ((EMU >> 5) & 1) ? dsub_int(sum, bb[i]) : dsub(sum, bb[i]);
    p[i] = div6_int(r);
}

// applyPressureBC, project.go:139-163 (see pbc_cell).
__global__ void k_pressure_bc(Geom g, double* __restrict__ p, Status* st, int gate) {
    if (gated(st, gate)) return;
    const int set = blockIdx.y;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pbc_set_count(g, set)) return;
    pbc_cell(g, view(p, g.p.count, DK_F64_PBC, 0), set, i);
}

// subtractGradient, project.go:172-205.
__global__ void k_gradient_fp64(Geom g, const double* __restrict__ p, double* __restrict__ u, double* __restrict__ v,
                                double* __restrict__ w, double scale, Status* st, int gate) {
    if (gated(st, gate)) return;
    const int G = g.G;
    const int zr = g.NZ + 1;
    const int c = blockIdx.z / zr;
    const int z = G + (int)(blockIdx.z % zr);
    const int x = G + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = G + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int x1 = G + g.NX + (c == 0), y1 = G + g.NY + (c == 1), z1 = G + g.NZ + (c == 2);
    if (x >= x1 || y >= y1 || z >= z1) return;
    grad_face(g, view(p, g.p.count, DK_F64_GRAD, 0), view(u, g.u.count, DK_F64_GRAD, 0),
              view(v, g.v.count, DK_F64_GRAD, 0), view(w, g.w.count, DK_F64_GRAD, 0), scale, c, x, y, z);
}

__global__ void k_step_tick(Status* st) { st->step += 1; }

// B = h2*Div over the interior, for the red-black phase hook when Div was
// supplied directly instead of by the divergence kernel.
__global__ void k_b_from_div(Geom g, const double* __restrict__ dv_, double* __restrict__ bb_, double h2) {
    const int G = g.G;
    AF_PTR(const double) AF_RESTRICT dv = view(dv_, g.p.count, DK_F64_B, 0);
    AF_PTR(double) AF_RESTRICT bb = view(bb_, g.p.count, DK_F64_B, 0);
    const int x = G + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = G + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int z = G + (int)blockIdx.z;
    if (x >= G + g.NX || y >= G + g.NY) return;
    const long long i = x + y * g.p.sy + z * g.p.sz;
    bb[i] = dmul(h2, dv[i]);
}

// ---------------------------------------------------------------------------
// Diagnostics.  A max is exact in any order; NaN is skipped as the
// reference's `if a > mx` skips it.  Non-negative doubles order like their
// bit patterns, so one atomicMax per block combines the blocks.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long abs_bits(double d) {
    const double a = fabs(d);
    return isnan(a) ? 0ull : (unsigned long long)__double_as_longlong(a);
}

__device__ __forceinline__ void block_max_commit(unsigned long long m, unsigned long long* out) {
    __shared__ unsigned long long sm[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    if ((tid & 31) == 0) sm[tid >> 5] = m;
    __syncthreads();
    if (tid < 32) {
        m = tid < (nthreads + 31) / 32 ? sm[tid] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
            m = t > m ? t : m;
        }
        if (tid == 0 && m) atomicMax(out, m);
    }
}

// MaxDivergence, project.go:210-232.
__global__ void k_max_divergence(Geom g, const double* __restrict__ u_, const double* __restrict__ v_,
                                 const double* __restrict__ w_, double invH, unsigned long long* out) {
    const int G = g.G;
    AF_PTR(const double) AF_RESTRICT u = view(u_, g.u.count, DK_F64_MAXDIV, 0);
    AF_PTR(const double) AF_RESTRICT v = view(v_, g.v.count, DK_F64_MAXDIV, 0);
    AF_PTR(const double) AF_RESTRICT w = view(w_, g.w.count, DK_F64_MAXDIV, 0);
    const int x = G + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = G + (int)blockIdx.y;
    const int z = G + (int)blockIdx.z;
    unsigned long long m = 0;
    if (x < G + g.NX) {
        const long long iu = x + y * g.u.sy + z * g.u.sz;
        const long long iv = x + y * g.v.sy + z * g.v.sz;
        const long long iw = x + y * g.w.sy + z * g.w.sz;
        const double d = dmul(invH, dadd(dadd(dsub(u[iu + 1], u[iu]), dsub(v[iv + g.v.sy], v[iv])),
                                         dsub(w[iw + g.w.sz], w[iw])));
        m = abs_bits(d);
    }
    block_max_commit(m, out);
}

// MaxVelocity, stencil.go:319-331: every element of U, V, W, ghosts included.
__global__ void k_max_abs3(const double* __restrict__ u_, long long nu, const double* __restrict__ v_, long long nv,
                           const double* __restrict__ w_, long long nw, unsigned long long* out) {
    AF_PTR(const double) AF_RESTRICT u = view(u_, nu, DK_F64_MAXABS, 0);
    AF_PTR(const double) AF_RESTRICT v = view(v_, nv, DK_F64_MAXABS, 0);
    AF_PTR(const double) AF_RESTRICT w = view(w_, nw, DK_F64_MAXABS, 0);
    unsigned long long m = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nu; i += stride) {
        const unsigned long long t = abs_bits(u[i]);
        m = t > m ? t : m;
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
        const unsigned long long t = abs_bits(v[i]);
        m = t > m ? t : m;
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += stride) {
        const unsigned long long t = abs_bits(w[i]);
        m = t > m ? t : m;
    }
    block_max_commit(m, out);
}

// KineticEnergy, project.go:238-258.  The reference sums serially; this sums
// each z-plane in a fixed per-thread order and a fixed shuffle tree, then the
// planes in a fixed tree, so the result depends on the grid only and is
// bit-identical run to run (it differs from the serial sum by rounding).
constexpr int kKeThreads = 256;

__device__ __forceinline__ double block_sum_fixed(double s) {
    __shared__ double sm[kKeThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = dadd(s, __shfl_xor_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    s = threadIdx.x < kKeThreads / 32 ? sm[threadIdx.x] : 0.0;
    if (threadIdx.x < 32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = dadd(s, __shfl_xor_sync(0xffffffffu, s, o));
    }
    return s;
}

__global__ void __launch_bounds__(kKeThreads) k_ke_planes(Geom g, const double* __restrict__ u_,
                                                          const double* __restrict__ v_,
                                                          const double* __restrict__ w_, double* partials_) {
    const int G = g.G;
    AF_PTR(const double) AF_RESTRICT u = view(u_, g.u.count, DK_F64_KE, 0);
    AF_PTR(const double) AF_RESTRICT v = view(v_, g.v.count, DK_F64_KE, 0);
    AF_PTR(const double) AF_RESTRICT w = view(w_, g.w.count, DK_F64_KE, 0);
    AF_PTR(double) partials = view(partials_, (long long)gridDim.x, DK_F64_KE, 0);
    const int z = G + (int)blockIdx.x;
    const long long n = (long long)g.NX * g.NY;
    double s = 0.0;
    for (long long k = threadIdx.x; k < n; k += kKeThreads) {
        const int x = G + (int)(k % g.NX), y = G + (int)(k / g.NX);
        const long long iu = x + y * g.u.sy + z * g.u.sz;
        const long long iv = x + y * g.v.sy + z * g.v.sz;
        const long long iw = x + y * g.w.sy + z * g.w.sz;
        const double uc = dmul(0.5, dadd(u[iu], u[iu + 1]));
        const double vc = dmul(0.5, dadd(v[iv], v[iv + g.v.sy]));
        const double wc = dmul(0.5, dadd(w[iw], w[iw + g.w.sz]));
        s = dadd(s, dadd(dadd(dmul(uc, uc), dmul(vc, vc)), dmul(wc, wc)));
    }
    s = block_sum_fixed(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kKeThreads) k_ke_final(const double* partials_, int n, double* out) {
    AF_PTR(const double) partials = view(partials_, (long long)n, DK_F64_KE, 0);
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += kKeThreads) s = dadd(s, partials[k]);
    s = block_sum_fixed(s);
    if (threadIdx.x == 0) *out = s;
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Self-test of the exact /6 forms against IEEE division over PCG32-random
// doubles: uniform significands, exponents spread over the whole range
// (including subnormals, zero, Inf and NaN patterns).  Counts mismatching
// bit patterns (NaNs compare by NaN-ness).
__global__ void k_selftest_div6(unsigned long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        // splitmix64 of (seed, i): every input independent of the launch shape
        unsigned long long z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const double x = __longlong_as_double((long long)z);
        const double ref = x / 6.0;
        const double a = div6_int(x), c = div6(x);
        const bool ok_a = __double_as_longlong(a) == __double_as_longlong(ref) || (isnan(a) && isnan(ref));
        const bool ok_c = __double_as_longlong(c) == __double_as_longlong(ref) || (isnan(c) && isnan(ref));
        local += (ok_a ? 0 : 1) + (ok_c ? 0 : 1);
    }
    if (local) atomicAdd(bad, local);
}

// Eight independent DFMA chains per thread: issue-rate bound, not latency bound.
constexpr int kRateIters = 2048, kRateChains = 8;
__global__ void k_fp64_rate(double* out, double seed) {
    double a[kRateChains];
#pragma unroll
    for (int c = 0; c < kRateChains; ++c) a[c] = seed + threadIdx.x + c;
    const double m = 0.999999999, k = 1e-9;
    for (int i = 0; i < kRateIters; ++i) {
#pragma unroll
        for (int c = 0; c < kRateChains; ++c) a[c] = __fma_rn(a[c], m, k);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < kRateChains; ++c) s += a[c];
    if (s == 12345.678) out[0] = s;  // keeps the chains live
}

}  // namespace

// dadd_int against __dadd_rn on pairs built to hit every path: random bit
// patterns, close exponents (cancellation), exact ties, far exponents.
__global__ void k_selftest_dadd(unsigned long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        auto mix = [](unsigned long long z) {
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            return z ^ (z >> 31);
        };
        const unsigned long long r1 = mix(seed + (2 * i + 1) * 0x9E3779B97F4A7C15ull);
        const unsigned long long r2 = mix(seed + (2 * i + 2) * 0x9E3779B97F4A7C15ull);
        const unsigned long long ua = r1;
        unsigned long long ub;
        switch (i & 3) {
        case 0: ub = r2; break;  // independent
        case 1: {                // exponent within +-60 of a's, random sign
            const long long ea = (long long)((ua >> 52) & 0x7FF);
            long long eb = ea + (long long)(r2 % 121) - 60;
            eb = eb < 0 ? 0 : (eb > 0x7FF ? 0x7FF : eb);
            ub = (r2 & 0x8000000000000000ull) | ((unsigned long long)eb << 52) | ((r2 >> 11) & 0xFFFFFFFFFFFFFull);
            break;
        }
        case 2: {                // same exponent and close significand: cancellation
            ub = (r2 & 0x8000000000000000ull) | (ua & 0x7FF0000000000000ull) |
                 ((ua + (r2 & 0xFFF) - 0x800) & 0xFFFFFFFFFFFFFull);
            break;
        }
        default: {               // half an ulp of a (a tie) times a small power of two
            const unsigned long long ea = (ua >> 52) & 0x7FF;
            const unsigned long long sh = 53 + (r2 & 3);
            const unsigned long long eb = ea > sh ? ea - sh : 0;
            ub = (r2 & 0x8000000000000000ull) | (eb << 52) | (r2 & 0xFull);
            break;
        }
        }
        const double a = __longlong_as_double((long long)ua), b = __longlong_as_double((long long)ub);
        const double ref = __dadd_rn(a, b), got = dadd_int(a, b), got2 = dsub_int(a, b), ref2 = __dsub_rn(a, b);
        const bool ok = __double_as_longlong(got) == __double_as_longlong(ref) || (isnan(got) && isnan(ref));
        const bool ok2 = __double_as_longlong(got2) == __double_as_longlong(ref2) || (isnan(got2) && isnan(ref2));
        local += (ok ? 0 : 1) + (ok2 ? 0 : 1);
    }
    if (local) atomicAdd(bad, local);
}

bool selftest_dadd(unsigned long long n, unsigned long long seed, unsigned long long* mismatches) {
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&bad, sizeof *bad) != cudaSuccess) return false;
    cudaMemset(bad, 0, sizeof *bad);
    k_selftest_dadd<<<152 * 8, 256>>>(n, seed, bad);
    const bool ok = cudaMemcpy(mismatches, bad, sizeof *bad, cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(bad);
    return ok && cudaGetLastError() == cudaSuccess;
}

bool selftest_div6(unsigned long long n, unsigned long long seed, unsigned long long* mismatches) {
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&bad, sizeof *bad) != cudaSuccess) return false;
    cudaMemset(bad, 0, sizeof *bad);
    k_selftest_div6<<<152 * 8, 256>>>(n, seed, bad);
    const bool ok = cudaMemcpy(mismatches, bad, sizeof *bad, cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(bad);
    return ok && cudaGetLastError() == cudaSuccess;
}

bool measure_fp64_rate(double* fma_per_s) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return false;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, threads = 256;
    k_fp64_rate<<<blocks, threads>>>(out, 1.0);  // warm-up
    cudaEventRecord(a);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) k_fp64_rate<<<blocks, threads>>>(out, 1.0 + r);
    cudaEventRecord(b);
    bool ok = cudaEventSynchronize(b) == cudaSuccess;
    float ms = 0;
    ok = ok && cudaEventElapsedTime(&ms, a, b) == cudaSuccess;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (!ok || ms <= 0) return false;
    *fma_per_s = (double)blocks * threads * kRateIters * kRateChains * reps / (ms * 1e-3);
    return true;
}

namespace {
}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
void launch_velocity_bc(const Geom& g, double* u, double* v, double* w, Status* st, int gate, cudaStream_t s) {
    long long mx = 0;
    const int N[3][3] = {{g.NX, g.NY, g.NZ}, {g.NY, g.NX, g.NZ}, {g.NZ, g.NX, g.NY}};  // Nn, N1, N2 per component
    for (const auto& n : N) {
        mx = std::max(mx, 2ll * n[1] * n[2]);
        mx = std::max(mx, 2ll * (n[0] + 1) * n[2]);
        mx = std::max(mx, 2ll * (n[0] + 1) * (n[1] + 2));
    }
    dim3 grid(cdiv(mx, 256), 9);
    k_velocity_bc<<<grid, 256, 0, s>>>(g, u, v, w, st, gate);
}

void launch_sweep_fp64(const Geom& g, int axis, const Fields& f, double dt, double invH, double lam, Status* st,
                       int phase, cudaStream_t s) {
    SweepArgs a;
    a.u = view((const double*)f.u, g.u.count, DK_F64_SWEEP, 0);
    a.v = view((const double*)f.v, g.v.count, DK_F64_SWEEP, 0);
    a.w = view((const double*)f.w, g.w.count, DK_F64_SWEEP, 0);
    a.tu = view(f.t0, g.u.count, DK_F64_SWEEP, 0);
    a.tv = view(f.t1, g.v.count, DK_F64_SWEEP, 0);
    a.tw = view(f.t2, g.w.count, DK_F64_SWEEP, 0);
    a.du = g.u; a.dv = g.v; a.dw = g.w;
    a.NX = g.NX; a.NY = g.NY; a.NZ = g.NZ; a.G = g.G;
    a.dt = dt; a.invH = invH; a.lam = lam;
    a.st = st; a.phase = phase;
    dim3 block(64, 4);
    dim3 grid(cdiv(g.NX + 1, 64), cdiv(g.NY + 1, 4), 3 * (g.NZ + 1));
    if (axis == 0) k_sweep_fp64<0><<<grid, block, 0, s>>>(a);
    else if (axis == 1) k_sweep_fp64<1><<<grid, block, 0, s>>>(a);
    else k_sweep_fp64<2><<<grid, block, 0, s>>>(a);
}

void launch_maccormack_fp64(const Geom& g, int axis, const Fields& f, const Fields& fwd, double dt, double invH,
                            double lam, Status* st, int phase, cudaStream_t s) {
    // Forward step: the reference sweep without diffusion, into fwd.t0..t2.
    launch_sweep_fp64(g, axis, fwd, dt, invH, 0.0, st, phase, s);
    SweepArgs a;
    a.u = view((const double*)f.u, g.u.count, DK_F64_SWEEP, 0);
    a.v = view((const double*)f.v, g.v.count, DK_F64_SWEEP, 0);
    a.w = view((const double*)f.w, g.w.count, DK_F64_SWEEP, 0);
    a.tu = view(f.t0, g.u.count, DK_F64_SWEEP, 0);
    a.tv = view(f.t1, g.v.count, DK_F64_SWEEP, 0);
    a.tw = view(f.t2, g.w.count, DK_F64_SWEEP, 0);
    a.du = g.u; a.dv = g.v; a.dw = g.w;
    a.NX = g.NX; a.NY = g.NY; a.NZ = g.NZ; a.G = g.G;
    a.dt = dt; a.invH = invH; a.lam = lam;
    a.st = st; a.phase = phase;
    dim3 block(64, 4);
    dim3 grid(cdiv(g.NX + 1, 64), cdiv(g.NY + 1, 4), 3 * (g.NZ + 1));
    if (axis == 0) k_maccormack_fp64<0><<<grid, block, 0, s>>>(a, fwd.t0, fwd.t1, fwd.t2);
    else if (axis == 1) k_maccormack_fp64<1><<<grid, block, 0, s>>>(a, fwd.t0, fwd.t1, fwd.t2);
    else k_maccormack_fp64<2><<<grid, block, 0, s>>>(a, fwd.t0, fwd.t1, fwd.t2);
}

void launch_divergence_fp64(const Geom& g, const Fields& f, double* b, double scale, double h2, bool zero_p,
                            Status* st, int gate, cudaStream_t s) {
    dim3 block(64, 4);
    dim3 grid(cdiv(g.p.nx, 64), cdiv(g.p.ny, 4), g.p.nz);
    k_divergence_fp64<<<grid, block, 0, s>>>(g, f.u, f.v, f.w, f.p, f.div, b, scale, h2, zero_p ? 1 : 0, st, gate);
}

// Integer-pipe share of the red-black chain: AEROFLUX_RBGS_EMU picks the
// mask.  Measured on GB300 at 256^3, every emulated add slows the update
// (all six native: 41 ms per 200-pair projection; all six emulated: 146 ms),
// so the default keeps the adds on the FP64 pipe; the exact /6 stays on the
// integer pipe, where it wins over its three-operation FP64 sequence.
static int rbgs_emu_mask() {
    static int m = -1;
    if (m < 0) {
        const char* v = getenv("AEROFLUX_RBGS_EMU");
        m = v ? atoi(v) : 0x00;
    }
    return m;
}

void launch_rbgs_fp64(const Geom& g, double* p, const double* b, int color, Status* st, int gate, cudaStream_t s) {
    dim3 block(32, 4);
    dim3 grid(cdiv((g.NX + 1) / 2, 32), cdiv(g.NY, 4), g.NZ);
    switch (rbgs_emu_mask()) {
    case 0x00: k_rbgs_fp64<0x00><<<grid, block, 0, s>>>(g, p, b, color, st, gate); break;
    case 0x01: k_rbgs_fp64<0x01><<<grid, block, 0, s>>>(g, p, b, color, st, gate); break;
    case 0x05: k_rbgs_fp64<0x05><<<grid, block, 0, s>>>(g, p, b, color, st, gate); break;
    case 0x15: k_rbgs_fp64<0x15><<<grid, block, 0, s>>>(g, p, b, color, st, gate); break;
    case 0x2A: k_rbgs_fp64<0x2A><<<grid, block, 0, s>>>(g, p, b, color, st, gate); break;
    case 0x35: k_rbgs_fp64<0x35><<<grid, block, 0, s>>>(g, p, b, color, st, gate); break;
    default: k_rbgs_fp64<0x3F><<<grid, block, 0, s>>>(g, p, b, color, st, gate); break;
    }
}

void launch_pressure_bc_fp64(const Geom& g, double* p, Status* st, int gate, cudaStream_t s) {
    long long mx = std::max(2ll * g.NY * g.NZ, std::max(2ll * (g.NX + 2) * g.NZ, 2ll * (g.NX + 2) * (g.NY + 2)));
    dim3 grid(cdiv(mx, 256), 3);
    k_pressure_bc<<<grid, 256, 0, s>>>(g, p, st, gate);
}

void launch_gradient_fp64(const Geom& g, const Fields& f, double scale, Status* st, int gate, cudaStream_t s) {
    dim3 block(64, 4);
    dim3 grid(cdiv(g.NX + 1, 64), cdiv(g.NY + 1, 4), 3 * (g.NZ + 1));
    k_gradient_fp64<<<grid, block, 0, s>>>(g, f.p, f.u, f.v, f.w, scale, st, gate);
}

void launch_step_tick(Status* st, cudaStream_t s) { k_step_tick<<<1, 1, 0, s>>>(st); }

void launch_b_from_div(const Geom& g, const double* div, double* b, double h2, cudaStream_t s) {
    dim3 block(64, 4);
    dim3 grid(cdiv(g.NX, 64), cdiv(g.NY, 4), g.NZ);
    k_b_from_div<<<grid, block, 0, s>>>(g, div, b, h2);
}

void launch_max_divergence(const Geom& g, const double* u, const double* v, const double* w, double invH,
                           unsigned long long* out, cudaStream_t s) {
    dim3 grid(cdiv(g.NX, 128), g.NY, g.NZ);
    k_max_divergence<<<grid, 128, 0, s>>>(g, u, v, w, invH, out);
}

void launch_max_abs3(const double* u, long long nu, const double* v, long long nv, const double* w, long long nw,
                     unsigned long long* out, cudaStream_t s) {
    long long n = std::max(nu, std::max(nv, nw));
    unsigned blocks = (unsigned)std::min<long long>(cdiv(n, 256), 152 * 8);
    k_max_abs3<<<blocks, 256, 0, s>>>(u, nu, v, nv, w, nw, out);
}

bool fp64_debug_bounds(unsigned long long* first, unsigned* count, bool reset) {
#if AEROFLUX_DEBUG_BOUNDS
    if (cudaMemcpyFromSymbol(first, g_dbg_first, sizeof *first) != cudaSuccess ||
        cudaMemcpyFromSymbol(count, g_dbg_count, sizeof *count) != cudaSuccess)
        return false;
    if (reset) {
        const unsigned long long none = ~0ull;
        const unsigned zero = 0;
        cudaMemcpyToSymbol(g_dbg_first, &none, sizeof none);
        cudaMemcpyToSymbol(g_dbg_count, &zero, sizeof zero);
    }
#else
    (void)reset;
    *first = ~0ull;
    *count = 0;
#endif
    return true;
}

void launch_kinetic_energy(const Geom& g, const double* u, const double* v, const double* w, double* partials,
                           double* out, cudaStream_t s) {
    k_ke_planes<<<g.NZ, kKeThreads, 0, s>>>(g, u, v, w, partials);
    k_ke_final<<<1, kKeThreads, 0, s>>>(partials, g.NZ, out);
}

}  // namespace af

// ---------------------------------------------------------------------------
// Kinetic energy without any allocation.
//
// Some callers cannot allocate device memory while they run: hosts that hand
// all device memory to their own pool up front and forbid cudaMalloc
// afterwards, and latency-bound loops that cannot afford the implicit
// device-wide synchronisation of cudaMalloc/cudaFree.  This entry point runs
// the same fixed-order reduction as af_kinetic_energy over caller-owned
// device fields, with its scratch (one partial per z-plane plus the final
// sum) in the file-scope array below.  Every GPU that loads the library holds
// the array until the process exits.
// ---------------------------------------------------------------------------
namespace af {
namespace {

constexpr int kNoAllocMaxPlanes = 16384;  // 128 KiB of partials
static __device__ __align__(256) double g_ke_scratch[kNoAllocMaxPlanes + 1];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_ke_scratch on the current device, resolved once per
// device (host code only sees a host-side stand-in for the symbol).
cudaError_t scratch_address(int dev, double** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t rc = cudaGetSymbolAddress(&p, g_ke_scratch);
        if (rc != cudaSuccess) return rc;
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

void put(char* err, size_t errlen, const char* msg) {
    if (err && errlen) snprintf(err, errlen, "%s", msg);
}

}  // namespace
}  // namespace af

extern "C" int af_kinetic_energy_noalloc(const af_config* cfg, const double* u, const double* v, const double* w,
                                         void* stream, double* out, char* err, size_t errlen) {
    using namespace af;
    if (!cfg || !u || !v || !w || !out) {
        put(err, errlen, "aeroflux: kinetic energy without allocation: NULL argument");
        return AF_ERR_ARG;
    }
    if (cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1 || cfg->ghost < 1 || !(cfg->h > 0) || std::isinf(cfg->h)) {
        put(err, errlen, "aeroflux: kinetic energy without allocation: extents, ghost and h must be positive");
        return AF_ERR_ARG;
    }
    // The kernels index planes and rows in int: extents and the ghost stay
    // below 2^20 so every padded coordinate fits.
    if (cfg->nz > kNoAllocMaxPlanes || cfg->nx >= (1 << 20) || cfg->ny >= (1 << 20) || cfg->ghost >= (1 << 20)) {
        char m[256];
        snprintf(m, sizeof m,
                 "aeroflux: kinetic energy without allocation supports at most %d z-planes (and nx, ny, ghost "
                 "< 2^20), got %lldx%lldx%lld ghost %lld",
                 kNoAllocMaxPlanes, (long long)cfg->nx, (long long)cfg->ny, (long long)cfg->nz,
                 (long long)cfg->ghost);
        put(err, errlen, m);
        return AF_ERR_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        put(err, errlen, "aeroflux: kinetic energy without allocation: no usable current device");
        return AF_ERR_CUDA;
    }
    double* scratch = nullptr;
    cudaError_t rc = scratch_address(dev, &scratch);
    if (rc != cudaSuccess) {
        put(err, errlen, cudaGetErrorString(rc));
        return AF_ERR_CUDA;
    }
    Geom g{};
    g.NX = (int)cfg->nx;
    g.NY = (int)cfg->ny;
    g.NZ = (int)cfg->nz;
    g.G = (int)cfg->ghost;
    const long long cx = cfg->nx + 2 * cfg->ghost, cy = cfg->ny + 2 * cfg->ghost;
    g.u.sy = cx + 1;
    g.u.sz = (cx + 1) * cy;
    g.v.sy = cx;
    g.v.sz = cx * (cy + 1);
    g.w.sy = cx;
    g.w.sz = cx * cy;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Every partial the final pass reads is rewritten by this call, so the
    // array needs no clearing; concurrent calls on the GPU share it and race.
    k_ke_planes<<<g.NZ, kKeThreads, 0, s>>>(g, u, v, w, scratch);
    k_ke_final<<<1, kKeThreads, 0, s>>>(scratch, g.NZ, scratch + kNoAllocMaxPlanes);
    double sum = 0;
    if ((rc = cudaGetLastError()) != cudaSuccess ||
        (rc = cudaMemcpyAsync(&sum, scratch + kNoAllocMaxPlanes, sizeof sum, cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (rc = cudaStreamSynchronize(s)) != cudaSuccess) {
        put(err, errlen, cudaGetErrorString(rc));
        return AF_ERR_CUDA;
    }
    const double h = cfg->h;
    const double vol = h * h * h;
    *out = 0.5 * sum * vol;
    return AF_OK;
}
