// af_cells.cuh -- per-cell device logic shared by the single-grid kernels
// (af_fp64.cu) and the batched kernels (af_batch.cu), so both compute every
// cell with the same instructions.  Internal to libaeroflux_cuda.
#pragma once

#include "af_debug.cuh"
#include "af_internal.h"

#include <math.h>

namespace af {
namespace cells {

// --- exact binary64 (Go amd64 semantics: no contraction, RN) --------------
constexpr unsigned long long kSign = 0x8000000000000000ull;

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
// Go's unary minus: a sign-bit flip (-0 for +0, payload kept for NaN).
__device__ __forceinline__ double flip(double a) {
    return __longlong_as_double((long long)((unsigned long long)__double_as_longlong(a) ^ kSign));
}

// --- exact binary64 steps on the integer pipe ------------------------------
// GB300's FP64 pipe (about two operations per SM per clock) also executes
// binary64 compares and conversions; the sweeps move the exact ones here.
constexpr unsigned long long kFrac = 0xFFFFFFFFFFFFFull;
__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ double dfrom(unsigned long long b) { return __longlong_as_double((long long)b); }

// (double)n for 0 <= n < 2^31.
__device__ __forceinline__ double i2d_small(int n) {
    if (n == 0) return 0.0;
    const int lz = __clz(n);
    return dfrom(((unsigned long long)(1023 + 31 - lz) << 52) | (((unsigned long long)(unsigned)n << (21 + lz)) & kFrac));
}

// Truncation toward zero of +-0 <= x < 2^31 (finite).
__device__ __forceinline__ long long d2i_trunc_small(double x) {
    const unsigned long long b = dbits(x) & ~kSign;
    const int e = (int)(b >> 52) - 1023;
    if (e < 0) return 0;
    return (long long)(((b & kFrac) | (1ull << 52)) >> (52 - e));
}

// x - a0 for finite 0 <= x < 2^31 (or -0) and an integer a0 with
// trunc(x) - 1 <= a0 <= trunc(x) and x - a0 <= 1: the exact difference (the
// binary64 subtraction is exact here too), including -0 - 0 = -0.
__device__ __forceinline__ double frac_sub(double x, long long a0) {
    const unsigned long long b = dbits(x);
    const int e = (int)((b & ~kSign) >> 52) - 1023;
    if (e < 0) return a0 == 0 ? x : dsub(x, (double)a0);  // x < 1: a0 is 0 here
    const unsigned long long m = (b & kFrac) | (1ull << 52);
    const long long t = (long long)(m >> (52 - e));
    if (t != a0) return 1.0;  // a0 = t - 1 only when x = t: difference 1
    const unsigned long long f = m & ((1ull << (52 - e)) - 1ull);
    if (f == 0) return 0.0;
    const int p = 63 - __clzll((long long)f);  // leading bit of f, value f * 2^(e-52)
    return dfrom(((unsigned long long)(1023 + e - 52 + p) << 52) | ((f << (52 - p)) & kFrac));
}

// RN(0.25 * x) and RN(2 * x): exact exponent shifts while the result stays
// normal (and for 0, Inf, NaN, which pass through); the FP64 multiply
// otherwise, so every input rounds as the multiply would.
__device__ __forceinline__ double quarter(double x) {
    const unsigned long long b = dbits(x);
    const unsigned e = (unsigned)((b >> 52) & 0x7FF);
    if (e >= 3u && e < 0x7FFu) return dfrom(b - (2ull << 52));
    if (e == 0x7FFu || (b & ~kSign) == 0ull) return x;
    return dmul(0.25, x);
}
__device__ __forceinline__ double twice(double x) {
    const unsigned long long b = dbits(x);
    const unsigned e = (unsigned)((b >> 52) & 0x7FF);
    if (e >= 1u && e < 0x7FEu) return dfrom(b + (1ull << 52));
    if (e == 0x7FFu || (b & ~kSign) == 0ull) return x;
    return dmul(2.0, x);
}

// Correctly rounded x/6.  Because 6 = 3*2, x/6 is never within ulp/6 of a
// rounding midpoint, while q + r*c below is within 2^-54 ulp of x/6 (q =
// RN(x*RN(1/6)), r = x - 6q computed exactly by the FMA, RN(1/6) = (1-2^-54)/6).
// So RN(q + r*c) = RN(x/6).  This is the multiply-by-reciprocal-plus-remainder
// division of Markstein (1990) / Brisebarre-Muller-Raina (2004), specialised
// to divisor 6.  Outside the range where q and r stay normal (and for zero,
// Inf, NaN) the IEEE division is used.  Three FP64 pipe operations instead of
// a full reciprocal-refinement sequence.
__device__ __forceinline__ double div6(double x) {
    const double c = 0x1.5555555555555p-3;  // RN(1/6)
    const double ax = fabs(x);
    if (ax >= 0x1p-960 && ax < 0x1p1020) {
        const double q = dmul(x, c);
        const double r = __fma_rn(-6.0, q, x);
        return __fma_rn(r, c, q);
    }
    return x / 6.0;
}

// Correctly rounded x/6 on the integer pipe.  For normal x with significand
// M (53-bit integer) and biased exponent E, x/6 = 2^(E-1076-t) * (M*2^t/3)
// with t = 1 when M >= 3*2^51, else t = 2, which puts N/3 (N = M*2^t) in
// [2^52, 2^53).  Q = floor(N/3) by a multiply-high with the 2^65/3 magic
// constant (exact for every 64-bit N); the remainder N - 3Q is 0, 1 or 2, so
// the fraction is 0, 1/3 or 2/3: round up exactly when it is 2 (no ties).
// Zero, subnormal, Inf, NaN and results that would be subnormal (E < 5) take
// the IEEE division.  No binary64 arithmetic instruction is issued.
__device__ __forceinline__ double div6_int(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned E = (unsigned)(b >> 52) & 0x7FFu;
    if (E < 5u || E == 0x7FFu) return x / 6.0;
    const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const unsigned t = M >= 0x18000000000000ull ? 1u : 2u;  // 3*2^51
    const unsigned long long N = M << t;
    unsigned long long Q = __umul64hi(N, 0xAAAAAAAAAAAAAAABull) >> 1;
    const unsigned long long rem = N - 3ull * Q;
    unsigned long long e = (unsigned long long)(E - 1u - t);
    Q += rem == 2ull ? 1ull : 0ull;
    if (Q == 0x20000000000000ull) {  // rounded up to 2^53
        Q >>= 1;
        e += 1;
    }
    return __longlong_as_double((long long)((b & kSign) | (e << 52) | (Q & 0xFFFFFFFFFFFFFull)));
}

// RN(a + b) in binary64 on the integer pipe.  Significands are aligned in
// 64-bit integers with the leading bit at 62, leaving 10 guard bits; bits
// shifted out of the smaller operand fold into a sticky bit.  Equal signs
// add (one carry renormalisation), opposite signs subtract and renormalise
// left (exact whenever more than the guard bits would be needed, i.e. for
// exponent gaps of 0 or 1), then round to nearest, ties to even.  Zero and
// subnormal operands, Inf, NaN and results that are subnormal or overflow
// take the native add, so the result always equals __dadd_rn(a, b).
__device__ __forceinline__ double dadd_int(double a, double b) {
    unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    unsigned long long ma = ua & ~kSign, mb = ub & ~kSign;
    if (ma < mb) {
        const unsigned long long t = ua; ua = ub; ub = t;
        const unsigned long long m = ma; ma = mb; mb = m;
    }
    const unsigned ea = (unsigned)(ma >> 52), eb = (unsigned)(mb >> 52);
    if (eb == 0u || ea == 0x7FFu) return __dadd_rn(a, b);
    const unsigned long long frac = 0xFFFFFFFFFFFFFull, one = 0x10000000000000ull;
    const unsigned long long A = ((ma & frac) | one) << 10;
    unsigned long long B = ((mb & frac) | one) << 10;
    const unsigned d = ea - eb;
    if (d >= 64u) B = 1ull;
    else if (d) B = (B >> d) | ((B << (64u - d)) != 0ull ? 1ull : 0ull);
    int e = (int)ea;
    unsigned long long S;
    if (((ua ^ ub) & kSign) == 0ull) {
        S = A + B;
        if (S >> 63) {
            S = (S >> 1) | (S & 1ull);
            e += 1;
        }
    } else {
        S = A - B;
        if (S == 0ull) return 0.0;  // x + (-x) = +0 under round to nearest
        const int lz = __clzll((long long)S) - 1;
        S <<= lz;
        e -= lz;
    }
    unsigned long long M = S >> 10;
    const unsigned long long R = S & 0x3FFull;
    if (R > 0x200ull || (R == 0x200ull && (M & 1ull))) {
        M += 1ull;
        if (M >> 53) {
            M >>= 1;
            e += 1;
        }
    }
    if (e <= 0 || e >= 0x7FF) return __dadd_rn(a, b);
    return __longlong_as_double((long long)((ua & kSign) | ((unsigned long long)e << 52) | (M & frac)));
}

// a - b through dadd_int (negation is exact).
__device__ __forceinline__ double dsub_int(double a, double b) { return dadd_int(a, flip(b)); }

__device__ __forceinline__ bool gated(const Status* st, int gate) {
    return st->fault_gate < st->step * 8u + (unsigned)gate;
}

// --- applyVelocityBC, stencil.go:246-315 ----------------------------------
//
// The reference writes the wall faces, then reflects tangential ghosts in a
// fixed order where later passes read ghosts written by earlier ones (edges
// and corners).  Composed, every written cell equals the sign-flipped value
// of one interior cell: reflect each ghost coordinate into the interior,
// flip the sign once per reflection, and read +0 where the source lies on a
// wall face (zeroed by the first pass).  So every cell is written once from
// cells nobody writes, and the reference's bits come out, -0 included.
struct BcComp {
    AF_PTR(double) f;
    long long s_n, s_1, s_2;  // strides along the normal axis and the two tangential axes
    int Nn, N1, N2;           // interior extents along those axes
};

__device__ __forceinline__ long long bc_set_count(const BcComp& c, int set) {
    return set == 0 ? 2ll * c.N1 * c.N2 : (set == 1 ? 2ll * (c.Nn + 1) * c.N2 : 2ll * (c.Nn + 1) * (c.N1 + 2));
}

__device__ __forceinline__ double bc_src(const BcComp& c, int G, int n, int a, int b) {
    if (n == G || n == G + c.Nn) return 0.0;
    return c.f[(long long)n * c.s_n + (long long)a * c.s_1 + (long long)b * c.s_2];
}

// Divides by a divisor fixed per call (the plain 32-bit division).
struct HwDiv {
    unsigned d;
    __device__ __forceinline__ unsigned div(unsigned n) const { return n / d; }
};

// Writes element i (< bc_set_count) of write set `set` of one component:
// 0 = wall faces, 1 = ghosts of the first tangential axis, 2 = ghosts of the
// second tangential axis (edges included).  A set holds fewer than 2^32
// elements (2 (N+2)^2 for extents N below 46000), so the index decoding
// divides in 32 bits.  Consecutive elements walk the axis with stride 1
// where the set has one (set 2 of V and W walks x, the first tangential
// axis, instead of the normal one), so a warp's stores fill whole sectors;
// every cell is written once from cells nobody writes, so the order does not
// change a bit.  bc_divisors gives the two divisors; D is any divider with
// the quotients of plain division.
__device__ __forceinline__ bool bc_t1_first(const BcComp& c, int set) { return set == 2 && c.s_1 == 1; }
__device__ __host__ __forceinline__ void bc_divisors(int Nn, int N1, int N2, bool t1_first, int set, unsigned* d1,
                                                     unsigned* d2) {
    if (set == 0) *d1 = (unsigned)N1, *d2 = (unsigned)N2;
    else if (set == 1) *d1 = (unsigned)(Nn + 1), *d2 = (unsigned)N2;
    else if (t1_first) *d1 = (unsigned)(N1 + 2), *d2 = (unsigned)(Nn + 1);
    else *d1 = (unsigned)(Nn + 1), *d2 = (unsigned)(N1 + 2);
}
template <class D>
__device__ __forceinline__ void bc_cell_div(const BcComp& c, int G, int set, unsigned i, const D& d1, const D& d2) {
    int n, t1, t2;
    double val;
    const unsigned r = d1.div(i), q = d2.div(r);
    int lo = (int)(i - r * d1.d), mid = (int)(r - q * d2.d);
    if (bc_t1_first(c, set)) {  // lo walks t1, mid the normal axis
        const int t = lo;
        lo = mid;
        mid = t;
    }
    if (set == 0) {
        t1 = G + lo;
        t2 = G + mid;
        n = q ? G + c.Nn : G;
        val = 0.0;
    } else if (set == 1) {
        n = G + lo;
        t2 = G + mid;
        const int side = (int)q;
        t1 = side ? G + c.N1 : G - 1;
        const int s1 = side ? G + c.N1 - 1 : G;
        val = flip(bc_src(c, G, n, s1, t2));
    } else {
        n = G + lo;
        t1 = G - 1 + mid;
        const int side = (int)q;
        t2 = side ? G + c.N2 : G - 1;
        const int s2 = side ? G + c.N2 - 1 : G;
        int s1 = t1;
        bool odd = true;
        if (t1 == G - 1) { s1 = G; odd = false; }
        else if (t1 == G + c.N1) { s1 = G + c.N1 - 1; odd = false; }
        const double s = bc_src(c, G, n, s1, s2);
        val = odd ? flip(s) : s;
    }
    c.f[(long long)n * c.s_n + (long long)t1 * c.s_1 + (long long)t2 * c.s_2] = val;
}

__device__ __forceinline__ void bc_cell(const BcComp& c, int G, int set, long long il) {
    HwDiv d1, d2;
    bc_divisors(c.Nn, c.N1, c.N2, bc_t1_first(c, set), set, &d1.d, &d2.d);
    bc_cell_div(c, G, set, (unsigned)il, d1, d2);
}

__device__ __forceinline__ BcComp bc_comp(const Geom& g, int comp, AF_PTR(double) u, AF_PTR(double) v,
                                          AF_PTR(double) w) {
    if (comp == 0) return BcComp{u, 1, g.u.sy, g.u.sz, g.NX, g.NY, g.NZ};
    if (comp == 1) return BcComp{v, g.v.sy, 1, g.v.sz, g.NY, g.NX, g.NZ};
    return BcComp{w, g.w.sz, 1, g.w.sy, g.NZ, g.NX, g.NY};
}

// --- applyPressureBC, project.go:139-163 -----------------------------------
// Composed, every first-layer ghost holds the interior cell at the clamped
// coordinates.  Element i of set 0 (x ghosts), 1 (y ghosts), 2 (z ghosts).
__device__ __forceinline__ long long pbc_set_count(const Geom& g, int set) {
    return set == 0 ? 2ll * g.NY * g.NZ : (set == 1 ? 2ll * (g.NX + 2) * g.NZ : 2ll * (g.NX + 2) * (g.NY + 2));
}

// A set holds fewer than 2^32 elements: 32-bit index decoding.
__device__ __forceinline__ void pbc_cell(const Geom& g, AF_PTR(double) p, int set, long long il) {
    const int G = g.G, NX = g.NX, NY = g.NY, NZ = g.NZ;
    const unsigned i = (unsigned)il;
    int x, y, z;
    if (set == 0) {
        const unsigned r = i / (unsigned)NY, q = r / (unsigned)NZ;
        y = G + (int)(i - r * (unsigned)NY);
        z = G + (int)(r - q * (unsigned)NZ);
        x = q ? G + NX : G - 1;
    } else if (set == 1) {
        const unsigned r = i / (unsigned)(NX + 2), q = r / (unsigned)NZ;
        x = G - 1 + (int)(i - r * (unsigned)(NX + 2));
        z = G + (int)(r - q * (unsigned)NZ);
        y = q ? G + NY : G - 1;
    } else {
        const unsigned r = i / (unsigned)(NX + 2), q = r / (unsigned)(NY + 2);
        x = G - 1 + (int)(i - r * (unsigned)(NX + 2));
        y = G - 1 + (int)(r - q * (unsigned)(NY + 2));
        z = q ? G + NZ : G - 1;
    }
    const int cx = min(max(x, G), G + NX - 1);
    const int cy = min(max(y, G), G + NY - 1);
    const int cz = min(max(z, G), G + NZ - 1);
    p[x + y * g.p.sy + z * g.p.sz] = p[cx + cy * g.p.sy + cz * g.p.sz];
}

// --- computeDivergence (project.go:42-62) + P zeroing + B = h2*Div ---------
// (x, y, z) is any cell of the padded P extent.
__device__ __forceinline__ void div_cell(const Geom& g, AF_PTR(const double) AF_RESTRICT u,
                                         AF_PTR(const double) AF_RESTRICT v, AF_PTR(const double) AF_RESTRICT w,
                                         AF_PTR(double) AF_RESTRICT p, AF_PTR(double) AF_RESTRICT dv,
                                         AF_PTR(double) AF_RESTRICT bb, double scale, double h2, bool zero_p, int x,
                                         int y, int z) {
    const long long i = x + y * g.p.sy + z * g.p.sz;
    if (zero_p) p[i] = 0.0;
    const int G = g.G;
    if (x < G || x >= G + g.NX || y < G || y >= G + g.NY || z < G || z >= G + g.NZ) return;
    const long long iu = x + y * g.u.sy + z * g.u.sz;
    const long long iv = x + y * g.v.sy + z * g.v.sz;
    const long long iw = x + y * g.w.sy + z * g.w.sz;
    const double du = dsub(u[iu + 1], u[iu]);
    const double dvv = dsub(v[iv + g.v.sy], v[iv]);
    const double dw = dsub(w[iw + g.w.sz], w[iw]);
    const double d = dmul(scale, dadd(dadd(du, dvv), dw));
    dv[i] = d;
    bb[i] = dmul(h2, d);
}

// --- subtractGradient, project.go:172-205 ----------------------------------
// Face (x, y, z) of component c, inside that component's write range: the
// new value of the face of f (the component's field) is stored to out at the
// same index -- f itself for the reference's in-place update.
__device__ __forceinline__ void grad_face_to(const Geom& g, AF_PTR(const double) AF_RESTRICT p,
                                             AF_PTR(const double) f, AF_PTR(double) out, double scale, int c, int x,
                                             int y, int z) {
    const long long ip = x + y * g.p.sy + z * g.p.sz;
    if (c == 0) {
        const long long i = x + y * g.u.sy + z * g.u.sz;
        out[i] = dsub(f[i], dmul(scale, dsub(p[ip], p[ip - 1])));
    } else if (c == 1) {
        const long long i = x + y * g.v.sy + z * g.v.sz;
        out[i] = dsub(f[i], dmul(scale, dsub(p[ip], p[ip - g.p.sy])));
    } else {
        const long long i = x + y * g.w.sy + z * g.w.sz;
        out[i] = dsub(f[i], dmul(scale, dsub(p[ip], p[ip - g.p.sz])));
    }
}

__device__ __forceinline__ void grad_face(const Geom& g, AF_PTR(const double) AF_RESTRICT p, AF_PTR(double) u,
                                          AF_PTR(double) v, AF_PTR(double) w, double scale, int c, int x, int y,
                                          int z) {
    AF_PTR(double) f = c == 0 ? u : (c == 1 ? v : w);
    grad_face_to(g, p, f, f, scale, c, x, y, z);
}

// --- binary64 <-> binary32 on the integer pipe -----------------------------
// GB300 issues about two binary64 operations per SM per clock; these
// conversions keep the mixed form off that pipe.

// Round half away from zero on the magnitude; below FLT_MIN flushes to zero;
// Inf/NaN kept.
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
    return __uint_as_float(sign | (((unsigned)ef << 23) + mant + rnd));  // a carry rounds into the exponent
}

// Exact; subnormal floats flush to zero.
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

// --- binary32 advection + diffusion of one face (stencil.go:44-225) --------
// The sweep interpolates along its axis only (the other two weights are 0).
// Every rounding is explicit, so the result does not depend on how the
// compiler contracts multiplies and adds.

// Face velocity from the four axis-component faces around it, summed in the
// order given: 0.25 * (((t0 + t1) + t2) + t3).
__device__ __forceinline__ float mx_face_vel4(float t0, float t1, float t2, float t3) {
    return __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3));
}

// Semi-Lagrangian backtrace of a face at coordinate ca (na: the field's
// padded extent along the sweep axis) by velocity vel, relative to the face
// so binary32 keeps the fraction accurate at any grid size (departure =
// ca + off, off = -dt*vel/h), clamped into the padded field as
// stencil.go:174-188 clamps: the interpolation taps are i0 and i0 + 1 with
// weight t on the second.  Returns false on a NaN backtrace (a contained
// fault; the face is then not written).
__device__ __forceinline__ bool mx_backtrace(float vel, int ca, int na, float dt_invh, int* i0_out, float* t_out) {
    const float off = -__fmul_rn(vel, dt_invh);
    if (isnan(off)) return false;
    const float fl = floorf(off);
    const float pos = __fadd_rn((float)ca, off);
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
        t = __fsub_rn(off, fl);
        if (i0 >= na - 1) {
            i0 = na - 2;
            t = 1.0f;
        }
    }
    *i0_out = i0;
    *t_out = t;
    return true;
}

// Linear interpolation d0 + t*(d1 - d0) plus lam times the second
// difference (fm - 2 f0) + fp of the face's own values along the axis.
__device__ __forceinline__ float mx_face_value(float t, float d0, float d1, float fm, float f0, float fp, float lam) {
    const float adv = __fmaf_rn(t, __fsub_rn(d1, d0), d0);
    if (lam != 0.0f) return __fmaf_rn(lam, __fadd_rn(__fsub_rn(fm, __fmul_rn(2.0f, f0)), fp), adv);
    return __fadd_rn(adv, 0.0f);
}

// New value of the face whose binary32 value sits at f[0] (its neighbours
// along the sweep axis at f[-s] and f[s]): mx_backtrace, then mx_face_value
// with the taps read through f.
__device__ __forceinline__ bool mx_face_update(AF_PTR(const float) AF_RESTRICT f, long long s, float vel, int ca,
                                               int na, float dt_invh, float lam, float* out) {
    int i0;
    float t;
    if (!mx_backtrace(vel, ca, na, dt_invh, &i0, &t)) return false;
    AF_PTR(const float) p0 = f + (long long)(i0 - ca) * s;
    *out = mx_face_value(t, p0[0], p0[s], f[-s], f[0], f[s], lam);
    return true;
}

}  // namespace cells
}  // namespace af
