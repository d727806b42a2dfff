// af_batch.cu -- batched mixed-precision fractional step.
//
// Many independent grids (slots) of uneven sizes step together.  Every stage
// is ONE persistent launch over a device-side work list: per stage, a prefix
// array gives each slot's number of tiles, a block finds its slot by binary
// search and processes one tile of that slot's iteration space, and the grid
// (a fixed multiple of the SM count) strides over all tiles.  Because the
// work lists live in device memory, slots can be assigned, released,
// activated and deactivated between steps without recapturing the step
// graph (continuous batching); the graph is recaptured only when the
// deepest multigrid hierarchy grows or the launch shapes are retuned.
//
// Arithmetic: binary32 advection/diffusion with integer-pipe conversions
// (af_cells.cuh); binary64 divergence, residual, pressure accumulator,
// gradient and BCs (bit-identical to the FP64 form's cells); binary32
// multigrid V-cycles with over-relaxed red-black smoothing inside binary64
// refinement.  The
// refinement loop is one WHILE node for the whole batch: it runs while any
// slot is unconverged, and a converged slot skips every later pass, so each
// slot performs exactly the passes it performs alone.  Every cell's result is
// independent of the tile that computes it, and reductions are exact maxima
// or fixed trees over one slot, so a slot's bits do not depend on the other
// slots or on the tuned launch shapes.
#include "af_batch.h"
#include "af_cells.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

namespace af {
namespace {

using namespace cells;

constexpr int kMaxLev = 16;
constexpr int kCoarseThreads = 512;
constexpr int kCoarseMax = 4096;

// Unsigned 32-bit division by an invariant divisor with one multiply-high
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", 1994): l = ceil(log2 d), m = ceil(2^(32+l)/d) - 2^32,
// n/d = (umulhi(n, m) + n) >> l for every n < 2^32.
struct FastDiv {
    unsigned d = 1, m = 0, l = 0;
    FastDiv() = default;
    __host__ explicit FastDiv(unsigned div) : d(div) {
        while ((1ull << l) < d) ++l;
        m = (unsigned)((((1ull << (32 + l)) + d - 1) / d) - (1ull << 32));
    }
    __device__ __forceinline__ unsigned div(unsigned n) const {
        return (unsigned)(((unsigned long long)__umulhi(n, m) + n) >> l);
    }
};

struct Lvl {
    int nx, ny, nz;
    float wx, wy, wz;   // (h0 / h_axis)^2
    int cx, cy, cz;     // 1 when the axis coarsens into the next level
    float* e;
    float* r;
    FastDiv fnx, fny, fhx;  // nx, ny, (nx+1)/2
    float* e2;              // second buffer of the fused red-black pair (levels below the tail)
    FastDiv ftx;            // fused-pair wide tiles along x
    FastDiv fty[3];         // fused-pair tiles along y, per tile variant (kPairVarTY)
    int nxw;                // 64 x the wide pair tiles along x; a narrow tile column covers nxw .. nx-1
    int tma;                // 1: the level's e, e2, r have tensor maps (the TMA-staged pair may run on it)
};

struct Ctl {
    unsigned long long maxr_bits;  // max |r| of the current pass (binary64 bits)
    unsigned int passes;
    unsigned int stopped;
    double last_div;               // dt/(rho h^2) * max|r| at the last check
    unsigned int nv;               // V-cycles the next pass runs (0: all of them)
    double vfac;                   // measured max|div| reduction per V-cycle (0: none yet); kept across projections
    unsigned int vtotal;           // V-cycles the current projection has run
};

// Whether the multigrid kernels of V-cycle vc of a pass skip a slot.
__device__ __forceinline__ bool mg_off(const Ctl& c, int vc) { return c.stopped || (c.nv && (unsigned)vc >= c.nv); }
// ctl[n] (n = the batch's capacity) is the batch's own record: its nv is the
// number of V-cycles some slot runs in the current pass, so a V-cycle no
// slot runs returns at once instead of walking the slots' tiles.
__device__ __forceinline__ bool vc_idle(const Ctl* ctl, int n, int vc) { return (unsigned)vc >= ctl[n].nv; }

struct InstDev {
    Geom g;
    double* slot[8];   // arena field slots P, U, V, W, Div, Tmp0, Tmp1, Tmp2
    double* b;         // h^2 * Div, P-shaped
    float dt_invh;     // (DT/2)/H for the sweeps
    float lam;         // nu*(DT/2)/H^2
    double div_scale;  // rho/(DT*H)
    double h2;
    double grad_scale;  // DT/(rho*H)
    double res_scale;   // DT/(rho*H^2): max|div| per unit residual
    double thresh;      // 0.5 * div_tol
    unsigned max_refine;
    int nlev;
    int coarse_sweeps;  // sweeps of the coarsest solve inside the tail V-cycle
    int tail;           // first level of the one-block tail V-cycle; -1: coarsest too large, smoothed instead
    int tail_floats;    // shared-memory floats of the tail levels (e and r)
    int parity;         // 1 when U/V/W live in the Tmp slots
    int active;
    FastDiv fpx, fpy;        // padded P extents
    FastDiv ffx, ffy, ffz;   // NX+1, NY+1, NZ+1 (the face box)
    FastDiv fnx, fny;        // NX, NY
    float* sh[3];            // binary32 shadow of the current U, V, W (the sweeps' taps)
    int shp[3];              // row pitch of each shadow (floats): its padded x extent rounded up to 4
    int shq[4];              // shadow conversion: prefix of the components' (row, quad) counts
    FastDiv fsq[3];          // quads per shadow row
    const CUtensorMap* pmap; // 3 tensor maps per level for the TMA-staged pair: e, e2 and r
    const CUtensorMap* tmap; // 12 tensor maps over the shadows: [component][role], role 0-2 the staged
                             // tile of a sweep along axis 0-2, role 3 the axis-velocity tile
    int sw_tiles;            // staged sweep: work items (3 components x the spatial tiles)
    FastDiv swx, swy;        // staged sweep: spatial tiles along x and along y
    int warm;                // 1: a projection starts from the last pressure, 0: from zero
    int bc_off[10];          // velocity BC write sets: prefix of the nine (component, set) counts
    FastDiv bcd[9][2];       // their index decoding's divisors (bc_cell_div's d1, d2)
    Lvl lev[kMaxLev];
};

// Stage ids.  Level stages take kMaxLev consecutive ids.
enum {
    S_BC = 0, S_SWEEP, S_DIV, S_INT, S_PBC, S_GRAD, S_COARSE, S_SHADOW, S_CORR,
    S_SMOOTH = 9,
    S_RESTRICT = S_SMOOTH + kMaxLev,
    S_PROLONG = S_RESTRICT + kMaxLev,
    S_BIGCOARSE = S_PROLONG + kMaxLev,
    S_PAIR = S_BIGCOARSE + kMaxLev,
    S_PAIRN = S_PAIR + kMaxLev,
    S_SWEEPT = S_PAIRN + kMaxLev,
    S_COUNT = S_SWEEPT + 1
};

struct Shape {
    int tpb = 256;   // threads per block
    int ept = 1;     // elements per thread
    int bpsm = 8;    // persistent blocks per SM
    int var = 0;     // fused-pair stages: the tile variant (kPairVarTY, kPairVarTZ)
};

// A stage's device work list: prefix[0..n] of tiles per slot.
struct Tab {
    const int* prefix;
    int n;
    int ept;
};

// Every lane of a warp asks for the same item (callers are block-uniform
// and blocks are whole warps): lane 0 searches, the warp shares the result.
__device__ __forceinline__ int find_slot(const int* prefix, int n, int item) {
    int lo = 0;
    if ((threadIdx.x & 31) == 0) {
        int hi = n;  // prefix[lo] <= item < prefix[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (prefix[mid] <= item) lo = mid;
            else hi = mid;
        }
    }
    return __shfl_sync(0xffffffffu, lo, 0);
}

// Loop over this block's tiles; `s` is the slot, `first` the first element
// of the tile; body sees element index `el` (< the slot's count, checked by
// the body).
#define FOR_TILES(tab)                                                                   \
    for (int item = blockIdx.x, total = (tab).prefix[(tab).n]; item < total; item += gridDim.x) { \
        const int s = find_slot((tab).prefix, (tab).n, item);                            \
        const long long first = (long long)(item - (tab).prefix[s]) * blockDim.x * (tab).ept;
#define FOR_ELEMS(tab) \
        for (int k_ = 0; k_ < (tab).ept; ++k_) {      \
            const long long el = first + (long long)k_ * blockDim.x + threadIdx.x;
#define END_ELEMS }
#define END_TILES }

__device__ __forceinline__ double* cur(const InstDev& I, int field, int parity) {
    const int p = parity ^ I.parity;
    if (!p || field == 0 || field == 4) return I.slot[field];
    return I.slot[field <= 3 ? field + 4 : field - 4];
}

// --- counts of each stage's iteration space -------------------------------
__host__ __device__ inline long long bc_count(const Geom& g) {
    const long long N[3][3] = {{g.NX, g.NY, g.NZ}, {g.NY, g.NX, g.NZ}, {g.NZ, g.NX, g.NY}};
    long long c = 0;
    for (int k = 0; k < 3; ++k) c += 2 * N[k][1] * N[k][2] + 2 * (N[k][0] + 1) * N[k][2] + 2 * (N[k][0] + 1) * (N[k][1] + 2);
    return c;
}
__host__ __device__ inline long long face_box(const Geom& g) {
    return (long long)(g.NX + 1) * (g.NY + 1) * 3 * (g.NZ + 1);
}
__host__ __device__ inline long long pbc_count(const Geom& g) {
    return 2ll * g.NY * g.NZ + 2ll * (g.NX + 2) * g.NZ + 2ll * (g.NX + 2) * (g.NY + 2);
}
__host__ __device__ inline long long lvl_cells(const Lvl& L) { return (long long)L.nx * L.ny * L.nz; }

// --- binary64 stages (bit-identical to the FP64 form's cells) -------------
__global__ void kb_bc(const InstDev* inst, Status* st, Tab tab, int parity, int gate) {
    FOR_TILES(tab)
    const InstDev& I = inst[s];
    if (gated(&st[s], gate)) continue;
    AF_PTR(double) u = view(cur(I, 1, parity), I.g.u.count, DK_BC, s);
    AF_PTR(double) v = view(cur(I, 2, parity), I.g.v.count, DK_BC, s);
    AF_PTR(double) w = view(cur(I, 3, parity), I.g.w.count, DK_BC, s);
    int off[10];  // the offsets in registers: no reload per element
#pragma unroll
    for (int j = 0; j < 10; ++j) off[j] = I.bc_off[j];
    FOR_ELEMS(tab)
    if (el >= off[9]) break;
    // Write set k = 3 * component + set holds elements bc_off[k] ..
    // bc_off[k+1]-1 (bc_set_count in that order).
    const int e = (int)el;
    int k = 0, base = 0;
#pragma unroll
    for (int j = 1; j < 9; ++j)
        if (e >= off[j]) {
            k = j;
            base = off[j];
        }
    const int comp = k / 3;
    bc_cell_div(bc_comp(I.g, comp, u, v, w), I.g.G, k - 3 * comp, (unsigned)(e - base), I.bcd[k][0], I.bcd[k][1]);
    END_ELEMS
    END_TILES
}

__global__ void kb_div(const InstDev* inst, Status* st, Tab tab, int parity, int gate) {
    FOR_TILES(tab)
    const InstDev& I = inst[s];
    if (gated(&st[s], gate)) continue;
    const Geom& g = I.g;
    const long long n = (long long)g.p.nx * g.p.ny * g.p.nz;
    FOR_ELEMS(tab)
    if (el >= n) break;
    const unsigned e = (unsigned)el, r = I.fpx.div(e), z = I.fpy.div(r);
    div_cell(g, view((const double*)cur(I, 1, parity), g.u.count, DK_DIV, s),
             view((const double*)cur(I, 2, parity), g.v.count, DK_DIV, s),
             view((const double*)cur(I, 3, parity), g.w.count, DK_DIV, s), view(I.slot[0], g.p.count, DK_DIV, s),
             view(I.slot[4], g.p.count, DK_DIV, s), view(I.b, g.p.count, DK_DIV, s), I.div_scale, I.h2, !I.warm,
             (int)(e - r * g.p.nx), (int)(r - z * g.p.ny), (int)z);
    END_ELEMS
    END_TILES
}

__global__ void kb_pbc(const InstDev* inst, Status* st, Tab tab, int gate) {
    FOR_TILES(tab)
    const InstDev& I = inst[s];
    if (gated(&st[s], gate)) continue;
    const Geom& g = I.g;
    const long long c0 = pbc_set_count(g, 0), c1 = pbc_set_count(g, 1), n = pbc_count(g);
    FOR_ELEMS(tab)
    if (el >= n) break;
    AF_PTR(double) p = view(I.slot[0], g.p.count, DK_PBC, s);
    if (el < c0) pbc_cell(g, p, 0, el);
    else if (el < c0 + c1) pbc_cell(g, p, 1, el - c0);
    else pbc_cell(g, p, 2, el - c0 - c1);
    END_ELEMS
    END_TILES
}

// subtractGradient over every face, a warp per (component, y, z) face row.
// scratch = 1 (the autotuner's timing runs) stores the new values into the
// Tmp fields instead, so timing leaves the slots' velocities untouched.
__global__ void kb_grad(const InstDev* inst, Status* st, Tab tab, int parity, int gate, int scratch) {
    FOR_TILES(tab)
    const InstDev& I = inst[s];
    if (gated(&st[s], gate)) continue;
    const Geom& g = I.g;
    const long long rows = 3ll * (g.NY + 1) * (g.NZ + 1);
    AF_PTR(double) u = view(cur(I, 1, parity), g.u.count, DK_GRAD, s);
    AF_PTR(double) v = view(cur(I, 2, parity), g.v.count, DK_GRAD, s);
    AF_PTR(double) w = view(cur(I, 3, parity), g.w.count, DK_GRAD, s);
    FOR_ELEMS(tab)
    const long long row = el >> 5;
    if (row >= rows) break;
    const int lane = (int)(el & 31);
    const unsigned r = (unsigned)row, r2 = I.ffy.div(r), cc = I.ffz.div(r2);
    const int c = (int)cc;
    const int y = g.G + (int)(r - r2 * (unsigned)(g.NY + 1)), z = g.G + (int)(r2 - cc * (unsigned)(g.NZ + 1));
    if (y >= g.G + g.NY + (c == 1) || z >= g.G + g.NZ + (c == 2)) continue;
    const int x1 = g.G + g.NX + (c == 0);
    AF_PTR(const double) f = c == 0 ? u : (c == 1 ? v : w);
    const long long fc = c == 0 ? g.u.count : (c == 1 ? g.v.count : g.w.count);
    AF_PTR(double) out = scratch ? view(cur(I, 5 + c, parity), fc, DK_GRAD, s) : (c == 0 ? u : (c == 1 ? v : w));
    AF_PTR(const double) p = view((const double*)I.slot[0], g.p.count, DK_GRAD, s);
    for (int x = g.G + lane; x < x1; x += 32) grad_face_to(g, p, f, out, I.grad_scale, c, x, y, z);
    END_ELEMS
    END_TILES
}

// binary32 shadow of the current U, V, W (every element, ghosts included),
// converted once per sweep instead of once per tap.  A shadow row holds the
// field row's nx values and is padded to a multiple of four floats (the row
// pitch shp), so rows start on 16-byte boundaries and a TMA tensor map can
// describe the shadow.  A thread converts four consecutive elements of one
// row and stores them with one 16-byte store (padding: zeros).
__global__ void kb_shadow(const InstDev* inst, Tab tab, int parity) {
    FOR_TILES(tab)
    const InstDev& I = inst[s];
    const long long n = I.shq[3];
    FOR_ELEMS(tab)
    if (el >= n) break;
    const int e = (int)el;
    const int f = e < I.shq[1] ? 0 : (e < I.shq[2] ? 1 : 2);
    const unsigned r = (unsigned)(e - I.shq[f]);
    const unsigned row = I.fsq[f].div(r), q = r - row * I.fsq[f].d;
    const Dims& d = f == 0 ? I.g.u : (f == 1 ? I.g.v : I.g.w);
    AF_PTR(const double) src =
        view((const double*)cur(I, 1 + f, parity), d.count, DK_SHADOW, s) + ((long long)row * d.nx + 4 * q);
    AF_PTR(float) dst = view(I.sh[f], (long long)I.shp[f] * d.ny * d.nz, DK_SHADOW, s) +
                        ((long long)row * I.shp[f] + 4 * q);
    const int left = d.nx - 4 * (int)q;
    float4 o;
    o.x = f64_to_f32(src[0]);
    o.y = left > 1 ? f64_to_f32(src[1]) : 0.0f;
    o.z = left > 2 ? f64_to_f32(src[2]) : 0.0f;
    o.w = left > 3 ? f64_to_f32(src[3]) : 0.0f;
    AF_VEC(float4, dst, 0, 4) = o;
    END_ELEMS
    END_TILES
}

// One axis sweep of every face.  A warp owns one (component, y, z) face row
// (32 lanes per row of the face box) and its lanes stride over x; taps come
// from the binary32 shadow.  Per row the kernel fixes the component (a
// template parameter), the row pointers of the face's own field and of the
// axis component that gives the face velocity, and the four 32-bit offsets
// of that velocity's taps, so a face costs its nine loads, the arithmetic
// of mx_face_update and one store.
template <int AX, int C>
__device__ __forceinline__ void sweep_row(const InstDev& I, Status* st, AF_PTR(double) AF_RESTRICT dd, int y, int z,
                                          int x0, int x1, int phase, int slot) {
    const Geom& g = I.g;
    const Dims& d = C == 0 ? g.u : (C == 1 ? g.v : g.w);
    const Dims& a = AX == 0 ? g.u : (AX == 1 ? g.v : g.w);
    const long long py = I.shp[C], pz = py * d.ny;  // shadow strides
    AF_PTR(const float) AF_RESTRICT src =
        view((const float*)I.sh[C], py * d.ny * d.nz, DK_SWEEP_ROWS, slot) + (y * py + z * pz);
    dd += (long long)y * d.sy + (long long)z * d.sz;
    const long long s = AX == 0 ? 1 : (AX == 1 ? py : pz);
    const int na = AX == 0 ? d.nx : (AX == 1 ? d.ny : d.nz);
    // Face velocity taps (summed by mx_face_vel4): offsets from (x, y, z) in the axis
    // component's shadow, in the order they are summed.
    const int ay = I.shp[AX], az = I.shp[AX] * a.ny;
    AF_PTR(const float) AF_RESTRICT va = view((const float*)I.sh[AX], (long long)az * a.nz, DK_SWEEP_ROWS, slot) +
                                         ((long long)y * ay + (long long)z * az);
    int o0 = 0, o1 = 0, o2 = 0, o3 = 0;
    if (C == 0 && AX == 1) { o0 = -1; o1 = 0; o2 = ay - 1; o3 = ay; }
    if (C == 0 && AX == 2) { o0 = -1; o1 = 0; o2 = az - 1; o3 = az; }
    if (C == 1 && AX == 0) { o0 = -ay; o1 = 1 - ay; o2 = 0; o3 = 1; }
    if (C == 1 && AX == 2) { o0 = -ay; o1 = 0; o2 = az - ay; o3 = az; }
    if (C == 2 && AX == 0) { o0 = -az; o1 = 1 - az; o2 = 0; o3 = 1; }
    if (C == 2 && AX == 1) { o0 = -az; o1 = ay - az; o2 = 0; o3 = ay; }
    const float dt_invh = I.dt_invh, lam = I.lam;
    auto vel_at = [&](int x) {
        return C == AX ? src[x] : mx_face_vel4(va[x + o0], va[x + o1], va[x + o2], va[x + o3]);
    };
    // The next face's velocity taps load before this face's dependent taps,
    // so a lane keeps two faces' loads in flight.
    float vel_next = x0 < x1 ? vel_at(x0) : 0.0f;
    for (int x = x0; x < x1; x += 32) {
        const float vel = vel_next;
        if (x + 32 < x1) vel_next = vel_at(x + 32);
        const int ca = AX == 0 ? x : (AX == 1 ? y : z);
        float res;
        if (!mx_face_update(src + x, s, vel, ca, na, dt_invh, lam, &res)) {
            atomicMin(&st->fault_gate, st->step * 8u + (unsigned)phase);
            atomicMin(&st->fault_key, fault_key(C, x, y, z));
            continue;
        }
        dd[x] = (double)res;  // widening is exact
    }
}

// Iteration space of the sweep: 32 lanes per face row of the three
// components, then the U rows' last faces (x = G + NX), 32 rows to a warp:
// a U row has NX + 1 faces, and with NX a multiple of 32 its last face would
// otherwise cost a whole warp iteration of one lane.
__host__ __device__ inline long long sweep_box(const Geom& g) {
    return 32ll * (3ll * (g.NY + 1) * (g.NZ + 1) + ((long long)g.NY * g.NZ + 31) / 32);
}

template <int AX>
__global__ void kb_sweep(const InstDev* inst, Status* st, Tab tab, int parity, int phase) {
    FOR_TILES(tab)
    const InstDev& I = inst[s];
    if (gated(&st[s], phase)) continue;
    const Geom& g = I.g;
    const long long rows = 3ll * (g.NY + 1) * (g.NZ + 1), n = sweep_box(g);
    FOR_ELEMS(tab)
    if (el >= n) break;
    const long long row = el >> 5;
    const int lane = (int)(el & 31);
    if (row >= rows) {
        // Last U face of U row q.
        const long long q = (row - rows) * 32 + lane;
        if (q >= (long long)g.NY * g.NZ) continue;
        const unsigned zz = I.fny.div((unsigned)q);
        const int y = g.G + (int)((unsigned)q - zz * (unsigned)g.NY), z = g.G + (int)zz;
        sweep_row<AX, 0>(I, st + s, view(cur(I, 5, parity), g.u.count, DK_SWEEP_ROWS, s), y, z, g.G + g.NX,
                         g.G + g.NX + 1, phase, s);
        continue;
    }
    const unsigned r = (unsigned)row, r2 = I.ffy.div(r), cc = I.ffz.div(r2);
    const int c = (int)cc;
    const int y = g.G + (int)(r - r2 * (unsigned)(g.NY + 1)), z = g.G + (int)(r2 - cc * (unsigned)(g.NZ + 1));
    if (y >= g.G + g.NY + (c == 1) || z >= g.G + g.NZ + (c == 2)) continue;
    const int x0 = g.G + lane, x1 = g.G + g.NX;  // the U rows' last faces come after the rows
    if (c == 0) sweep_row<AX, 0>(I, st + s, view(cur(I, 5, parity), g.u.count, DK_SWEEP_ROWS, s), y, z, x0, x1, phase, s);
    else if (c == 1)
        sweep_row<AX, 1>(I, st + s, view(cur(I, 6, parity), g.v.count, DK_SWEEP_ROWS, s), y, z, x0, x1, phase, s);
    else sweep_row<AX, 2>(I, st + s, view(cur(I, 7, parity), g.w.count, DK_SWEEP_ROWS, s), y, z, x0, x1, phase, s);
    END_ELEMS
    END_TILES
}

// --- staged tile sweep ---------------------------------------------------
// The same sweep with its gathers served from shared memory.  A block owns a
// tile of kSwTX x kSwTY x kSwTZ faces of one component, x tiles starting at
// the first interior face (G + 32k; a U row's extra last face joins its last
// tile).  One thread stages, with TMA tensor loads over the binary32
// shadows, the tile of the face's own component with a halo along the sweep
// axis (at least 4 cells along x, kSwHA along y or z: the diffusion taps and
// every backtrace with |dt*vel/h| < kSwHA) and, when the component is not
// the sweep axis's, the tile of the axis component whose four faces give the
// face velocity (a one-cell halo).  A TMA box must start on a 16-byte
// boundary, so each box starts at the x below its tile's halo rounded down
// to a multiple of four (sw_box_x) and is wide enough for any rounding.
// Backtraces that leave the staged halo read the shadow in global memory
// instead.  Every face's arithmetic is the row kernel's (mx_face_vel4,
// mx_backtrace, mx_face_value): the same bits.
// Six planes deep: a thread computes six faces per tile, so the tile's
// set-up (decode, slot search, geometry, transfer wait, barriers) is spread
// over more faces than with four planes, while four blocks still fit an SM
// (measured per sweep launch at 256^3: 4 planes 268-281 us, 6 planes
// 236-250 us, 8 planes at three blocks per SM 290-311 us).
constexpr int kSwTX = 32, kSwTY = 8, kSwTZ = 6, kSwHA = 2, kSwThreads = kSwTX * kSwTY;
// Box roles: 0-2 the own component for a sweep along x, y, z; 3 the axis
// component.  First x of a box (a multiple of 4) and its width.
__host__ __device__ constexpr int sw_box_x(int role, int x0) {
    return (role == 0 ? x0 - 4 : (role == 3 ? x0 - 1 : x0)) & ~3;
}
__host__ __device__ constexpr int sw_bx(int role) {
    return role == 0 ? kSwTX + 12 : (role == 3 ? kSwTX + 8 : kSwTX + 4);
}
__host__ __device__ constexpr int sw_by(int role) {
    return role == 1 ? kSwTY + 2 * kSwHA : (role == 3 ? kSwTY + 2 : kSwTY);
}
__host__ __device__ constexpr int sw_bz(int role) {
    return role == 2 ? kSwTZ + 2 * kSwHA : (role == 3 ? kSwTZ + 2 : kSwTZ);
}
__host__ __device__ constexpr int sw_box_floats(int role) { return sw_bx(role) * sw_by(role) * sw_bz(role); }
__host__ __device__ constexpr int sw_max(int a, int b) { return a > b ? a : b; }
// Floats of the largest own-component box, rounded up to 32 (128 bytes: the
// buffers are TMA destinations).
constexpr int kSwOwnMax = (sw_max(sw_box_floats(0), sw_max(sw_box_floats(1), sw_box_floats(2))) + 31) / 32 * 32;
constexpr int kSwAxCount = (kSwTX + 8) * (kSwTY + 2) * (kSwTZ + 2);
static_assert(kSwAxCount % 32 == 0, "axis-box buffers start on 128-byte boundaries");
// Two buffer pairs (own, axis) per block, in dynamic shared memory.
constexpr size_t kSwSmem = (size_t)2 * (kSwOwnMax + kSwAxCount) * sizeof(float);
static_assert(sw_bx(0) * sw_by(0) * sw_bz(0) <= kSwOwnMax && sw_bx(1) * sw_by(1) * sw_bz(1) <= kSwOwnMax &&
              sw_bx(2) * sw_by(2) * sw_bz(2) <= kSwOwnMax, "own box exceeds its buffer");
static_assert(sw_bx(3) * sw_by(3) * sw_bz(3) == kSwAxCount, "axis box size");
// A wait on a TMA transfer gives up after this many polls (each poll itself
// blocks for a bounded, hardware-defined time); the kernel then records the
// failure in the batch's diagnostic word and returns.
constexpr unsigned kSwSpinLimit = 1u << 22;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// A wait also gives up after this long (a transfer lands in microseconds).
constexpr unsigned long long kWaitLimitNs = 200000000ull;
// Suspend-time hint of one poll: a waiting thread sleeps in the barrier
// until the phase completes (or this long) instead of re-issuing the poll,
// so waiting warps take no issue slots from the working ones.
constexpr unsigned kPollSuspendNs = 20000u;
__device__ __forceinline__ bool mbar_try_wait_sleep(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "n"(kPollSuspendNs)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Polls the barrier's phase `parity` at most kSwSpinLimit times and for at
// most kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 1; it < kSwSpinLimit; ++it) {
        if (mbar_try_wait_sleep(bar, parity)) return true;
        if ((it & 15u) == 0u && global_ns() - t0 > kWaitLimitNs) return false;
    }
    return false;
}
// Whether an earlier kernel of the work gave up a wait (its results are
// invalid, so later staged kernels return at once instead of waiting again).
__device__ __forceinline__ bool diag_set(const unsigned* diag) { return *(const volatile unsigned*)diag != 0u; }
__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_addr(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// Faces of one tile of component C (the loads have landed in own / axv).
template <int AX, int C>
__device__ __forceinline__ void sweep_tile_faces(const InstDev& I, Status* st, const float* own_, const float* axv_,
                                                 double* __restrict__ dd_, int x0, int y0, int z0, int phase,
                                                 int slot) {
    const Geom& g = I.g;
    const Dims& d = C == 0 ? g.u : (C == 1 ? g.v : g.w);
    AF_PTR(const float) own = view(own_, (long long)kSwOwnMax, DK_SWEEP_TMA, slot);
    AF_PTR(const float) axv = view(axv_, (long long)kSwAxCount, DK_SWEEP_TMA, slot);
    AF_PTR(double) AF_RESTRICT dd = view(dd_, d.count, DK_SWEEP_TMA, slot);
    constexpr int BX = sw_bx(AX), BY = sw_by(AX), BZ = sw_bz(AX);
    constexpr int SO = AX == 0 ? 1 : (AX == 1 ? BX : BX * BY);  // own-box stride along the sweep axis
    constexpr int AXX = sw_bx(3), AXY = sw_by(3);
    // Axis-box strides along the component's axis and the sweep axis.
    constexpr int EC = C == 0 ? 1 : (C == 1 ? AXX : AXX * AXY);
    constexpr int EA = AX == 0 ? 1 : (AX == 1 ? AXX : AXX * AXY);
    const int ox = sw_box_x(AX, x0), oy = y0 - (AX == 1 ? kSwHA : 0), oz = z0 - (AX == 2 ? kSwHA : 0);
    const int oa = AX == 0 ? ox : (AX == 1 ? oy : oz);  // own box's first coordinate along the axis
    const int ax0 = sw_box_x(3, x0);
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    const int y = y0 + ly;
    const int G = g.G;
    if (y >= G + g.NY + (C == 1)) return;
    // The last tile of a row runs to the component's last face.
    const int xhi = x0 + kSwTX >= G + g.NX ? G + g.NX + (C == 0) : x0 + kSwTX;
    const int zend = min(z0 + kSwTZ, G + g.NZ + (C == 2));
    const int na = AX == 0 ? d.nx : (AX == 1 ? d.ny : d.nz);
    const long long py = I.shp[C], pz = py * d.ny;
    const long long gs = AX == 0 ? 1 : (AX == 1 ? py : pz);
    const float dt_invh = I.dt_invh, lam = I.lam;
    const long long dsy = d.sy, dsz = d.sz;
    const float* shc = I.sh[C];
    for (int x = x0 + lx; x < xhi; x += kSwTX) {
        // Walk z with every index advanced by its plane stride: the face's
        // own box, the axis box and the binary64 destination.
        int io = ((z0 - oz) * BY + (y - oy)) * BX + (x - ox);
        int ia = (AXY + (y - y0 + 1)) * AXX + (x - ax0);
        AF_PTR(double) dz = dd + ((long long)x + (long long)y * dsy + (long long)z0 * dsz);
        for (int z = z0; z < zend; ++z, io += BX * BY, ia += AXX * AXY, dz += dsz) {
            float vel;
            if (C == AX) {
                vel = own[io];
            } else {
                // The row kernel's tap order: before the sweep axis's own
                // component, (-e_C, 0, e_AX - e_C, e_AX); after it,
                // (-e_C, e_AX - e_C, 0, e_AX).
                if (AX > C) vel = mx_face_vel4(axv[ia - EC], axv[ia], axv[ia + EA - EC], axv[ia + EA]);
                else vel = mx_face_vel4(axv[ia - EC], axv[ia + EA - EC], axv[ia], axv[ia + EA]);
            }
            const int ca = AX == 0 ? x : (AX == 1 ? y : z);
            int i0;
            float t;
            if (!mx_backtrace(vel, ca, na, dt_invh, &i0, &t)) {
                atomicMin(&st->fault_gate, st->step * 8u + (unsigned)phase);
                atomicMin(&st->fault_key, fault_key(C, x, y, z));
                continue;
            }
            float d0, d1;
            const int rel = i0 - ca;
            if (i0 >= oa && i0 + 1 < oa + (AX == 0 ? BX : (AX == 1 ? BY : BZ))) {
                d0 = own[io + rel * SO];
                d1 = own[io + (rel + 1) * SO];
            } else {
                AF_PTR(const float) gp =
                    view(shc, pz * d.nz, DK_SWEEP_TMA, slot) + (x + y * py + z * pz + rel * gs);
                d0 = gp[0];
                d1 = gp[gs];
            }
            const float res = mx_face_value(t, d0, d1, own[io - SO], own[io], own[io + SO], lam);
            dz[0] = (double)res;  // widening is exact
        }
    }
}

// A decoded tile of the staged sweep: slot, component and first face; dead
// when past the work list or its slot is gated by a fault.
struct SwTile {
    int s, c, x0, y0, z0;
    bool live;
};

__device__ __forceinline__ SwTile sw_decode(const InstDev* inst, const Status* st, const Tab& tab, int item, int total,
                                            int phase) {
    SwTile t{0, 0, 0, 0, 0, false};
    if (item >= total) return t;
    t.s = find_slot(tab.prefix, tab.n, item);
    const InstDev& I = inst[t.s];
    if (gated(&st[t.s], phase)) return t;
    // The three components of one spatial tile are consecutive items, so
    // the axis component's box, staged again for the other two, is still in
    // L2.  A spatial tile past one component's last face row or plane holds
    // no faces of it.
    const unsigned local = (unsigned)(item - tab.prefix[t.s]);
    const unsigned r = local / 3u;
    t.c = (int)(local - 3u * r);
    const unsigned q1 = I.swx.div(r), q2 = I.swy.div(q1);
    t.x0 = I.g.G + (int)(r - q1 * I.swx.d) * kSwTX;
    t.y0 = I.g.G + (int)(q1 - q2 * I.swy.d) * kSwTY;
    t.z0 = I.g.G + (int)q2 * kSwTZ;
    t.live = t.y0 < I.g.G + I.g.NY + (t.c == 1) && t.z0 < I.g.G + I.g.NZ + (t.c == 2);
    return t;
}

// Thread 0: the TMA loads of tile t into one buffer pair.  The buffers' last
// reads (generic proxy) finished before the caller's barrier; the fence
// orders them before these writes (async proxy).
template <int AX>
__device__ __forceinline__ void sw_issue(const InstDev& I, const SwTile& t, float* own, float* axv,
                                         unsigned long long* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    constexpr unsigned own_bytes = sw_bx(AX) * sw_by(AX) * sw_bz(AX) * 4u;
    mbar_expect_tx(bar, own_bytes + (t.c != AX ? kSwAxCount * 4u : 0u));
    tma_load_3d(own, I.tmap + t.c * 4 + AX, sw_box_x(AX, t.x0), t.y0 - (AX == 1 ? kSwHA : 0),
                t.z0 - (AX == 2 ? kSwHA : 0), bar);
    if (t.c != AX) tma_load_3d(axv, I.tmap + AX * 4 + 3, sw_box_x(3, t.x0), t.y0 - 1, t.z0 - 1, bar);
}

// Persistent blocks walk their tiles with two buffer pairs: the loads of the
// next tile are in flight while the current tile's faces are computed.
template <int AX>
__global__ void __launch_bounds__(kSwThreads, 4)
    kb_sweep_tma(const InstDev* inst, Status* st, Tab tab, int parity, int phase, unsigned* diag) {
    extern __shared__ __align__(128) float swsm[];
    // Buffer pair k: own-component box and axis box.
    auto own = [&](int k) { return swsm + k * kSwOwnMax; };
    auto axv = [&](int k) { return swsm + 2 * kSwOwnMax + k * kSwAxCount; };
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ unsigned stop;
    if (smem_addr(swsm) & 127u) {  // the buffers are TMA destinations: 128-byte aligned base
        if (threadIdx.x == 0) atomicOr(diag, 4u);
        return;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        stop = diag_set(diag) ? 1u : 0u;
    }
    __syncthreads();
    if (stop) return;
    const int total = tab.prefix[tab.n];
    unsigned ph = 0u;  // bit k: the phase parity buffer k waits for next
    int item = blockIdx.x, k = 0;
    SwTile tile = sw_decode(inst, st, tab, item, total, phase);
    if (tile.live && threadIdx.x == 0) sw_issue<AX>(inst[tile.s], tile, own(0), axv(0), &bar[0]);
    while (item < total) {
        const int next_item = item + gridDim.x;
        const SwTile next = sw_decode(inst, st, tab, next_item, total, phase);
        if (next.live && threadIdx.x == 0) sw_issue<AX>(inst[next.s], next, own(k ^ 1), axv(k ^ 1), &bar[k ^ 1]);
        if (tile.live) {
            const bool ok = __syncthreads_and(mbar_wait_bounded(&bar[k], (ph >> k) & 1u) ? 1 : 0) != 0;
            ph ^= 1u << k;
            if (!ok) {
                // A transfer did not land in time: record it, give the copies
                // in flight a second bounded wait, and stop.
                if (threadIdx.x == 0) {
                    atomicOr(diag, 1u);
                    mbar_wait_bounded(&bar[k], ((ph >> k) & 1u) ^ 1u);
                    if (next.live) mbar_wait_bounded(&bar[k ^ 1], (ph >> (k ^ 1)) & 1u);
                }
                __syncthreads();
                return;
            }
            const InstDev& I = inst[tile.s];
            double* dd = cur(I, 5 + tile.c, parity);
            if (tile.c == 0)
                sweep_tile_faces<AX, 0>(I, st + tile.s, own(k), axv(k), dd, tile.x0, tile.y0, tile.z0, phase, tile.s);
            else if (tile.c == 1)
                sweep_tile_faces<AX, 1>(I, st + tile.s, own(k), axv(k), dd, tile.x0, tile.y0, tile.z0, phase, tile.s);
            else sweep_tile_faces<AX, 2>(I, st + tile.s, own(k), axv(k), dd, tile.x0, tile.y0, tile.z0, phase, tile.s);
        }
        __syncthreads();  // every thread is done with buffer k before it is loaded again
        tile = next;
        item = next_item;
        k ^= 1;
    }
}

__global__ void kb_tick(const InstDev* inst, Status* st, int n) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        if (inst[s].active) st[s].step += 1;
}

// --- refinement control ---------------------------------------------------
__global__ void kb_init(const InstDev* inst, Ctl* ctl, int n) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl[n].nv = 0xFFFFFFFFu;  // until a check counts them
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        ctl[s].maxr_bits = 0;
        ctl[s].passes = 0;
        ctl[s].stopped = inst[s].active ? 0u : 1u;
        ctl[s].nv = 0u;
        ctl[s].vtotal = 0u;
        ctl[s].last_div = 0;
    }
}

// r = b - L(p) in binary64 over the interior, r (binary32) for the inner
// solve, inner solution zeroed, max|r| reduced per slot.  In the loop a
// converged slot is skipped.
__device__ __forceinline__ void warp_max_commit(unsigned long long m, unsigned long long* out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// r = b - L(p) in binary64 over the interior, r (binary32) for the inner
// solve, inner solution zeroed, max|r| reduced per slot.  A block keeps its
// running maximum over consecutive tiles of one slot and commits it (one
// atomic per warp) when the slot changes or the block finishes, so the
// atomics are per block, not per warp-sized tile.  In the loop a converged
// slot is skipped.
__global__ void kb_residual(const InstDev* inst, Status* st, Ctl* ctl, Tab tab, int gate, int in_loop) {
    int held = -1;
    unsigned long long m = 0;
    for (int item = blockIdx.x, total = tab.prefix[tab.n]; item < total; item += gridDim.x) {
        const int s = find_slot(tab.prefix, tab.n, item);
        const long long first = (long long)(item - tab.prefix[s]) * blockDim.x * tab.ept;
        const InstDev& I = inst[s];
        if (gated(&st[s], gate) || (in_loop && ctl[s].stopped)) continue;
        if (s != held) {
            if (held >= 0) warp_max_commit(m, &ctl[held].maxr_bits);
            held = s;
            m = 0;
        }
        const Geom& g = I.g;
        const long long nl0 = lvl_cells(I.lev[0]);
        AF_PTR(const double) AF_RESTRICT p = view((const double*)I.slot[0], g.p.count, DK_RESIDUAL, s);
        AF_PTR(const double) AF_RESTRICT bb = view((const double*)I.b, g.p.count, DK_RESIDUAL, s);
        AF_PTR(float) AF_RESTRICT r0 = view(I.lev[0].r, nl0, DK_RESIDUAL, s);
        AF_PTR(float) AF_RESTRICT e0 = view(I.lev[0].e, nl0, DK_RESIDUAL, s);
        const long long n = (long long)g.NX * g.NY * g.NZ;
        for (int k = 0; k < tab.ept; ++k) {
            const long long el = first + (long long)k * blockDim.x + threadIdx.x;
            if (el >= n) continue;
            const unsigned e = (unsigned)el, r2 = I.fnx.div(e), zz = I.fny.div(r2);
            const int xi = (int)(e - r2 * (unsigned)g.NX), yi = (int)(r2 - zz * (unsigned)g.NY), zi = (int)zz;
            const long long sy = g.p.sy, sz = g.p.sz;
            const long long i = (g.G + xi) + (g.G + yi) * sy + (g.G + zi) * sz;
            const double pc = p[i];
            const double xm = xi > 0 ? p[i - 1] : pc;
            const double xp = xi < g.NX - 1 ? p[i + 1] : pc;
            const double ym = yi > 0 ? p[i - sy] : pc;
            const double yp = yi < g.NY - 1 ? p[i + sy] : pc;
            const double zm = zi > 0 ? p[i - sz] : pc;
            const double zp = zi < g.NZ - 1 ? p[i + sz] : pc;
            const double res = bb[i] - fma(-6.0, pc, ((xm + xp) + (ym + yp)) + (zm + zp));
            r0[el] = f64_to_f32(res);
            e0[el] = 0.0f;
            // |res| and NaN on the bit pattern (integer pipe); NaN reads as
            // +Inf so the loop stops.
            const unsigned long long a = (unsigned long long)__double_as_longlong(res) & ~kSign;
            const unsigned long long v = a > 0x7FF0000000000000ull ? 0x7FF0000000000000ull : a;
            m = v > m ? v : m;
        }
    }
    if (held >= 0) warp_max_commit(m, &ctl[held].maxr_bits);
}

// p += e over the interior, a warp per (y, z) row (32 lanes per row).
__global__ void kb_correct(const InstDev* inst, Ctl* ctl, Tab tab) {
    FOR_TILES(tab)
    const InstDev& I = inst[s];
    if (ctl[s].stopped) continue;
    const Geom& g = I.g;
    const long long rows = (long long)g.NY * g.NZ;
    FOR_ELEMS(tab)
    const long long row = el >> 5;
    if (row >= rows) break;
    const int lane = (int)(el & 31);
    const unsigned zz = I.fny.div((unsigned)row);
    const int y = (int)((unsigned)row - zz * (unsigned)g.NY), z = (int)zz;
    AF_PTR(double) p = view(I.slot[0], g.p.count, DK_CORRECT, s) +
                       (g.G + (long long)(g.G + y) * g.p.sy + (long long)(g.G + z) * g.p.sz);
    AF_PTR(const float) e = view((const float*)I.lev[0].e, lvl_cells(I.lev[0]), DK_CORRECT, s) +
                            ((long long)g.NX * y + (long long)g.NX * g.NY * z);
    for (int x = lane; x < g.NX; x += 32) p[x] += f32_to_f64(e[x]);
    END_ELEMS
    END_TILES
}

// One block: per slot, whether another refinement pass runs; the WHILE
// condition is "any slot continues".  Bounded by each slot's max_refine.
__global__ void kb_check(const InstDev* inst, Status* st, Ctl* ctl, int n, cudaGraphConditionalHandle h, int use_cond,
                         int count_pass, int gate, int vcycles, double pass_floor) {
    __shared__ unsigned most;  // V-cycles of the next pass, most over the slots
    if (threadIdx.x == 0) most = 0u;
    __syncthreads();
    int any = 0;
    for (int s = threadIdx.x; s < n; s += blockDim.x) {
        const InstDev& I = inst[s];
        if (!I.active) continue;
        Ctl& c = ctl[s];
        const double r = __longlong_as_double((long long)c.maxr_bits);
        c.maxr_bits = 0;
        if (c.stopped) continue;
        const double div = I.res_scale * r;
        // A pass that removes less than a tenth of max|r| has reached the
        // binary64 round-off floor of the residual (|B| * 2^-53 and up):
        // stop there rather than spin to the pass cap.
        const bool stalled = count_pass && div > 0.9 * c.last_div;
        const double prev = c.last_div;
        c.last_div = div;
        if (count_pass) c.passes += 1;
        const bool more =
            !gated(&st[s], gate) && div > I.thresh && !isinf(div) && !stalled && c.passes < I.max_refine;
        // The last pass often needs fewer V-cycles than the others: from the
        // reduction per V-cycle the pass just achieved, predict how many more
        // bring max|div| below half the threshold, and run only those.
        // The first pass of a projection uses the factor the slot's last
        // projection measured.
        if (count_pass) c.vtotal += c.nv ? c.nv : (unsigned)vcycles;
        if (count_pass && prev > 0.0) {
            const double ran = c.nv ? (double)c.nv : (double)vcycles;
            const double f = pow(div / prev, 1.0 / ran);
            if (f < 1.0) c.vfac = f;
        }
        // A pass cannot take max|r| below its binary32 floor (the inner
        // solve's correction carries about 24 bits), so V-cycles past
        // log(pass_floor) / log(vfac) are cut as well (pass_floor = 0: no
        // such cut).
        unsigned nv = 0u;
        if (more && c.vfac > 0.0 && c.vfac < 1.0) {
            double k = ceil(log(0.5 * I.thresh / div) / log(c.vfac));
            if (pass_floor > 0.0) k = fmin(k, ceil(log(pass_floor) / log(c.vfac)));
            if (k < 1.0) k = 1.0;
            if (k < (double)vcycles) nv = (unsigned)k;
        }
        c.nv = nv;
        if (!more) c.stopped = 1;
        else atomicMax(&most, nv ? nv : (unsigned)vcycles);
        any |= more ? 1 : 0;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) ctl[n].nv = most;
    if (threadIdx.x == 0 && use_cond) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// --- binary32 multigrid ---------------------------------------------------
__device__ __forceinline__ long long lidx(int x, int y, int z, int nx, int ny) {
    return x + (long long)nx * (y + (long long)ny * z);
}

// Binary32 cell formulas of the multigrid with every rounding written out
// (no contraction left to the compiler), so the per-level kernels, the fused
// red-black pair and the one-block tail V-cycle compute the same bits.
// Over-relaxed update of one cell from its value c:
//   c + omega * ((wx*sx + wy*sy + wz*sz - r) / (2*(wx+wy+wz)) - c).
// omega = 1.5 was measured best on cubes of 128^3-512^3 (refinement passes
// to max|div| <= 1e-10 per projection at 256^3: 8 at omega = 1, 6 at 1.3,
// 5 at 1.5, 7 at 1.6).
constexpr float kMgOmega = 1.5f;
__device__ __forceinline__ float mg_relax(const Lvl& L, float sx, float sy, float sz, float r, float inv, float c) {
    const float v = __fmul_rn(__fsub_rn(__fmaf_rn(L.wz, sz, __fmaf_rn(L.wy, sy, __fmul_rn(L.wx, sx))), r), inv);
    return __fmaf_rn(kMgOmega, __fsub_rn(v, c), c);
}
// Residual of one cell: r - (wx*dxx + wy*dyy + wz*dzz), d** the second differences.
__device__ __forceinline__ float mg_res(const Lvl& L, float sx, float sy, float sz, float c, float r) {
    const float c2 = 2.0f * c;
    return __fsub_rn(r, __fmaf_rn(L.wz, __fsub_rn(sz, c2), __fmaf_rn(L.wy, __fsub_rn(sy, c2), __fmul_rn(L.wx, __fsub_rn(sx, c2)))));
}
// Trilinear weights (a* on the parent, b* = 1 - a* on its neighbour).
__device__ __forceinline__ float mg_interp(float ax, float ay, float az, float e000, float e100, float e010, float e110,
                                           float e001, float e101, float e011, float e111) {
    const float bx = 1.0f - ax, by = 1.0f - ay, bz = 1.0f - az;
    auto lx = [&](float p, float q) { return __fmaf_rn(bx, q, __fmul_rn(ax, p)); };
    auto ly = [&](float p, float q) { return __fmaf_rn(by, q, __fmul_rn(ay, p)); };
    const float z0 = ly(lx(e000, e100), lx(e010, e110)), z1 = ly(lx(e001, e101), lx(e011, e111));
    return __fmaf_rn(bz, z1, __fmul_rn(az, z0));
}

// One red-black colour sweep of L e = r in place.  A warp owns one (y, z) row
// and its lanes stride over the row's cells of the colour; the neighbour
// rows are addressed through pointers clamped to the row itself at the
// walls (the Neumann reflection, the same values as per-cell selects), so a
// cell costs its eight loads, the relaxation and a store.  The iteration
// space counts 32 lanes per row (row_box).
__host__ __device__ inline long long row_box(const Lvl& L) { return 32ll * L.ny * L.nz; }

__global__ void kb_smooth(const InstDev* inst, const Ctl* ctl, Tab tab, int l, int color, int vc) {
    if (vc_idle(ctl, tab.n, vc)) return;
    FOR_TILES(tab)
    if (mg_off(ctl[s], vc)) continue;
    const Lvl L = inst[s].lev[l];
    const long long rows = (long long)L.ny * L.nz;
    const long long nxy = (long long)L.nx * L.ny;
    const float inv = 1.0f / (2.0f * (L.wx + L.wy + L.wz));
    FOR_ELEMS(tab)
    const long long row = el >> 5;
    if (row >= rows) break;
    const int lane = (int)(el & 31);
    const unsigned zz = L.fny.div((unsigned)row);
    const int y = (int)((unsigned)row - zz * (unsigned)L.ny), z = (int)zz;
    AF_PTR(float) AF_RESTRICT e = view(L.e, lvl_cells(L), DK_SMOOTH, s) + ((long long)L.nx * y + nxy * z);
    AF_PTR(const float) AF_RESTRICT rr =
        view((const float*)L.r, lvl_cells(L), DK_SMOOTH, s) + ((long long)L.nx * y + nxy * z);
    AF_PTR(const float) ym = y > 0 ? e - L.nx : e;
    AF_PTR(const float) yp = y < L.ny - 1 ? e + L.nx : e;
    AF_PTR(const float) zm = z > 0 ? e - nxy : e;
    AF_PTR(const float) zp = z < L.nz - 1 ? e + nxy : e;
    const int p = ((y + z) & 1) != color ? 1 : 0;
    for (int x = p + 2 * lane; x < L.nx; x += 64) {
        const int xm = x > 0 ? x - 1 : x, xp = x < L.nx - 1 ? x + 1 : x;
        const float c = e[x];
        const float sx = e[xm] + e[xp];
        const float sy = ym[x] + yp[x];
        const float sz = zm[x] + zp[x];
        e[x] = mg_relax(L, sx, sy, sz, rr[x], inv, c);
    }
    END_ELEMS
    END_TILES
}

__device__ __forceinline__ float mg_residual(const Lvl& L, int x, int y, int z, int slot) {
    const long long nxy = (long long)L.nx * L.ny;
    const long long i = lidx(x, y, z, L.nx, L.ny);
    AF_PTR(const float) le = view((const float*)L.e, lvl_cells(L), DK_RESTRICT, slot);
    AF_PTR(const float) lr = view((const float*)L.r, lvl_cells(L), DK_RESTRICT, slot);
    const float c = le[i];
    const float sx = (x > 0 ? le[i - 1] : c) + (x < L.nx - 1 ? le[i + 1] : c);
    const float sy = (y > 0 ? le[i - L.nx] : c) + (y < L.ny - 1 ? le[i + L.nx] : c);
    const float sz = (z > 0 ? le[i - nxy] : c) + (z < L.nz - 1 ? le[i + nxy] : c);
    return mg_res(L, sx, sy, sz, c, lr[i]);
}

// Coarse rhs = mean of the children's residuals; coarse solution = 0.  One
// thread per coarse cell (row-wise forms of this kernel measured slower).
// 32 registers a thread (without spilling) let a whole SM's threads be
// resident: the finest restriction at 256^3 measured 43.5 -> 37.4 us against
// the compiler's 56 registers.  (The prolongation spills at 32 and measured
// slower at 32 and 40.)
__global__ void __launch_bounds__(1024, 2) kb_restrict(const InstDev* inst, const Ctl* ctl, Tab tab, int l, int vc) {
    if (vc_idle(ctl, tab.n, vc)) return;
    FOR_TILES(tab)
    if (mg_off(ctl[s], vc)) continue;
    const Lvl F = inst[s].lev[l];
    const Lvl C = inst[s].lev[l + 1];
    const long long n = lvl_cells(C);
    const int ex = F.cx ? 2 : 1, ey = F.cy ? 2 : 1, ez = F.cz ? 2 : 1;
    const float inv = 1.0f / (float)(ex * ey * ez);
    const bool full = ex == 2 && ey == 2 && ez == 2;
    const long long nxy = (long long)F.nx * F.ny;
    FOR_ELEMS(tab)
    if (el >= n) break;
    const unsigned e = (unsigned)el, r = C.fnx.div(e), zz = C.fny.div(r);
    const int X = (int)(e - r * (unsigned)C.nx), Y = (int)(r - zz * (unsigned)C.ny), Z = (int)zz;
    float sum = 0.0f;
    if (full) {
        // The 2x2x2 children and their 24 face neighbours, each loaded once
        // (a neighbour across a wall is the child itself); then the eight
        // residuals of mg_residual in the same order.
        const int x0 = 2 * X, y0 = 2 * Y, z0 = 2 * Z;
        AF_PTR(const float) b = view((const float*)F.e, lvl_cells(F), DK_RESTRICT, s) + lidx(x0, y0, z0, F.nx, F.ny);
        AF_PTR(const float) rb = view((const float*)F.r, lvl_cells(F), DK_RESTRICT, s) + lidx(x0, y0, z0, F.nx, F.ny);
        const long long sy = F.nx, sz = nxy;
        float E[2][2][2], R[2][2][2];
#pragma unroll
        for (int dz = 0; dz < 2; ++dz)
#pragma unroll
            for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    E[dz][dy][dx] = b[dx + dy * sy + dz * sz];
                    R[dz][dy][dx] = rb[dx + dy * sy + dz * sz];
                }
        const bool xl = x0 > 0, xh = x0 + 2 < F.nx, yl = y0 > 0, yh = y0 + 2 < F.ny, zl = z0 > 0, zh = z0 + 2 < F.nz;
#pragma unroll
        for (int dz = 0; dz < 2; ++dz)
#pragma unroll
            for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    const long long o = dx + dy * sy + dz * sz;
                    const float c = E[dz][dy][dx];
                    const float xm = dx ? E[dz][dy][0] : (xl ? b[o - 1] : c);
                    const float xp = dx ? (xh ? b[o + 1] : c) : E[dz][dy][1];
                    const float ym = dy ? E[dz][0][dx] : (yl ? b[o - sy] : c);
                    const float yp = dy ? (yh ? b[o + sy] : c) : E[dz][1][dx];
                    const float zm = dz ? E[0][dy][dx] : (zl ? b[o - sz] : c);
                    const float zp = dz ? (zh ? b[o + sz] : c) : E[1][dy][dx];
                    sum += mg_res(F, xm + xp, ym + yp, zm + zp, c, R[dz][dy][dx]);
                }
    } else {
        for (int dz = 0; dz < ez; ++dz)
            for (int dy = 0; dy < ey; ++dy)
                for (int dx = 0; dx < ex; ++dx) sum += mg_residual(F, X * ex + dx, Y * ey + dy, Z * ez + dz, s);
    }
    view(C.r, lvl_cells(C), DK_RESTRICT, s)[el] = sum * inv;
    view(C.e, lvl_cells(C), DK_RESTRICT, s)[el] = 0.0f;
    END_ELEMS
    END_TILES
}

// e_fine += cell-centred trilinear interpolation of e_coarse: per coarsened
// axis the parent weighs 3/4 and the next coarse cell toward the fine cell
// 1/4 (clamped at the walls, the Neumann reflection).  A row of 2^lg lanes
// owns one fine (y, z) row, whose four coarse rows are fixed; short rows
// (at most 16 lane iterations) share a warp two or four to a warp, so the
// per-row setup is not paid by idle lanes.  The iteration space counts 32
// lanes per warp (prolong_box).
__host__ __device__ inline int prolong_lanes_log(const Lvl& F, const Lvl& C) {
    const int w = F.cx ? C.nx : F.nx;  // lane iterations of a row
    return w > 16 ? 5 : (w > 8 ? 4 : 3);
}
// Where every axis coarsens, a work row is a coarse row (Y0, Z0) and covers
// the four fine rows (2 Y0 + {0, 1}, 2 Z0 + {0, 1}), which share the coarse
// rows Y0 - 1 .. Y0 + 1 x Z0 - 1 .. Z0 + 1: 27 coarse loads per 8 fine
// cells instead of 48.  Otherwise a work row is a fine row.
__host__ __device__ inline bool prolong_blocks(const Lvl& F) { return F.cx && F.cy && F.cz; }
__host__ __device__ inline long long prolong_rows(const Lvl& F, const Lvl& C) {
    return prolong_blocks(F) ? (long long)C.ny * C.nz : (long long)F.ny * F.nz;
}
__host__ __device__ inline long long prolong_box(const Lvl& F, const Lvl& C) {
    const int sh = 5 - prolong_lanes_log(F, C);
    return 32ll * ((prolong_rows(F, C) + (1 << sh) - 1) >> sh);
}

__global__ void kb_prolong(const InstDev* inst, const Ctl* ctl, Tab tab, int l, int vc) {
    if (vc_idle(ctl, tab.n, vc)) return;
    FOR_TILES(tab)
    if (mg_off(ctl[s], vc)) continue;
    const Lvl F = inst[s].lev[l];
    const Lvl C = inst[s].lev[l + 1];
    const long long rows = prolong_rows(F, C);
    const int lg = prolong_lanes_log(F, C), lanes = 1 << lg;
    FOR_ELEMS(tab)
    const long long row = ((el >> 5) << (5 - lg)) + ((el & 31) >> lg);
    if (row >= rows) break;
    const int lane = (int)(el & (lanes - 1));
    if (prolong_blocks(F)) {
        // Coarse rows Ym, Y0, Yp x Zm, Z0, Zp (clamped at the walls, as the
        // fine rows' neighbours are); fine row (2 Y0 + b, 2 Z0 + c) takes
        // neighbour row Yp if b else Ym, and plane Zp if c else Zm.
        const unsigned cz = C.fny.div((unsigned)row);
        const int Y0 = (int)((unsigned)row - cz * (unsigned)C.ny), Z0 = (int)cz;
        const int Ys[3] = {max(Y0 - 1, 0), Y0, min(Y0 + 1, C.ny - 1)};
        const int Zs[3] = {max(Z0 - 1, 0), Z0, min(Z0 + 1, C.nz - 1)};
        AF_PTR(const float) ce = view((const float*)C.e, lvl_cells(C), DK_PROLONG, s);
        AF_PTR(float) fe = view(F.e, lvl_cells(F), DK_PROLONG, s);
        int co[3][3];  // coarse row offsets [z][y]
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) co[a][b] = (int)lidx(0, Ys[b], Zs[a], C.nx, C.ny);
        int fo[2][2];  // fine row offsets [c][b]
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int b = 0; b < 2; ++b) fo[c][b] = (int)lidx(0, 2 * Y0 + b, 2 * Z0 + c, F.nx, F.ny);
        for (int X = lane; X < C.nx; X += lanes) {
            const int Xm = max(X - 1, 0), Xp = min(X + 1, C.nx - 1);
            float a0[3][3], am[3][3], ap[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    a0[a][b] = ce[co[a][b] + X];
                    am[a][b] = ce[co[a][b] + Xm];
                    ap[a][b] = ce[co[a][b] + Xp];
                }
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    const int y1 = b ? 2 : 0, z1 = c ? 2 : 0;  // the neighbour row and plane
                    float2 f = AF_VEC(float2, fe, fo[c][b] + 2 * X, 2);
                    f.x = __fadd_rn(f.x, mg_interp(0.75f, 0.75f, 0.75f, a0[1][1], am[1][1], a0[1][y1], am[1][y1],
                                                   a0[z1][1], am[z1][1], a0[z1][y1], am[z1][y1]));
                    f.y = __fadd_rn(f.y, mg_interp(0.75f, 0.75f, 0.75f, a0[1][1], ap[1][1], a0[1][y1], ap[1][y1],
                                                   a0[z1][1], ap[z1][1], a0[z1][y1], ap[z1][y1]));
                    AF_VEC(float2, fe, fo[c][b] + 2 * X, 2) = f;
                }
        }
        continue;
    }
    const unsigned zz = F.fny.div((unsigned)row);
    const int y = (int)((unsigned)row - zz * (unsigned)F.ny), z = (int)zz;
    int Y0 = y, Y1 = y, Z0 = z, Z1 = z;
    float ay = 1.0f, az = 1.0f;
    if (F.cy) { Y0 = y >> 1; Y1 = min(max(Y0 + ((y & 1) ? 1 : -1), 0), C.ny - 1); ay = 0.75f; }
    if (F.cz) { Z0 = z >> 1; Z1 = min(max(Z0 + ((z & 1) ? 1 : -1), 0), C.nz - 1); az = 0.75f; }
    AF_PTR(const float) ce = view((const float*)C.e, lvl_cells(C), DK_PROLONG, s);
    AF_PTR(const float) c00 = ce + lidx(0, Y0, Z0, C.nx, C.ny);
    AF_PTR(const float) c10 = ce + lidx(0, Y1, Z0, C.nx, C.ny);
    AF_PTR(const float) c01 = ce + lidx(0, Y0, Z1, C.nx, C.ny);
    AF_PTR(const float) c11 = ce + lidx(0, Y1, Z1, C.nx, C.ny);
    AF_PTR(float) fe = view(F.e, lvl_cells(F), DK_PROLONG, s) + lidx(0, y, z, F.nx, F.ny);
    if (F.cx) {
        // A lane owns the fine pair (2X, 2X+1): both take parent X, the even
        // one neighbour X-1 and the odd one X+1 (clamped at the walls), so
        // the pair shares its coarse loads and one 8-byte access of e (nx is
        // even and every row starts on an even element).
        for (int X = lane; X < C.nx; X += lanes) {
            const int Xm = max(X - 1, 0), Xp = min(X + 1, C.nx - 1);
            const float a00 = c00[X], a10 = c10[X], a01 = c01[X], a11 = c11[X];
            float2 f = AF_VEC(float2, fe, 2 * X, 2);
            f.x = __fadd_rn(f.x, mg_interp(0.75f, ay, az, a00, c00[Xm], a10, c10[Xm], a01, c01[Xm], a11, c11[Xm]));
            f.y = __fadd_rn(f.y, mg_interp(0.75f, ay, az, a00, c00[Xp], a10, c10[Xp], a01, c01[Xp], a11, c11[Xp]));
            AF_VEC(float2, fe, 2 * X, 2) = f;
        }
    } else {
        for (int x = lane; x < F.nx; x += lanes)
            fe[x] = __fadd_rn(fe[x], mg_interp(1.0f, ay, az, c00[x], c00[x], c10[x], c10[x], c01[x], c01[x], c11[x],
                                               c11[x]));
    }
    END_ELEMS
    END_TILES
}

__device__ float block_sum(float v, float* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = threadIdx.x < kCoarseThreads / 32 ? red[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) red[0] = s;
    }
    __syncthreads();
    const float s = red[0];
    __syncthreads();
    return s;
}

// --- fused red-black pair ---------------------------------------------------
// One red sweep then one black sweep of L e = r, from e_in into e_out.  The
// red values read only e_in (their black neighbours are unchanged by the red
// sweep); the black values read the new red values.  Each block owns an
// output tile of TX x TY x TZ cells.  It first computes the new
// red values of the tile plus a one-cell halo -- only the red cells, kept
// compactly in shared memory (a row of the halo alternates colours, so
// x >> 1 indexes its red cells) -- then, after one barrier, each lane writes
// an adjacent (x, x+1) pair of the tile, one red cell (from shared memory)
// and one black cell (from its red neighbours there), so lanes never diverge
// on colour.  Nothing reads what the kernel writes, so blocks never race, and
// the result equals the two in-place colour sweeps bit for bit (mg_relax in
// both).  Per pair it moves e and r once and writes e once.
//
// Wide tiles (LANES = 32, TX = 64, a warp per row) cover x < nxw; a level
// whose x extent leaves 1..32 cells past the last wide tile (nx = 32, 96,
// ...) covers them with one narrow tile column (LANES = 16, TX = 32, a warp
// per two rows) instead of a half-idle wide tile.
//
// Three tile variants trade the red halo's recomputation (1.45x the tile's
// red cells at 16 x 8 rows and planes, 1.9x at 8 x 4, 2.3x at 4 x 4) against
// parallelism: a 64^3 level holds 32 of the largest tiles for 152 SMs.  The
// autotuner picks a variant per level; untuned, the level's size does.
// Variant 3 is the TMA-staged z-marching pair (kb_smooth_pair_zm): 64 x 16
// columns of 16 planes.
// Variant 4: 64 x 16 x 16 tiles, the red halo recomputed over 1.27x the
// tile's red cells.
constexpr int kPairVarTY[5] = {16, 8, 4, 16, 16}, kPairVarTZ[5] = {8, 4, 4, 16, 16};
constexpr int kPairWideX = 64;

template <int LANES, int V>
struct PairTile {
    static constexpr int TY = kPairVarTY[V];
    static constexpr int TZ = kPairVarTZ[V];
    static constexpr int FY = V == 4 ? 0 : V;  // Lvl::fty entry of TY
    static constexpr int HY = TY + 2, HZ = TZ + 2;
    static constexpr int TX = 2 * LANES;        // cells along x
    static constexpr int RX = LANES + 1;        // red cells of a halo row
    static constexpr int RPW = 32 / LANES;      // tile rows per warp
    static constexpr int THREADS = TY * LANES;
    // Resident threads per SM the launch bounds ask for: all 2048 for the
    // largest tiles (32 registers suffice), 1536 for the others (their
    // index arithmetic would spill at 32).
    static constexpr int RESIDENT = V == 0 || V == 4 ? 2048 : 1536;
};

template <int LANES, int V>
__global__ void __launch_bounds__(PairTile<LANES, V>::THREADS, PairTile<LANES, V>::RESIDENT / PairTile<LANES, V>::THREADS)
    kb_smooth_pair(const InstDev* inst, const Ctl* ctl, Tab tab, int l, int dir, int vc) {
    if (vc_idle(ctl, tab.n, vc)) return;
    using T = PairTile<LANES, V>;
    __shared__ float red[T::HZ][T::HY][T::RX];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k = lane % LANES;                        // pair of the row
    const int wrow = warp * T::RPW + lane / LANES;     // tile row, 0 .. TY-1
    for (int item = blockIdx.x, total = tab.prefix[tab.n]; item < total; item += gridDim.x) {
        const int s = find_slot(tab.prefix, tab.n, item);
        if (mg_off(ctl[s], vc)) continue;
        const Lvl L = inst[s].lev[l];
        AF_PTR(const float) AF_RESTRICT ein = view((const float*)(dir ? L.e2 : L.e), lvl_cells(L), DK_PAIR, s);
        AF_PTR(float) AF_RESTRICT eout = view(dir ? L.e : L.e2, lvl_cells(L), DK_PAIR, s);
        AF_PTR(const float) AF_RESTRICT r = view((const float*)L.r, lvl_cells(L), DK_PAIR, s);
        const int nx = L.nx, ny = L.ny, nz = L.nz, nxy = nx * ny;  // a level holds < 2^31 cells
        const unsigned local = (unsigned)(item - tab.prefix[s]);
        int x0, y0, z0;
        if (LANES == 32) {
            const unsigned q1 = L.ftx.div(local), q2 = L.fty[T::FY].div(q1);
            x0 = (int)(local - q1 * L.ftx.d) * T::TX;
            y0 = (int)(q1 - q2 * L.fty[T::FY].d) * T::TY;
            z0 = (int)q2 * T::TZ;
        } else {
            const unsigned q2 = L.fty[T::FY].div(local);
            x0 = L.nxw;
            y0 = (int)(local - q2 * L.fty[T::FY].d) * T::TY;
            z0 = (int)q2 * T::TZ;
        }
        const float inv = 1.0f / (2.0f * (L.wx + L.wy + L.wz));
        // Red cells of the halo tile, a row of lanes per halo row (hy, hz):
        // halo x = x0 - 1 + hx, hx = 2j + ((y + z + 1) & 1); lanes take
        // j < LANES and the rows' last cells (j = LANES) go one per thread
        // afterwards.
        auto red_row = [&](int hy, int hz, int j) {
            const int y = y0 - 1 + hy, z = z0 - 1 + hz;
            const int x = x0 - 1 + 2 * j + ((y + z + 1) & 1);
            float v = 0.0f;
            if ((unsigned)x < (unsigned)nx && (unsigned)y < (unsigned)ny && (unsigned)z < (unsigned)nz) {
                const int i = x + nx * y + nxy * z;
                const int oym = y > 0 ? -nx : 0, oyp = y < ny - 1 ? nx : 0;
                const int ozm = z > 0 ? -nxy : 0, ozp = z < nz - 1 ? nxy : 0;
                const int oxm = x > 0 ? -1 : 0, oxp = x < nx - 1 ? 1 : 0;
                AF_PTR(const float) p = ein + i;
                v = mg_relax(L, p[oxm] + p[oxp], p[oym] + p[oyp], p[ozm] + p[ozp], r[i], inv, p[0]);
            }
            red[hz][hy][j] = v;
        };
        for (int row = wrow; row < T::HY * T::HZ; row += T::TY) red_row(row % T::HY, row / T::HY, k);
        for (int row = tid; row < T::HY * T::HZ; row += T::THREADS)
            red_row(row % T::HY, row / T::HY, LANES);
        __syncthreads();
        // Output pairs: lane k -> x = x0 + 2k + {0, 1}, tile row -> y, loop over z.
        const int y = y0 + wrow, hy = wrow + 1;
        const int xa = x0 + 2 * k;
        if (y < ny && xa < nx) {
            const int zend = min(T::TZ, nz - z0);
            int i0 = xa + nx * y + nxy * z0;
            for (int tz = 0; tz < zend; ++tz, i0 += nxy) {
                const int z = z0 + tz, hz = tz + 1;
                // Of the pair, the red cell is xa + pr and the black one xa + 1 - pr.
                const int pr = (xa + y + z) & 1;
                const int xr = xa + pr, xb = xa + 1 - pr;
                if (xr < nx) eout[i0 + pr] = red[hz][hy][(xr - x0 + 1) >> 1];
                if (xb < nx) {
                    const int h = (xb - x0 + 1) >> 1, hm = (xb - x0) >> 1, hp = (xb - x0 + 2) >> 1;
                    const int ib = i0 + 1 - pr;
                    const float c = ein[ib];
                    const float sx = (xb > 0 ? red[hz][hy][hm] : c) + (xb < nx - 1 ? red[hz][hy][hp] : c);
                    const float sy = (y > 0 ? red[hz][hy - 1][h] : c) + (y < ny - 1 ? red[hz][hy + 1][h] : c);
                    const float sz = (z > 0 ? red[hz - 1][hy][h] : c) + (z < nz - 1 ? red[hz + 1][hy][h] : c);
                    eout[ib] = mg_relax(L, sx, sy, sz, r[ib], inv, c);
                }
            }
        }
        __syncthreads();
    }
}

// --- TMA-staged, z-marching fused pair -----------------------------------------
// The red-black pair of kb_smooth_pair on 64 x 16 columns of ZC planes,
// marching along z with its inputs in shared-memory rings filled by TMA
// plane loads (e_in planes of the column plus a two-cell ring, r planes plus
// a one-cell ring).  Step k computes the red cells of halo plane z0-1+k (the
// tile's rows plus one on each side) into a ring of red planes, then the
// black cells of plane z0-2+k from the three red planes around it.  The red
// halo is recomputed only across the column's sides and the chunk's two end
// planes (1.3x the tile's red cells at ZC = 16), not around every 3-D tile.
//
// Walls cost no per-cell work.  The e ring holds, for the planes z0-2+p, the
// plane clamped into the level (the plane beyond a z wall is the wall plane
// loaded again), and once a plane lands, the cells just beyond an x or y wall
// are overwritten with the wall cell they face.  So every neighbour of an
// in-level red cell is read at a fixed offset and is exactly the value
// kb_smooth_pair uses (at a wall: the cell's own).  A red position just
// outside the level takes the old value stored there, i.e. the wall cell it
// faces, which is the value the black cell beside it uses for its wall
// neighbour: the black pass needs no selects either.  Arithmetic and operand
// order are those of kb_smooth_pair: the same bits.
//
// Every thread keeps its rows for the whole column: warp w of 18 computes
// the red cells of halo row w (warp 16 also the rows' 33rd cells) and warps
// 0-15 the black cells of tile row w.  Plane loads run five steps ahead; a
// plane's loads are waited one step before it is first read, so its wall
// fix-up is published by the step's one block barrier.
//
// A level runs it only when its rows and arrays are 16-byte aligned (nx a
// multiple of 4; InstDev::pmap, Lvl::tma).  Boxes start at x0 - 4, a 16-byte
// boundary; box cells outside the level load as zeros and are never read.
constexpr int kZmTX = 64, kZmTY = 16, kZmZC = 16, kZmBX = 72;
static_assert(kPairVarTY[3] == kZmTY && kPairVarTZ[3] == kZmZC, "work-list tiles of pair variant 3");
constexpr int kZmEY = kZmTY + 4, kZmRY = kZmTY + 2;     // e rows: tile + 2 each side; r and red rows: + 1
constexpr int kZmNE = 8, kZmNR = 8, kZmNRed = 4, kZmLead = 5, kZmNB = 8;
constexpr int kZmEBox = kZmBX * kZmEY, kZmRBox = kZmBX * kZmRY;  // floats one plane load delivers
// Ring slots of e and r planes start on 128-byte boundaries (the rule for a
// TMA tensor load's shared-memory destination): plane pitches round up to 32 floats.
constexpr int kZmEPlane = (kZmEBox + 31) / 32 * 32, kZmRPlane = (kZmRBox + 31) / 32 * 32;
constexpr int kZmRedPlane = kZmRY * 33;
constexpr int kZmROff = kZmNE * kZmEPlane, kZmRedOff = kZmROff + kZmNR * kZmRPlane;  // ring offsets (floats)
constexpr int kZmFloats = kZmRedOff + kZmNRed * kZmRedPlane;
// 18 warps: warp w computes red halo row w, warps 0-15 also the black cells
// of tile row w and warp 16 the rows' 33rd red cells, so no warp does more
// than two row passes between the march's barriers.  Two blocks per SM keep
// every per-thread offset of the column in registers (with fewer, the
// compiler re-derives them from the thread index at every step).
constexpr int kZmWarps = kZmRY;
constexpr int kZmThreads = kZmWarps * 32;
constexpr int kZmBlocks = 2;
constexpr size_t kZmSmem = (size_t)kZmFloats * sizeof(float);
// Ring sizes for a lead of kZmLead groups with each group waited one step
// before its first read (a slot is rewritten only after its last reader).
static_assert(kZmNE >= kZmLead + 3 && kZmNR >= kZmLead + 2 && kZmNB > kZmLead, "ring sizes of the z-march");
// The march is unrolled by 8 steps, so every ring slot, red plane and
// barrier of a step is a compile-time constant.
static_assert(kZmNE == 8 && kZmNR == 8 && kZmNB == 8 && kZmNRed == 4, "ring sizes of the unrolled march");
static_assert(kZmEPlane % 32 == 0 && kZmRPlane % 32 == 0 && kZmROff % 32 == 0,
              "TMA destinations of the z-march rings on 128-byte boundaries");

// Shared-memory access of the z-march: byte addresses with compile-time
// offsets ([addr + imm]), so a neighbour costs no address arithmetic.  The
// bounds-checking build indexes the checked ring view instead.
#if AEROFLUX_DEBUG_BOUNDS
using ZmAddr = int;  // float index into the rings
#define ZM_A(i) (i)
#define ZM_LD(a, off) S[(a) + (off)]
#define ZM_ST(a, v) (S[(a)] = (v))
constexpr int kZmB = 1;  // address units per float
#else
using ZmAddr = unsigned;  // shared-window byte address
template <int OFF>
__device__ __forceinline__ float zm_lds(unsigned a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1+%2];" : "=f"(v) : "r"(a), "n"(OFF) : "memory");
    return v;
}
__device__ __forceinline__ void zm_sts(unsigned a, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
#define ZM_A(i) (sb + 4u * (unsigned)(i))
#define ZM_LD(a, off) zm_lds<4 * (off)>(a)
#define ZM_ST(a, v) zm_sts((a), (v))
constexpr int kZmB = 4;
#endif

template <int ZC>
__global__ void __launch_bounds__(kZmThreads, kZmBlocks)
    kb_smooth_pair_zm(const InstDev* inst, const Ctl* ctl, Tab tab, int l, int dir, int vc, unsigned* diag) {
    if (vc_idle(ctl, tab.n, vc)) return;
    extern __shared__ __align__(128) float zsm[];
    __shared__ __align__(8) unsigned long long bar[kZmNB];
    __shared__ unsigned stop;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned sb = smem_addr(zsm);
    if (sb & 127u) {  // the rings' TMA destinations need a 128-byte aligned base
        if (tid == 0) atomicOr(diag, 4u);
        return;
    }
    if (tid == 0) {
        for (int i = 0; i < kZmNB; ++i) mbar_init(&bar[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        stop = diag_set(diag) ? 1u : 0u;
    }
    __syncthreads();
    if (stop) return;
    // Group k of a column completes on barrier k % 8; bit b of `phase` is
    // the parity barrier b completes next (every thread waits every group).
    unsigned phase = 0;
    for (int item = blockIdx.x, total = tab.prefix[tab.n]; item < total; item += gridDim.x) {
        const int s = find_slot(tab.prefix, tab.n, item);
        if (mg_off(ctl[s], vc)) continue;
        const Lvl L = inst[s].lev[l];
        if (!L.tma) {  // the host switches the stage off this variant first; never stage through an unset map
            if (tid == 0) atomicOr(diag, 2u);
            continue;
        }
        AF_PTR(float) S = view(zsm, (long long)kZmFloats, DK_PAIR, s);  // the three rings
        (void)S;
        AF_PTR(float) AF_RESTRICT eout = view(dir ? L.e : L.e2, lvl_cells(L), DK_PAIR, s);
        const int nx = L.nx, ny = L.ny, nz = L.nz;
        const unsigned local = (unsigned)(item - tab.prefix[s]);
        const unsigned q1 = L.ftx.div(local), q2 = L.fty[0].div(q1);
        const int x0 = (int)(local - q1 * L.ftx.d) * kZmTX;
        const int y0 = (int)(q1 - q2 * L.fty[0].d) * kZmTY;
        const int z0 = (int)q2 * ZC;
        const int K = min(ZC, nz - z0);  // black planes z0 .. z0+K-1; steps 0 .. K+1
        // Group k: e plane z0+k into ring plane p = k+2 and r plane z0-1+k
        // into r slot k % kZmNR, when needed; group 0 also brings ring
        // planes 0 and 1 (z0-2, z0-1).  A plane just beyond a z wall loads
        // the wall plane; one further out is never read and not loaded.
        auto issue = [&](int k) {
            unsigned long long* b = &bar[k & 7];
            const int pa = k == 0 ? 0 : k + 2, pb = k + 2;
            int ne = 0;
            for (int p = pa; p <= pb; ++p) ne += (z0 - 2 + p >= -1 && z0 - 2 + p <= nz) ? 1 : 0;
            const int rz = z0 - 1 + k;
            const bool rr = rz >= 0 && rz < nz;
            mbar_expect_tx(b, (unsigned)((ne * kZmEBox + (rr ? kZmRBox : 0)) * sizeof(float)));
            const CUtensorMap* em = inst[s].pmap + 3 * l + dir;
            for (int p = pa; p <= pb; ++p) {
                const int z = z0 - 2 + p;
                if (z >= -1 && z <= nz)
                    tma_load_3d(zsm + (p & 7) * kZmEPlane, em, x0 - 4, y0 - 2, min(max(z, 0), nz - 1), b);
            }
            if (rr) tma_load_3d(zsm + kZmROff + (k & 7) * kZmRPlane, inst[s].pmap + 3 * l + 2, x0 - 4, y0 - 1, rz, b);
        };
        // Wall fix-up of a landed e plane: the cell beyond an x or y wall
        // takes the wall cell's value (box column 4 is x = x0, box row 2 is
        // y = y0).  Only cells beside an in-level cell matter; the corners
        // two walls share are never read.
        const int wx0 = x0 == 0, wx1 = x0 + kZmTX >= nx, wy0 = y0 == 0, wy1 = y0 + kZmRY - 1 >= ny;
        const bool walls = wx0 | wx1 | wy0 | wy1;
        const int gx = nx - x0 + 4, gy = ny - y0 + 2;  // box column of x = nx, box row of y = ny
        auto fill = [&](int slot) {
            const int P = slot * kZmEPlane;
            if (tid < kZmEY) {
                const ZmAddr r = ZM_A(P + tid * kZmBX);
                if (wx0) ZM_ST(r + 3 * kZmB, ZM_LD(r, 4));
                if (wx1) ZM_ST(r + gx * kZmB, ZM_LD(r + (gx - 1) * kZmB, 0));
            } else if (tid >= 32 && tid < 32 + kZmBX) {
                const ZmAddr c = ZM_A(P + tid - 32);
                if (wy0) ZM_ST(c + kZmBX * kZmB, ZM_LD(c, 2 * kZmBX));
                if (wy1) ZM_ST(c + gy * kZmBX * kZmB, ZM_LD(c + (gy - 1) * kZmBX * kZmB, 0));
            }
        };
        const float inv = 1.0f / (2.0f * (L.wx + L.wy + L.wz));
        // Red cells of this thread: cell `lane` of halo row `warp`, and for
        // warp 16 also cell 32 of halo row lane % 18 (lanes 18-31 repeat
        // lanes 0-13: the same value to the same place).  Per cell: e offset
        // for parity 0, red offset, level row + 1, level x for parity 0.
        const bool xe = warp == kZmTY;
        const int hyB = lane % kZmRY, jB = 32;
        const int eA = (warp + 1) * kZmBX + 3 + 2 * lane, eB = (hyB + 1) * kZmBX + 3 + 2 * jB;
        const int dA = warp * 33 + lane, dB = hyB * 33 + jB;
        const int yA = y0 + warp, yB = y0 + hyB;  // level row + 1
        const int xA = x0 - 1 + 2 * lane, xB = x0 - 1 + 2 * jB;
        // Black cells of this thread (warps 0-15): tile row `warp`, pair
        // x0 + 2 lane, +1; computed by every lane, stored where in the level.
        const bool bw = warp < kZmTY;
        const int by = y0 + warp;
        const bool bok = by < ny && x0 + 2 * lane < nx;
        const int ebk = (warp + 2) * kZmBX + 2 * lane + 5;  // e offset of the black cell when the pair starts red
        const int rbk = (warp + 1) * 33 + lane;              // red offset of cell lane in halo row warp+1
        const long long nxy = (long long)nx * ny;
        AF_PTR(float) gp = eout + ((long long)(x0 + 2 * lane) + (long long)nx * by + nxy * z0);
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            for (int k = 0; k < kZmLead && k <= K + 1; ++k) issue(k);
        }
        bool failed = !mbar_wait_bounded(&bar[0], phase & 1u);
        if (!failed) phase ^= 1u;
        if (walls && !failed) {
            fill(0);
            fill(1);
            fill(2);
        }
        if (__syncthreads_or(failed ? 1 : 0)) {
            if (tid == 0) {
                atomicOr(diag, 1u);
                for (int j = 0; j < kZmLead && j <= K + 1; ++j) mbar_wait_bounded(&bar[j], (phase >> j) & 1u);
            }
            __syncthreads();
            return;
        }
        // Step k (k = kb + J, J the compile-time step within a block of 8):
        // e ring slots of planes k .. k+3 are J .. J+3 (mod 8), r slots of
        // planes z0-1+k and z0-2+k are J and J-1, the red plane is J & 3 and
        // group k+1's barrier is J+1.
        auto step = [&](auto Jc, int kb) -> bool {  // false: a wait gave up (the block has returned its transfers)
            constexpr int J = decltype(Jc)::value;
            constexpr int s0 = J & 7, s1 = (J + 1) & 7, s2 = (J + 2) & 7, s3 = (J + 3) & 7;
            constexpr int sr = J & 7, srp = (J + 7) & 7, b1 = (J + 1) & 7;
            const int k = kb + J;
            if (k + 1 <= K + 1) {  // group k+1, first read at step k+1
                if (!failed) {
                    if (mbar_wait_bounded(&bar[b1], (phase >> b1) & 1u)) phase ^= 1u << b1;
                    else failed = true;
                }
                if (walls && !failed) fill(s3);
            }
            const int zr = z0 - 1 + k;
            const bool zin = (unsigned)zr < (unsigned)nz;
            const ZmAddr ec = ZM_A(s1 * kZmEPlane);
            constexpr int dzm = (s0 - s1) * kZmEPlane * kZmB, dzp = (s2 - s1) * kZmEPlane * kZmB;
            constexpr int drr = (kZmROff + sr * kZmRPlane - s1 * kZmEPlane - kZmBX) * kZmB;
            const ZmAddr rs = ZM_A(kZmRedOff + (J & 3) * kZmRedPlane);
            if (!failed) {
                auto red_cell = [&](int e0, int d0, int y1, int x) {
                    const int par = (y1 + zr) & 1;
                    const ZmAddr a = ec + (e0 + par) * kZmB;
                    const bool in = zin && (unsigned)(y1 - 1) < (unsigned)ny && (unsigned)(x + par) < (unsigned)nx;
                    const float c = ZM_LD(a, 0);
                    const float v = mg_relax(L, ZM_LD(a, -1) + ZM_LD(a, 1), ZM_LD(a, -kZmBX) + ZM_LD(a, kZmBX),
                                             ZM_LD(a + (ZmAddr)dzm, 0) + ZM_LD(a + (ZmAddr)dzp, 0), ZM_LD(a + (ZmAddr)drr, 0), inv, c);
                    ZM_ST(rs + d0 * kZmB, in ? v : c);
                };
                red_cell(eA, dA, yA, xA);
                if (xe) red_cell(eB, dB, yB, xB);
            }
            if (__syncthreads_or(failed ? 1 : 0)) {
                if (tid == 0) {
                    atomicOr(diag, 1u);
                    for (int j = k + 1; j <= k + kZmLead - 1 && j <= K + 1; ++j)  // groups issued, not yet waited
                        mbar_wait_bounded(&bar[j & 7], (phase >> (j & 7)) & 1u);
                }
                __syncthreads();
                return false;
            }
            if (tid == 0 && k + kZmLead <= K + 1) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(k + kZmLead);
            }
            if (k >= 2 && bw) {
                // Black cells of plane zr - 1: e ring plane k, r plane k-1,
                // red planes k-2, k-1, k.
                const int pr = (by + zr - 1) & 1;
                const ZmAddr eb = ZM_A(s0 * kZmEPlane + ebk - pr);
                const float c = ZM_LD(eb, 0);
                constexpr int drv = (kZmROff + srp * kZmRPlane - s0 * kZmEPlane - kZmBX) * kZmB;
                const float rv = ZM_LD(eb + (ZmAddr)drv, 0);
                const ZmAddr r1 = ZM_A(kZmRedOff + ((J + 3) & 3) * kZmRedPlane + rbk);
                const ZmAddr h1 = r1 + (1 - pr) * kZmB;
                constexpr int dz0 = (((J + 2) & 3) - ((J + 3) & 3)) * kZmRedPlane * kZmB;
                constexpr int dz2 = ((J & 3) - ((J + 3) & 3)) * kZmRedPlane * kZmB;
                const float sx = ZM_LD(r1, 0) + ZM_LD(r1, 1);
                const float sy = ZM_LD(h1, -33) + ZM_LD(h1, 33);
                const float sz = ZM_LD(h1 + (ZmAddr)dz0, 0) + ZM_LD(h1 + (ZmAddr)dz2, 0);
                const float bv = mg_relax(L, sx, sy, sz, rv, inv, c);
                const float red_v = ZM_LD(r1 + pr * kZmB, 0);
                if (bok) AF_VEC(float2, gp, 0, 2) = pr ? make_float2(bv, red_v) : make_float2(red_v, bv);
            }
            if (k >= 2) gp += nxy;
            return true;
        };
        bool ok = true;
        for (int kb = 0; ok && kb <= K + 1; kb += 8) {
            ok = step(std::integral_constant<int, 0>{}, kb);
            if (ok && kb + 1 <= K + 1) ok = step(std::integral_constant<int, 1>{}, kb);
            if (ok && kb + 2 <= K + 1) ok = step(std::integral_constant<int, 2>{}, kb);
            if (ok && kb + 3 <= K + 1) ok = step(std::integral_constant<int, 3>{}, kb);
            if (ok && kb + 4 <= K + 1) ok = step(std::integral_constant<int, 4>{}, kb);
            if (ok && kb + 5 <= K + 1) ok = step(std::integral_constant<int, 5>{}, kb);
            if (ok && kb + 6 <= K + 1) ok = step(std::integral_constant<int, 6>{}, kb);
            if (ok && kb + 7 <= K + 1) ok = step(std::integral_constant<int, 7>{}, kb);
        }
        if (!ok) return;
        __syncthreads();  // every thread is done with the rings before the next column's loads
    }
}
#undef ZM_A
#undef ZM_LD
#undef ZM_ST

// --- tail V-cycle: every level from the slot's tail down, in one block -------
// Levels of at most kCoarseMax cells live in shared memory: pre-smoothing and
// restriction down to the coarsest level, its solve (the mean of r removed --
// a Neumann problem is solvable only for zero-mean data -- red-black sweeps
// from zero, the mean of e removed), then prolongation and post-smoothing
// back up.  Sums use a fixed tree.  Replaces one launch per level and sweep.
// One colour: the threads walk that colour's cells only, (nx+1)/2 slots per
// (y, z) row (the last one past the row when the row's colour count is
// smaller), so a sweep costs half the index decoding of a walk over all cells.
__device__ void sm_smooth(const Lvl& L, AF_PTR(float) e, AF_PTR(const float) r, int color) {
    const int hx = (L.nx + 1) / 2, m = hx * L.ny * L.nz, nxy = L.nx * L.ny;
    const float inv = 1.0f / (2.0f * (L.wx + L.wy + L.wz));
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        const unsigned q = L.fhx.div((unsigned)j), zz = L.fny.div(q);
        const int y = (int)q - (int)zz * L.ny, z = (int)zz;
        const int x = (((y + z) & 1) != color ? 1 : 0) + 2 * (j - (int)q * hx);
        if (x >= L.nx) continue;
        const int i = x + L.nx * (int)q;
        const float c = e[i];
        const float sx = (x > 0 ? e[i - 1] : c) + (x < L.nx - 1 ? e[i + 1] : c);
        const float sy = (y > 0 ? e[i - L.nx] : c) + (y < L.ny - 1 ? e[i + L.nx] : c);
        const float sz = (z > 0 ? e[i - nxy] : c) + (z < L.nz - 1 ? e[i + nxy] : c);
        e[i] = mg_relax(L, sx, sy, sz, r[i], inv, c);
    }
    __syncthreads();
}

__device__ __forceinline__ float sm_res(const Lvl& L, AF_PTR(const float) e, AF_PTR(const float) r, int x, int y,
                                        int z) {
    const int nxy = L.nx * L.ny;
    const int i = x + L.nx * y + nxy * z;
    const float c = e[i];
    const float sx = (x > 0 ? e[i - 1] : c) + (x < L.nx - 1 ? e[i + 1] : c);
    const float sy = (y > 0 ? e[i - L.nx] : c) + (y < L.ny - 1 ? e[i + L.nx] : c);
    const float sz = (z > 0 ? e[i - nxy] : c) + (z < L.nz - 1 ? e[i + nxy] : c);
    return mg_res(L, sx, sy, sz, c, r[i]);
}

__global__ void __launch_bounds__(kCoarseThreads) kb_vtail(const InstDev* inst, const Ctl* ctl, Tab tab, int nu,
                                                           int vc) {
    if (vc_idle(ctl, tab.n, vc)) return;
    extern __shared__ float tsm[];
    __shared__ float red[32];
    for (int item = blockIdx.x, total = tab.prefix[tab.n]; item < total; item += gridDim.x) {
        const int s = find_slot(tab.prefix, tab.n, item);
        if (mg_off(ctl[s], vc)) continue;
        const InstDev& I = inst[s];
        const int t = I.tail, nl = I.nlev;
        AF_PTR(float) E[kMaxLev];
        AF_PTR(float) R[kMaxLev];
        {
            float* p = tsm;
            for (int l = t; l < nl; ++l) {
                const int n = lvl_cells(I.lev[l]);
                E[l] = view(p, (long long)n, DK_VTAIL, s);
                R[l] = view(p + n, (long long)n, DK_VTAIL, s);
                p += 2 * n;
            }
        }
        const Lvl T = I.lev[t];
        AF_PTR(float) te = view(T.e, lvl_cells(T), DK_VTAIL, s);
        AF_PTR(const float) tr = view((const float*)T.r, lvl_cells(T), DK_VTAIL, s);
        for (int i = threadIdx.x; i < lvl_cells(T); i += blockDim.x) {
            E[t][i] = te[i];
            R[t][i] = tr[i];
        }
        __syncthreads();
        for (int l = t; l + 1 < nl; ++l) {
            const Lvl F = I.lev[l], C = I.lev[l + 1];
            for (int k = 0; k < nu; ++k) {
                sm_smooth(F, E[l], R[l], 0);
                sm_smooth(F, E[l], R[l], 1);
            }
            const int ex = F.cx ? 2 : 1, ey = F.cy ? 2 : 1, ez = F.cz ? 2 : 1;
            const float inv = 1.0f / (float)(ex * ey * ez);
            for (int j = threadIdx.x; j < lvl_cells(C); j += blockDim.x) {
                const unsigned q = C.fnx.div((unsigned)j), zz = C.fny.div(q);
                const int X = j - (int)q * C.nx, Y = (int)q - (int)zz * C.ny, Z = (int)zz;
                float sum = 0.0f;
                for (int dz = 0; dz < ez; ++dz)
                    for (int dy = 0; dy < ey; ++dy)
                        for (int dx = 0; dx < ex; ++dx) sum += sm_res(F, E[l], R[l], X * ex + dx, Y * ey + dy, Z * ez + dz);
                R[l + 1][j] = sum * inv;
                E[l + 1][j] = 0.0f;
            }
            __syncthreads();
        }
        {  // coarsest solve
            const Lvl C = I.lev[nl - 1];
            const int n = lvl_cells(C);
            float part = 0.0f;
            for (int i = threadIdx.x; i < n; i += blockDim.x) part += R[nl - 1][i];
            const float mean_r = block_sum(part, red) / (float)n;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                R[nl - 1][i] -= mean_r;
                E[nl - 1][i] = 0.0f;
            }
            __syncthreads();
            for (int k = 0; k < I.coarse_sweeps; ++k) {
                sm_smooth(C, E[nl - 1], R[nl - 1], 0);
                sm_smooth(C, E[nl - 1], R[nl - 1], 1);
            }
            part = 0.0f;
            for (int i = threadIdx.x; i < n; i += blockDim.x) part += E[nl - 1][i];
            const float mean_e = block_sum(part, red) / (float)n;
            for (int i = threadIdx.x; i < n; i += blockDim.x) E[nl - 1][i] -= mean_e;
            __syncthreads();
        }
        for (int l = nl - 2; l >= t; --l) {
            const Lvl F = I.lev[l], C = I.lev[l + 1];
            for (int i = threadIdx.x; i < lvl_cells(F); i += blockDim.x) {
                const unsigned q = F.fnx.div((unsigned)i), zz = F.fny.div(q);
                const int x = i - (int)q * F.nx, y = (int)q - (int)zz * F.ny, z = (int)zz;
                int X0 = x, X1 = x, Y0 = y, Y1 = y, Z0 = z, Z1 = z;
                float ax = 1.0f, ay = 1.0f, az = 1.0f;
                if (F.cx) { X0 = x >> 1; X1 = min(max(X0 + ((x & 1) ? 1 : -1), 0), C.nx - 1); ax = 0.75f; }
                if (F.cy) { Y0 = y >> 1; Y1 = min(max(Y0 + ((y & 1) ? 1 : -1), 0), C.ny - 1); ay = 0.75f; }
                if (F.cz) { Z0 = z >> 1; Z1 = min(max(Z0 + ((z & 1) ? 1 : -1), 0), C.nz - 1); az = 0.75f; }
                AF_PTR(const float) ec = E[l + 1];
                auto Ev = [&](int a, int b, int c) { return ec[a + C.nx * (b + C.ny * c)]; };
                E[l][i] = __fadd_rn(E[l][i], mg_interp(ax, ay, az, Ev(X0, Y0, Z0), Ev(X1, Y0, Z0), Ev(X0, Y1, Z0),
                                                       Ev(X1, Y1, Z0), Ev(X0, Y0, Z1), Ev(X1, Y0, Z1), Ev(X0, Y1, Z1),
                                                       Ev(X1, Y1, Z1)));
            }
            __syncthreads();
            for (int k = 0; k < nu; ++k) {
                sm_smooth(F, E[l], R[l], 0);
                sm_smooth(F, E[l], R[l], 1);
            }
        }
        for (int i = threadIdx.x; i < lvl_cells(T); i += blockDim.x) te[i] = E[t][i];
        __syncthreads();
    }
}

// --- device-side synthetic initial field ---------------------------------
// The Taylor-Green vortex plus PCG32 noise of af_seed_taylor_green, generated
// in parallel: draw k (two PCG outputs) of the sequential U, V, W; z, y, x
// order comes from jumping the generator ahead 2k steps (F. Brown, "Random
// number generation with arbitrary strides", 1994, the pcg32_advance
// method).  The trigonometric factors use binary32 sinpi/cospi, so the field
// is bit-reproducible on the device but not identical to the host
// generator's libm values.
__device__ __forceinline__ unsigned long long pcg_advance(unsigned long long state, unsigned long long inc,
                                                          unsigned long long delta) {
    unsigned long long cur_mult = 6364136223846793005ull, cur_plus = inc, acc_mult = 1ull, acc_plus = 0ull;
    while (delta > 0) {
        if (delta & 1ull) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1ull) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1;
    }
    return acc_mult * state + acc_plus;
}

__device__ __forceinline__ unsigned pcg_output(unsigned long long old) {
    const unsigned xorshifted = (unsigned)(((old >> 18u) ^ old) >> 27u);
    const unsigned rot = (unsigned)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

__global__ void k_seed_tg(Geom g, double* u, double* v, double* w, float H, unsigned long long state0,
                          unsigned long long inc, double amp, double noise) {
    const long long cu = (long long)(g.NX + 1) * g.NY * g.NZ, cv = (long long)g.NX * (g.NY + 1) * g.NZ,
                    cw = (long long)g.NX * g.NY * (g.NZ + 1);
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < cu + cv + cw;
         k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long st = pcg_advance(state0, inc, 2ull * (unsigned long long)k);
        const unsigned a = pcg_output(st) >> 5;
        const unsigned b = pcg_output(st * 6364136223846793005ull + inc) >> 6;
        const double uni = ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
        int comp, ex, ey;
        long long r;
        if (k < cu) { comp = 0; r = k; ex = g.NX + 1; ey = g.NY; }
        else if (k < cu + cv) { comp = 1; r = k - cu; ex = g.NX; ey = g.NY + 1; }
        else { comp = 2; r = k - cu - cv; ex = g.NX; ey = g.NY; }
        const int x = (int)(r % ex), y = (int)((r / ex) % ey), z = (int)(r / ((long long)ex * ey));
        // Staggered face positions: u at (i, j+1/2, k+1/2) H, v at (i+1/2, j, k+1/2) H.
        const float X = ((float)x + (comp == 0 ? 0.0f : 0.5f)) * H;
        const float Y = ((float)y + (comp == 1 ? 0.0f : 0.5f)) * H;
        const float Z = ((float)z + 0.5f) * H;
        float tg = 0.0f;
        if (comp == 0) tg = sinpif(2.0f * X) * cospif(2.0f * Y) * cospif(2.0f * Z);
        else if (comp == 1) tg = -cospif(2.0f * X) * sinpif(2.0f * Y) * cospif(2.0f * Z);
        const double val = amp * (double)tg + noise * (2.0 * uni - 1.0);
        const Dims& d = comp == 0 ? g.u : (comp == 1 ? g.v : g.w);
        AF_PTR(double) f = view(comp == 0 ? u : (comp == 1 ? v : w), d.count, DK_SEED, 0);
        f[(x + g.G) + (long long)(y + g.G) * d.sy + (long long)(z + g.G) * d.sz] = val;
    }
}

inline long long cdivl(long long a, long long b) { return (a + b - 1) / b; }

constexpr int kFwd[3] = {0, 1, 2};  // aeroflux.go:373
constexpr int kRev[3] = {2, 1, 0};  // aeroflux.go:390

// Profile event slots.
constexpr int kEvStart = 0, kEvEnd = 1, kEvSweep = 2 /* 2 per sweep */, kEvProj = 14 /* 2 per projection */;
constexpr int kNumEvents = 18;

// Device memory pool with first-fit placement and coalescing frees.
struct Pool {
    char* base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> bytes
    bool init(size_t bytes) {
        if (cudaMalloc(&base, bytes) != cudaSuccess) return false;
        size = bytes;
        free_[0] = bytes;
        return true;
    }
    char* alloc(size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                const size_t off = it->first, rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[off + bytes] = rest;
                return base + off;
            }
        }
        return nullptr;
    }
    void release(char* p, size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        size_t off = (size_t)(p - base);
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + bytes == next->first) {
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += bytes;
                return;
            }
        }
        free_[off] = bytes;
    }
};

struct SlotHost {
    bool used = false;
    bool active = false;
    af_config cfg{};
    InstDev d{};
    af_field_desc desc[8]{};
    char* mem = nullptr;   // pool or cudaMalloc block (arena unless external, b, multigrid)
    size_t mem_bytes = 0;
    bool external_arena = false;
};

}  // namespace

struct Batch {
    int cap = 0;
    int sms = 152;
    std::vector<SlotHost> slots;
    Pool pool;
    bool use_pool = false;
    cudaStream_t stream = nullptr;
    cudaStream_t body = nullptr;
    InstDev* d_inst = nullptr;
    Status* d_st = nullptr;
    Ctl* d_ctl = nullptr;
    int* d_tab = nullptr;            // S_COUNT prefix arrays of cap+1 ints
    std::vector<int> h_tab;
    Shape shape[S_COUNT];
    int grid_sz[S_COUNT] = {};       // blocks per stage, fixed when the graph is captured
    int graph_levels = 0;            // levels the captured graph covers
    unsigned graph_big = 0;          // levels whose large-coarsest smoothing the graph carries
    unsigned graph_pair = 0;         // levels with wide fused-pair tiles in the graph
    unsigned graph_pairn = 0;        // levels with narrow fused-pair tiles in the graph
    unsigned graph_single = 0;       // levels with in-place colour sweeps in the graph
    size_t tail_smem = 0;            // dynamic shared memory of the tail V-cycle
    int graph_nu = 0;                // smoothing sweeps the captured graph carries
    bool per_level = false;          // multigrid without the tail V-cycle above the coarsest level
    bool pairs = true;               // fused red-black pair smoothing below the tail
    bool cold = false;               // every projection starts from P = 0 (the reference's zeroing)
    cudaGraphExec_t graph = nullptr;
    bool tables_dirty = true;
    bool profiling = false;
    cudaEvent_t ev[kNumEvents] = {};
    int64_t launches = 0;
    int nu = 2;
    int vcycles = 4;  // V-cycles per refinement pass at most (measured best of 2, 3, 4, 6, 8)
    double pass_floor = 0.0;  // max|r| reduction one pass can reach (0: not used to cut V-cycles)
    int fixed_passes = 0;
    cudaError_t capture_err = cudaSuccess;
    bool tma_sweep = true;             // staged tile sweep (false: the row kernel)
    CUtensorMap* d_tmaps = nullptr;    // 12 per slot, see InstDev::tmap
    std::vector<CUtensorMap> h_tmaps;
    bool tmaps_dirty = true;
    CUtensorMap* d_pmaps = nullptr;    // 3 per level and slot, see InstDev::pmap
    std::vector<CUtensorMap> h_pmaps;
    int force_pair_var = -1;           // AEROFLUX_PAIR_VARIANT: every fused pair stage's variant (-1: tuned)
    bool pair_chosen = false;          // the fused pairs' tile variants are set (tuned or by level size)
    unsigned* d_diag = nullptr;        // nonzero: a kernel gave up waiting on a transfer
};

namespace {

int max_levels(const Batch* b) {
    int m = 1;
    for (const auto& s : b->slots)
        if (s.used) m = std::max(m, s.d.nlev);
    return m;
}

// Levels at which some slot's coarsest grid is too large for the one-block
// solver (smoothed in place instead).
unsigned big_coarse_levels(const Batch* b) {
    unsigned m = 0;
    for (const auto& s : b->slots)
        if (s.used && s.d.tail < 0) m |= 1u << (s.d.nlev - 1);
    return m;
}

// Levels some slot smooths in place (in-place colour sweeps, no second buffer).
unsigned single_levels(const Batch* b) {
    unsigned m = 0;
    for (const auto& s : b->slots) {
        if (!s.used) continue;
        const int lim = s.d.tail >= 0 ? s.d.tail : s.d.nlev - 1;
        for (int l = 0; l < lim; ++l)
            if (!s.d.lev[l].e2) m |= 1u << l;
    }
    return m;
}

// Levels whose fused pairs need the narrow tile column (wide: the others).
unsigned pair_levels(const Batch* b, bool narrow) {
    unsigned m = 0;
    for (const auto& s : b->slots) {
        if (!s.used) continue;
        const int lim = s.d.tail >= 0 ? s.d.tail : s.d.nlev - 1;
        for (int l = 0; l < lim; ++l) {
            const Lvl& L = s.d.lev[l];
            if (L.e2 && (narrow ? L.nxw < L.nx : L.nxw > 0)) m |= 1u << l;
        }
    }
    return m;
}

size_t tail_smem_bytes(const Batch* b) {
    size_t m = 0;
    for (const auto& s : b->slots)
        if (s.used && s.d.tail >= 0) m = std::max(m, (size_t)s.d.tail_floats * sizeof(float));
    return m;
}

// Items of stage `st` for slot `s` under shape sh.
long long stage_items(const SlotHost& S, int st, const Shape& sh) {
    if (!S.used || !S.active) return 0;
    const InstDev& I = S.d;
    const long long per = (long long)sh.tpb * sh.ept;
    long long n = 0;
    if (st == S_BC) n = bc_count(I.g);
    else if (st == S_SWEEP) n = sweep_box(I.g);
    else if (st == S_GRAD) n = 32ll * 3 * (I.g.NY + 1) * (I.g.NZ + 1);
    else if (st == S_SHADOW) n = I.shq[3];
    else if (st == S_SWEEPT) return I.sw_tiles;
    else if (st == S_DIV) n = (long long)I.g.p.nx * I.g.p.ny * I.g.p.nz;
    else if (st == S_INT) n = (long long)I.g.NX * I.g.NY * I.g.NZ;
    else if (st == S_CORR) n = 32ll * I.g.NY * I.g.NZ;
    else if (st == S_PBC) n = pbc_count(I.g);
    else if (st == S_COARSE) return I.tail >= 0 ? 1 : 0;
    const int lim = I.tail >= 0 ? I.tail : I.nlev - 1;  // levels smoothed by per-level kernels
    if (st < S_SMOOTH) {
        // n set above
    } else if (st < S_RESTRICT) {
        const int l = st - S_SMOOTH;
        n = (l < lim && !I.lev[l].e2) ? row_box(I.lev[l]) : 0;
    } else if (st >= S_RESTRICT && st < S_PROLONG) {
        const int l = st - S_RESTRICT;
        n = l < lim ? lvl_cells(I.lev[l + 1]) : 0;
    } else if (st >= S_PROLONG && st < S_BIGCOARSE) {
        const int l = st - S_PROLONG;
        n = l < lim ? prolong_box(I.lev[l], I.lev[l + 1]) : 0;
    } else if (st >= S_BIGCOARSE && st < S_PAIR) {
        const int l = st - S_BIGCOARSE;
        n = (l == I.nlev - 1 && I.tail < 0) ? row_box(I.lev[l]) : 0;
    } else if (st >= S_PAIR && st < S_COUNT) {
        const bool wide = st < S_PAIRN;
        const int l = st - (wide ? S_PAIR : S_PAIRN);
        if (l >= lim || !I.lev[l].e2) return 0;
        const Lvl& L = I.lev[l];
        const long long cols = wide ? L.nxw / kPairWideX : (L.nxw < L.nx ? 1 : 0);
        return cols * cdivl(L.ny, kPairVarTY[sh.var]) * cdivl(L.nz, kPairVarTZ[sh.var]);
    }
    return cdivl(n, per);
}

cudaError_t upload_tables(Batch* b) {
    const int w = b->cap + 1;
    b->h_tab.assign((size_t)S_COUNT * w, 0);
    for (int st = 0; st < S_COUNT; ++st) {
        int* pre = &b->h_tab[(size_t)st * w];
        long long acc = 0;
        for (int s = 0; s < b->cap; ++s) {
            pre[s] = (int)acc;
            acc += stage_items(b->slots[s], st, b->shape[st]);
        }
        pre[b->cap] = (int)acc;
    }
    std::vector<InstDev> inst(b->cap);
    for (int s = 0; s < b->cap; ++s) {
        inst[s] = b->slots[s].d;
        inst[s].active = b->slots[s].used && b->slots[s].active ? 1 : 0;
    }
    cudaError_t rc;
    if ((rc = cudaMemcpyAsync(b->d_tab, b->h_tab.data(), b->h_tab.size() * sizeof(int), cudaMemcpyHostToDevice,
                              b->stream)) != cudaSuccess)
        return rc;
    if ((rc = cudaMemcpyAsync(b->d_inst, inst.data(), inst.size() * sizeof(InstDev), cudaMemcpyHostToDevice,
                              b->stream)) != cudaSuccess)
        return rc;
    if (b->tmaps_dirty) {
        if ((rc = cudaMemcpyAsync(b->d_tmaps, b->h_tmaps.data(), b->h_tmaps.size() * sizeof(CUtensorMap),
                                  cudaMemcpyHostToDevice, b->stream)) != cudaSuccess ||
            (rc = cudaMemcpyAsync(b->d_pmaps, b->h_pmaps.data(), b->h_pmaps.size() * sizeof(CUtensorMap),
                                  cudaMemcpyHostToDevice, b->stream)) != cudaSuccess)
            return rc;
        b->tmaps_dirty = false;
    }
    b->tables_dirty = false;
    return cudaStreamSynchronize(b->stream);
}

Tab tab(const Batch* b, int st) { return Tab{b->d_tab + (size_t)st * (b->cap + 1), b->cap, b->shape[st].ept}; }
int grid(const Batch* b, int st) { return b->grid_sz[st] > 0 ? b->grid_sz[st] : b->sms * b->shape[st].bpsm; }

// Persistent grid of a stage: up to shape.bpsm blocks per SM, no more blocks
// than tiles at capture time but at least one per SM, so slots assigned
// later still spread over the whole GPU.
void size_grids(Batch* b) {
    const int w = b->cap + 1;
    for (int st = 0; st < S_COUNT; ++st) {
        const int items = b->h_tab[(size_t)st * w + b->cap];
        b->grid_sz[st] = std::max(b->sms, std::min(items, b->sms * b->shape[st].bpsm));
    }
}

#define LAUNCH(b, st, kernel, ...)                                                          \
    do {                                                                                    \
        kernel<<<grid(b, st), b->shape[st].tpb, 0, s>>>(__VA_ARGS__);                       \
        ++b->launches;                                                                      \
    } while (0)

void rec(Batch* b, int idx, cudaStream_t s) {
    if (b->profiling) cudaEventRecordWithFlags(b->ev[idx], s, cudaEventRecordExternal);
}

void enq_bc(Batch* b, int parity, int gate, cudaStream_t s) { LAUNCH(b, S_BC, kb_bc, b->d_inst, b->d_st, tab(b, S_BC), parity, gate); }

void enq_sweep(Batch* b, int axis, int parity, int phase, cudaStream_t s) {
    LAUNCH(b, S_SHADOW, kb_shadow, b->d_inst, tab(b, S_SHADOW), parity);
    if (b->tma_sweep) {
        const Tab t = tab(b, S_SWEEPT);
        const int g = grid(b, S_SWEEPT);
        if (axis == 0) kb_sweep_tma<0><<<g, kSwThreads, kSwSmem, s>>>(b->d_inst, b->d_st, t, parity, phase, b->d_diag);
        else if (axis == 1)
            kb_sweep_tma<1><<<g, kSwThreads, kSwSmem, s>>>(b->d_inst, b->d_st, t, parity, phase, b->d_diag);
        else kb_sweep_tma<2><<<g, kSwThreads, kSwSmem, s>>>(b->d_inst, b->d_st, t, parity, phase, b->d_diag);
        ++b->launches;
        return;
    }
    const Tab t = tab(b, S_SWEEP);
    if (axis == 0) LAUNCH(b, S_SWEEP, kb_sweep<0>, b->d_inst, b->d_st, t, parity, phase);
    else if (axis == 1) LAUNCH(b, S_SWEEP, kb_sweep<1>, b->d_inst, b->d_st, t, parity, phase);
    else LAUNCH(b, S_SWEEP, kb_sweep<2>, b->d_inst, b->d_st, t, parity, phase);
}

void enq_smooth(Batch* b, int st, int l, int pairs, int vc, cudaStream_t s) {
    for (int k = 0; k < pairs; ++k) {
        LAUNCH(b, st, kb_smooth, b->d_inst, b->d_ctl, tab(b, st), l, 0, vc);
        LAUNCH(b, st, kb_smooth, b->d_inst, b->d_ctl, tab(b, st), l, 1, vc);
    }
}

// One fused red-black pair of level l with stage st's tile variant (wide
// tiles for S_PAIR + l, the narrow column for S_PAIRN + l).
template <int LANES, int V>
void launch_pair_v(Batch* b, int st, int l, int dir, int vc, cudaStream_t s) {
    kb_smooth_pair<LANES, V><<<grid(b, st), PairTile<LANES, V>::THREADS, 0, s>>>(b->d_inst, b->d_ctl, tab(b, st), l,
                                                                               dir, vc);
    ++b->launches;
}

void launch_pair(Batch* b, int st, int l, int dir, int vc, cudaStream_t s) {
    const bool wide = st < S_PAIRN;
    if (wide && b->shape[st].var == 3) {
        kb_smooth_pair_zm<kZmZC><<<grid(b, st), kZmThreads, kZmSmem, s>>>(b->d_inst, b->d_ctl, tab(b, st), l, dir,
                                                                         vc, b->d_diag);
        ++b->launches;
        return;
    }
    switch (b->shape[st].var) {
        case 0: wide ? launch_pair_v<32, 0>(b, st, l, dir, vc, s) : launch_pair_v<16, 0>(b, st, l, dir, vc, s); break;
        case 1: wide ? launch_pair_v<32, 1>(b, st, l, dir, vc, s) : launch_pair_v<16, 1>(b, st, l, dir, vc, s); break;
        case 2: wide ? launch_pair_v<32, 2>(b, st, l, dir, vc, s) : launch_pair_v<16, 2>(b, st, l, dir, vc, s); break;
        default: wide ? launch_pair_v<32, 4>(b, st, l, dir, vc, s) : launch_pair_v<16, 4>(b, st, l, dir, vc, s);
    }
}

Shape pair_shape(bool wide, int var) {
    if (var == 3) return Shape{kZmThreads, 1, kZmBlocks, 3};
    const int threads = kPairVarTY[var] * (wide ? 32 : 16);
    return Shape{threads, 1, (var == 0 || var == 4 ? 2048 : 1536) / threads, var};
}

// Whether a used slot has wide pair tiles at level l without the staged
// pair's maps.
bool pair_tma_missing(const Batch* b, int l) {
    for (const auto& S : b->slots)
        if (S.used && l < S.d.nlev && S.d.lev[l].e2 && S.d.lev[l].nxw > 0 && !S.d.lev[l].tma) return true;
    return false;
}

// Whether every used slot whose level l has wide pair tiles can run the
// TMA-staged pair there (and at least one has them).
bool pair_tma_ok(const Batch* b, int l) {
    bool any = false;
    for (const auto& S : b->slots) {
        if (!S.used || l >= S.d.nlev) continue;
        const Lvl& L = S.d.lev[l];
        if (!L.e2 || L.nxw == 0) continue;
        if (!L.tma) return false;
        any = true;
    }
    return any;
}

// Pre- or post-smoothing of level l: fused pairs ping-ponging through e2
// (an even count returns the result to e) for slots that have e2, in-place
// colour sweeps for the others.
void enq_level_smooth(Batch* b, int l, int vc, cudaStream_t s) {
    // A pair reads the previous pair's output across the wide / narrow
    // boundary, so both kinds finish pair k before either starts pair k+1.
    for (int k = 0; k < b->nu; ++k) {
        if (b->graph_pair & (1u << l)) launch_pair(b, S_PAIR + l, l, k & 1, vc, s);
        if (b->graph_pairn & (1u << l)) launch_pair(b, S_PAIRN + l, l, k & 1, vc, s);
    }
    if (b->graph_single & (1u << l)) enq_smooth(b, S_SMOOTH + l, l, b->nu, vc, s);
}

// V-cycle vc of a refinement pass; slots whose pass runs fewer V-cycles
// skip it.
void enq_vcycle(Batch* b, int vc, cudaStream_t s) {
    const int L = b->graph_levels;
    for (int l = 0; l + 1 < L; ++l) {
        enq_level_smooth(b, l, vc, s);
        LAUNCH(b, S_RESTRICT + l, kb_restrict, b->d_inst, b->d_ctl, tab(b, S_RESTRICT + l), l, vc);
    }
    kb_vtail<<<grid(b, S_COARSE), kCoarseThreads, b->tail_smem, s>>>(b->d_inst, b->d_ctl, tab(b, S_COARSE), b->nu,
                                                                      vc);
    ++b->launches;
    for (int l = 0; l < L; ++l)
        if (b->graph_big & (1u << l)) enq_smooth(b, S_BIGCOARSE + l, l, 8 * b->nu, vc, s);
    for (int l = L - 2; l >= 0; --l) {
        LAUNCH(b, S_PROLONG + l, kb_prolong, b->d_inst, b->d_ctl, tab(b, S_PROLONG + l), l, vc);
        enq_level_smooth(b, l, vc, s);
    }
}

void enq_pass(Batch* b, cudaStream_t s, cudaGraphConditionalHandle h, int use_cond, int gate) {
    for (int k = 0; k < b->vcycles; ++k) enq_vcycle(b, k, s);
    LAUNCH(b, S_CORR, kb_correct, b->d_inst, b->d_ctl, tab(b, S_CORR));
    LAUNCH(b, S_INT, kb_residual, b->d_inst, b->d_st, b->d_ctl, tab(b, S_INT), gate, 1);
    kb_check<<<1, 256, 0, s>>>(b->d_inst, b->d_st, b->d_ctl, b->cap, h, use_cond, 1, gate, b->vcycles, b->pass_floor);
    ++b->launches;
}

// project, project.go:12-34, with binary64 refinement; s must be capturing.
void enq_project(Batch* b, int parity, int gate, cudaStream_t s) {
    rec(b, kEvProj + (gate == 3 ? 0 : 2), s);
    enq_bc(b, parity, gate, s);
    LAUNCH(b, S_DIV, kb_div, b->d_inst, b->d_st, tab(b, S_DIV), parity, gate);
    kb_init<<<1, 256, 0, s>>>(b->d_inst, b->d_ctl, b->cap);
    ++b->launches;
    LAUNCH(b, S_INT, kb_residual, b->d_inst, b->d_st, b->d_ctl, tab(b, S_INT), gate, 0);
    if (b->fixed_passes > 0) {
        kb_check<<<1, 256, 0, s>>>(b->d_inst, b->d_st, b->d_ctl, b->cap, 0, 0, 0, gate, b->vcycles, b->pass_floor);
        ++b->launches;
        for (int k = 0; k < b->fixed_passes; ++k) enq_pass(b, s, 0, 0, gate);
    } else {
        cudaStreamCaptureStatus cs;
        cudaGraph_t graph = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        cudaError_t rc = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
        if (rc != cudaSuccess || cs != cudaStreamCaptureStatusActive) {
            b->capture_err = rc != cudaSuccess ? rc : cudaErrorStreamCaptureUnsupported;
            return;
        }
        cudaGraphConditionalHandle h;
        if ((rc = cudaGraphConditionalHandleCreate(&h, graph, 0, cudaGraphCondAssignDefault)) != cudaSuccess) {
            b->capture_err = rc;
            return;
        }
        kb_check<<<1, 256, 0, s>>>(b->d_inst, b->d_st, b->d_ctl, b->cap, h, 1, 0, gate, b->vcycles, b->pass_floor);
        ++b->launches;
        if ((rc = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps)) != cudaSuccess) {
            b->capture_err = rc;
            return;
        }
        cudaGraphNodeParams params{cudaGraphNodeTypeConditional};  // the other members value-initialised
        params.conditional.handle = h;
        params.conditional.type = cudaGraphCondTypeWhile;
        params.conditional.size = 1;
        cudaGraphNode_t node;
        if ((rc = cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &params)) != cudaSuccess) {
            b->capture_err = rc;
            return;
        }
        cudaGraph_t body = params.conditional.phGraph_out[0];
        if ((rc = cudaStreamBeginCaptureToGraph(b->body, body, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
            b->capture_err = rc;
            return;
        }
        enq_pass(b, b->body, h, 1, gate);
        cudaGraph_t body_out = nullptr;
        if ((rc = cudaStreamEndCapture(b->body, &body_out)) != cudaSuccess) {
            b->capture_err = rc;
            return;
        }
        if ((rc = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
            cudaSuccess) {
            b->capture_err = rc;
            return;
        }
    }
    LAUNCH(b, S_PBC, kb_pbc, b->d_inst, b->d_st, tab(b, S_PBC), gate);
    LAUNCH(b, S_GRAD, kb_grad, b->d_inst, b->d_st, tab(b, S_GRAD), parity, gate, 0);
    enq_bc(b, parity, gate, s);
    rec(b, kEvProj + (gate == 3 ? 1 : 3), s);
}

// Step, aeroflux.go:348-409, for every active slot.
void enq_step(Batch* b, cudaStream_t s) {
    rec(b, kEvStart, s);
    for (int k = 0; k < 6; ++k) {
        const int axis = k < 3 ? kFwd[k] : kRev[k - 3];
        enq_bc(b, k & 1, k, s);
        rec(b, kEvSweep + 2 * k, s);
        enq_sweep(b, axis, k & 1, k, s);
        rec(b, kEvSweep + 2 * k + 1, s);
        if (k == 2) enq_project(b, 1, 3, s);
    }
    enq_project(b, 0, 6, s);
    kb_tick<<<1, 256, 0, s>>>(b->d_inst, b->d_st, b->cap);
    ++b->launches;
    rec(b, kEvEnd, s);
}

template <class F>
cudaError_t capture(Batch* b, F body, cudaGraphExec_t* out) {
    cudaGraph_t graph = nullptr;
    cudaError_t rc = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (rc != cudaSuccess) return rc;
    body();
    rc = cudaStreamEndCapture(b->stream, &graph);
    if (rc != cudaSuccess) return rc;
    if (b->capture_err != cudaSuccess) {
        rc = b->capture_err;
        b->capture_err = cudaSuccess;
        cudaGraphDestroy(graph);
        return rc;
    }
    rc = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return rc;
}

// Untuned tile variants of the fused pairs, by the largest level each pair
// stage serves: the largest tiles from 4 Mi cells, the middle ones from
// 256 Ki, the smallest below.  Set once, before the first capture (the
// captured kernels and the work lists must agree); the autotuner may replace
// them.
void default_pair_variants(Batch* b) {
    // A slot assigned after the choice may lack the staged pair's maps at a
    // level that runs it: that level goes back to the plain variant 1 tiles.
    for (int l = 0; l < kMaxLev; ++l)
        if (b->shape[S_PAIR + l].var == 3 && pair_tma_missing(b, l)) {
            b->shape[S_PAIR + l] = pair_shape(true, 1);
            b->tables_dirty = true;
            if (b->graph) {
                cudaGraphExecDestroy(b->graph);
                b->graph = nullptr;
            }
        }
    if (b->pair_chosen || b->graph) return;
    for (int l = 0; l < kMaxLev; ++l) {
        long long most = 0;
        for (const auto& S : b->slots)
            if (S.used && l < S.d.nlev) most = std::max(most, lvl_cells(S.d.lev[l]));
        int var = most >= (4ll << 20) ? 0 : (most >= (256ll << 10) ? 1 : 2);
        if (b->force_pair_var >= 0) var = b->force_pair_var;
        b->shape[S_PAIR + l] = pair_shape(true, var == 3 && !pair_tma_ok(b, l) ? 1 : var);
        b->shape[S_PAIRN + l] = pair_shape(false, var == 3 ? 1 : var);
    }
    b->pair_chosen = true;
    b->tables_dirty = true;
}

cudaError_t prepare(Batch* b) {
    cudaError_t rc;
    default_pair_variants(b);
    if (b->tables_dirty && (rc = upload_tables(b)) != cudaSuccess) return rc;
    const int L = max_levels(b);
    const unsigned big = big_coarse_levels(b), pair = pair_levels(b, false), pairn = pair_levels(b, true),
                   single = single_levels(b);
    const size_t tsm = tail_smem_bytes(b);
    if (b->graph && (L > b->graph_levels || (big & ~b->graph_big) || (pair & ~b->graph_pair) ||
                     (pairn & ~b->graph_pairn) || (single & ~b->graph_single) || tsm > b->tail_smem ||
                     b->graph_nu != b->nu)) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!b->graph) {
        b->graph_levels = std::max(L, b->graph_levels);
        b->graph_big |= big;
        b->graph_pair |= pair;
        b->graph_pairn |= pairn;
        b->graph_single |= single;
        b->tail_smem = std::max(b->tail_smem, tsm);
        b->graph_nu = b->nu;
        cudaFuncSetAttribute(kb_vtail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->tail_smem);
        b->launches = 0;
        size_grids(b);
        if ((rc = capture(b, [&] { enq_step(b, b->stream); }, &b->graph)) != cudaSuccess) {
            b->graph = nullptr;
            return rc;
        }
    }
    return cudaSuccess;
}

// Clears every slot's status (the step counter restarts at 0).  stop_at,
// when given, holds per slot the Steps it performs in the coming call: a slot
// with 0 < stop_at[s] < nsteps is gated from step stop_at[s] on -- its fault
// gate marks the end of that step's last phase, with no fault key -- so every
// later kernel skips it and its state stays that of its last Step.
cudaError_t reset_status(Batch* b, const std::vector<int64_t>* stop_at = nullptr, int64_t nsteps = 0) {
    std::vector<Status> h(b->cap, Status{kNoFault, 0u, kNoKey});
    if (stop_at)
        for (int s = 0; s < b->cap && s < (int)stop_at->size(); ++s)
            if ((*stop_at)[s] > 0 && (*stop_at)[s] < nsteps) h[s].fault_gate = 8u * (unsigned)(*stop_at)[s] - 1u;
    return cudaMemcpyAsync(b->d_st, h.data(), h.size() * sizeof(Status), cudaMemcpyHostToDevice, b->stream);
}

// A recorded gate without a fault key is a planned stop, not a fault.
bool status_faulted(const Status& st) { return st.fault_gate != kNoFault && st.fault_key != kNoKey; }

}  // namespace

std::string fault_message_for(const Geom& g, unsigned gate, unsigned long long key);

namespace {

// cuTensorMapEncodeTiled from the driver, resolved once through the runtime
// (the library links no driver stub); NULL when the driver lacks it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// The 12 tensor maps of a slot over its three binary32 shadows: per
// component, the staged boxes of a sweep along x, y and z and the
// axis-velocity box.  Out-of-range box elements load as zeros (never read).
bool encode_slot_maps(const InstDev& I, CUtensorMap* maps) {
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    for (int k = 0; k < 3; ++k) {
        const Dims& d = k == 0 ? I.g.u : (k == 1 ? I.g.v : I.g.w);
        const cuuint64_t dims[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)d.nz};
        const cuuint64_t strides[2] = {(cuuint64_t)I.shp[k] * 4u, (cuuint64_t)I.shp[k] * d.ny * 4u};
        const cuuint32_t estr[3] = {1, 1, 1};
        for (int role = 0; role < 4; ++role) {
            const cuuint32_t box[3] = {(cuuint32_t)sw_bx(role), (cuuint32_t)sw_by(role), (cuuint32_t)sw_bz(role)};
            if (enc(&maps[k * 4 + role], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, I.sh[k], dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return false;
        }
    }
    return true;
}

// The three tensor maps of the z-marching pair per level (e, e2, r: one
// plane of a 64 x 16 column plus a two-cell ring for e and e2, a one-cell
// ring for r) for every level with wide pair tiles whose rows and arrays are
// 16-byte aligned; sets Lvl::tma on those levels.
void encode_pair_maps(InstDev& I, CUtensorMap* maps) {
    auto enc = tensor_map_encoder();
    for (int l = 0; l < I.nlev; ++l) {
        Lvl& L = I.lev[l];
        L.tma = 0;
        if (!enc || !L.e2 || L.nxw == 0 || L.nx % 4 != 0) continue;
        auto aligned = [](const void* q) { return ((uintptr_t)q & 15u) == 0; };
        if (!aligned(L.e) || !aligned(L.e2) || !aligned(L.r)) continue;
        const cuuint64_t dims[3] = {(cuuint64_t)L.nx, (cuuint64_t)L.ny, (cuuint64_t)L.nz};
        const cuuint64_t strides[2] = {(cuuint64_t)L.nx * 4u, (cuuint64_t)L.nx * L.ny * 4u};
        const cuuint32_t estr[3] = {1, 1, 1};
        const cuuint32_t ebox[3] = {kZmBX, kZmEY, 1}, rbox[3] = {kZmBX, kZmRY, 1};
        float* arr[3] = {L.e, L.e2, L.r};
        bool ok = true;
        for (int k = 0; k < 3 && ok; ++k)
            ok = enc(&maps[3 * l + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, arr[k], dims, strides, k < 2 ? ebox : rbox,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        L.tma = ok ? 1 : 0;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host API
// ---------------------------------------------------------------------------
Batch* batch_create(int capacity, size_t pool_bytes, std::string* err) {
    Batch* b = new Batch();
    b->cap = capacity;
    b->slots.resize(capacity);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (const char* fp = getenv("AEROFLUX_FIXED_REFINEMENT_PASSES")) b->fixed_passes = std::max(0, atoi(fp));
    // Per-level multigrid kernels only (no tail V-cycle above the coarsest
    // level), and fused red-black pairs on or off: the same bits either way.
    if (const char* pl = getenv("AEROFLUX_MG_PER_LEVEL")) b->per_level = atoi(pl) != 0;
    if (const char* fp = getenv("AEROFLUX_MG_PAIRS")) b->pairs = atoi(fp) != 0;
    // The refinement solves to a tolerance, so it may start from the last
    // projection's pressure instead of zero (project.go:81-83 zeroes it for
    // the fixed sweep count of the red-black solver).
    if (const char* cs = getenv("AEROFLUX_COLD_START")) b->cold = atoi(cs) != 0;
    if (const char* vc = getenv("AEROFLUX_MG_VCYCLES")) b->vcycles = std::min(8, std::max(1, atoi(vc)));
    if (const char* pf = getenv("AEROFLUX_MG_PASS_FLOOR")) b->pass_floor = atoi(pf) < 0 ? ldexp(1.0, atoi(pf)) : 0.0;
    // The row sweep (gathers through L1) instead of the staged tile sweep: the same bits.
    if (const char* sr = getenv("AEROFLUX_SWEEP_ROWS")) b->tma_sweep = atoi(sr) == 0;
    if (b->tma_sweep && !tensor_map_encoder()) b->tma_sweep = false;
    b->shape[S_SWEEPT] = Shape{kSwThreads, 1, 4};  // shared memory holds four blocks' buffers per SM
    cudaFuncSetAttribute(kb_sweep_tma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwSmem);
    cudaFuncSetAttribute(kb_sweep_tma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwSmem);
    cudaFuncSetAttribute(kb_sweep_tma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwSmem);
    // Shapes: the tiny per-slot control and coarse stages keep their own.
    b->shape[S_COARSE] = Shape{kCoarseThreads, 1, 2};
    for (int l = 0; l < kMaxLev; ++l) {
        b->shape[S_PAIR + l] = pair_shape(true, 0);
        b->shape[S_PAIRN + l] = pair_shape(false, 0);
    }
    cudaError_t rc;
    if ((rc = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (rc = cudaStreamCreateWithFlags(&b->body, cudaStreamNonBlocking)) != cudaSuccess ||
        (rc = cudaMalloc(&b->d_inst, sizeof(InstDev) * capacity)) != cudaSuccess ||
        (rc = cudaMalloc(&b->d_st, sizeof(Status) * capacity)) != cudaSuccess ||
        (rc = cudaMalloc(&b->d_ctl, sizeof(Ctl) * (capacity + 1))) != cudaSuccess ||
        (rc = cudaMalloc(&b->d_tab, sizeof(int) * (size_t)S_COUNT * (capacity + 1))) != cudaSuccess ||
        (rc = cudaMalloc(&b->d_tmaps, sizeof(CUtensorMap) * 12 * (size_t)capacity)) != cudaSuccess ||
        (rc = cudaMalloc(&b->d_pmaps, sizeof(CUtensorMap) * 3 * kMaxLev * (size_t)capacity)) != cudaSuccess ||
        (rc = cudaMalloc(&b->d_diag, sizeof(unsigned))) != cudaSuccess) {
        *err = std::string("aeroflux: batch tables: ") + cudaGetErrorString(rc);
        batch_destroy(b);
        return nullptr;
    }
    cudaMemsetAsync(b->d_ctl, 0, sizeof(Ctl) * (capacity + 1), b->stream);
    cudaMemsetAsync(b->d_diag, 0, sizeof(unsigned), b->stream);
    b->h_tmaps.assign(12 * (size_t)capacity, CUtensorMap{});
    b->h_pmaps.assign(3 * kMaxLev * (size_t)capacity, CUtensorMap{});
    cudaFuncSetAttribute(kb_smooth_pair_zm<kZmZC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZmSmem);
    // The fused pairs' tile variant for every level (0-2 and 4; 3: TMA-staged
    // where the levels allow it), instead of the tuned or size-based choice.
    if (const char* pv = getenv("AEROFLUX_PAIR_VARIANT")) b->force_pair_var = std::min(4, std::max(0, atoi(pv)));
    if (pool_bytes) {
        if (!b->pool.init(pool_bytes)) {
            *err = "aeroflux: batch device pool of " + std::to_string(pool_bytes) + " bytes: out of memory";
            batch_destroy(b);
            return nullptr;
        }
        b->use_pool = true;
    }
    if (reset_status(b) != cudaSuccess || upload_tables(b) != cudaSuccess) {
        *err = "aeroflux: batch setup failed";
        batch_destroy(b);
        return nullptr;
    }
    return b;
}

void batch_destroy(Batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (auto& ev : b->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto& s : b->slots)
        if (s.used && !b->use_pool) cudaFree(s.mem);
    if (b->use_pool) cudaFree(b->pool.base);
    cudaFree(b->d_inst);
    cudaFree(b->d_st);
    cudaFree(b->d_ctl);
    cudaFree(b->d_tab);
    cudaFree(b->d_tmaps);
    cudaFree(b->d_pmaps);
    cudaFree(b->d_diag);
    if (b->body) cudaStreamDestroy(b->body);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

namespace {

// x extent covered by wide pair tiles: every whole 64 plus a last partial
// one of more than 32 cells; 1..32 remaining cells go to a narrow tile.
int pair_wide_x(int nx) {
    const int w = nx / kPairWideX * kPairWideX;
    return nx - w > kPairWideX / 2 ? w + kPairWideX : w;
}

// Multigrid hierarchy of a grid: coarsen every axis whose extent is even and
// >= 4 until the grid has <= kCoarsestCells cells or no axis halves.  Going
// down to 8 cells instead of 64 measured 0.2-2 % faster (256^3, 512^3, the
// 256-grid batch): the coarsest red-black solve (2 nmax^2 pairs, at least 8)
// is shorter on the smaller grid.
constexpr long long kCoarsestCells = 8;
int plan_levels(int nx, int ny, int nz, Lvl* lev, int* coarse_sweeps) {
    int n = 0;
    float wx = 1.0f, wy = 1.0f, wz = 1.0f;
    while (true) {
        Lvl& L = lev[n++];
        L = Lvl{nx, ny, nz, wx, wy, wz, 0, 0, 0, nullptr, nullptr,
                FastDiv((unsigned)nx), FastDiv((unsigned)ny), FastDiv((unsigned)((nx + 1) / 2)), nullptr,
                FastDiv((unsigned)std::max(1, pair_wide_x(nx) / kPairWideX)),
                {FastDiv((unsigned)((ny + kPairVarTY[0] - 1) / kPairVarTY[0])),
                 FastDiv((unsigned)((ny + kPairVarTY[1] - 1) / kPairVarTY[1])),
                 FastDiv((unsigned)((ny + kPairVarTY[2] - 1) / kPairVarTY[2]))},
                pair_wide_x(nx)};
        // An axis of extent 1 adds nothing to L e (its Neumann neighbours are
        // the cell itself, so its second difference is exactly 0); with its
        // weight kept, the relaxation would count the cell's old value as
        // two neighbours and damp every update on levels whose other axes
        // coarsened (weights 1/4, 1/16, ...).  Its weight is 0 unless every
        // axis has extent 1.
        if (nx > 1 || ny > 1 || nz > 1) {
            if (nx == 1) L.wx = 0.0f;
            if (ny == 1) L.wy = 0.0f;
            if (nz == 1) L.wz = 0.0f;
        }
        const long long c = (long long)nx * ny * nz;
        const int cx = nx % 2 == 0 && nx >= 4, cy = ny % 2 == 0 && ny >= 4, cz = nz % 2 == 0 && nz >= 4;
        if (c <= kCoarsestCells || !(cx || cy || cz) || n == kMaxLev) break;
        L.cx = cx;
        L.cy = cy;
        L.cz = cz;
        if (cx) { nx /= 2; wx *= 0.25f; }
        if (cy) { ny /= 2; wy *= 0.25f; }
        if (cz) { nz /= 2; wz *= 0.25f; }
    }
    const Lvl& last = lev[n - 1];
    const int nmax = std::max(last.nx, std::max(last.ny, last.nz));
    *coarse_sweeps = std::min(1000, std::max(8, 2 * nmax * nmax));
    return n;
}

// First level of the one-block tail V-cycle (every level from it down has at
// most kCoarseMax cells), or -1 when the coarsest level is larger.
int plan_tail(const Lvl* lev, int n, int* floats, bool coarsest_only = false) {
    *floats = 0;
    if (lvl_cells(lev[n - 1]) > kCoarseMax) return -1;
    int t = n - 1;
    while (!coarsest_only && t > 0 && lvl_cells(lev[t - 1]) <= kCoarseMax) --t;
    for (int l = t; l < n; ++l) *floats += 2 * (int)lvl_cells(lev[l]);
    return t;
}

af_field_desc fdesc(int64_t* off, int64_t nx, int64_t ny, int64_t nz) {
    af_field_desc f{*off, nx, ny, nz, nx, nx * ny, nx * ny * nz};
    int64_t sz = f.count * 8;
    if (int64_t r = sz % 128) sz += 128 - r;
    *off += sz;
    return f;
}

Dims dims_of(const af_field_desc& d) {
    return Dims{(int)d.nx, (int)d.ny, (int)d.nz, d.sy, d.sz, d.count};
}

}  // namespace

bool batch_config_fits(const af_config& c, std::string* err) {
    const int64_t g = c.ghost, cx = c.nx + 2 * g, cy = c.ny + 2 * g, cz = c.nz + 2 * g;
    // The kernels decode 32-bit element numbers (FastDiv) and keep the nine
    // velocity-BC write sets' prefix in int (InstDev::bc_off).
    Geom G{};
    G.NX = (int)std::min<int64_t>(c.nx, INT32_MAX);
    G.NY = (int)std::min<int64_t>(c.ny, INT32_MAX);
    G.NZ = (int)std::min<int64_t>(c.nz, INT32_MAX);
    const bool dims_ok = c.nx < (1 << 30) && c.ny < (1 << 30) && c.nz < (1 << 30) && g < (1 << 20);
    const double big = 2147483648.0;  // 2^31, compared in double so no product overflows
    const bool fields_ok = (double)(cx + 1) * cy * cz < big && (double)cx * (cy + 1) * cz < big &&
                           (double)cx * cy * (cz + 1) < big;
    if (!dims_ok || !fields_ok || (double)face_box(G) >= 2.0 * big || (double)bc_count(G) >= big) {
        if (err)
            *err = "aeroflux: grid too large for one batch slot (2^31 elements per field and per velocity-BC "
                   "write set)";
        return false;
    }
    return true;
}

size_t batch_slot_bytes(const af_config& c) {
    int64_t off = 0;
    const int64_t g = c.ghost, cx = c.nx + 2 * g, cy = c.ny + 2 * g, cz = c.nz + 2 * g;
    fdesc(&off, cx, cy, cz);
    fdesc(&off, cx + 1, cy, cz);
    fdesc(&off, cx, cy + 1, cz);
    fdesc(&off, cx, cy, cz + 1);
    fdesc(&off, cx, cy, cz);
    fdesc(&off, cx + 1, cy, cz);
    fdesc(&off, cx, cy + 1, cz);
    fdesc(&off, cx, cy, cz + 1);
    const size_t arena = ((size_t)off + 255) & ~(size_t)255;
    const size_t bb = ((size_t)(cx * cy * cz) * 8 + 255) & ~(size_t)255;
    auto al = [](int64_t n) { return ((size_t)n * 4 + 255) & ~(size_t)255; };
    auto pitch = [](int64_t nx) { return (nx + 3) / 4 * 4; };
    const size_t shb = al(pitch(cx + 1) * cy * cz) + al(pitch(cx) * (cy + 1) * cz) + al(pitch(cx) * cy * (cz + 1));
    Lvl lev[kMaxLev];
    int cs = 0, tf = 0;
    const int nl = plan_levels((int)c.nx, (int)c.ny, (int)c.nz, lev, &cs);
    const int tail = plan_tail(lev, nl, &tf);
    const int lim = tail >= 0 ? tail : nl - 1;
    size_t mg = 0;
    for (int l = 0; l < nl; ++l) mg += ((l < lim && c.inner_sweeps % 2 == 0) ? 3 : 2) * (size_t)lvl_cells(lev[l]) * sizeof(float);
    return arena + bb + shb + ((mg + 255) & ~(size_t)255);
}

int batch_assign(Batch* b, const af_config& c, char* arena, std::string* err) {
    int s = -1;
    for (int i = 0; i < b->cap; ++i)
        if (!b->slots[i].used) {
            s = i;
            break;
        }
    if (s < 0) {
        *err = "aeroflux: batch is full";
        return -1;
    }
    SlotHost& S = b->slots[s];
    S = SlotHost();
    S.cfg = c;
    InstDev& I = S.d;
    // Layout, grid.go:101-134.
    int64_t off = 0;
    const int64_t g = c.ghost, cx = c.nx + 2 * g, cy = c.ny + 2 * g, cz = c.nz + 2 * g;
    S.desc[0] = fdesc(&off, cx, cy, cz);
    S.desc[1] = fdesc(&off, cx + 1, cy, cz);
    S.desc[2] = fdesc(&off, cx, cy + 1, cz);
    S.desc[3] = fdesc(&off, cx, cy, cz + 1);
    S.desc[4] = fdesc(&off, cx, cy, cz);
    S.desc[5] = fdesc(&off, cx + 1, cy, cz);
    S.desc[6] = fdesc(&off, cx, cy + 1, cz);
    S.desc[7] = fdesc(&off, cx, cy, cz + 1);
    I.g.NX = (int)c.nx;
    I.g.NY = (int)c.ny;
    I.g.NZ = (int)c.nz;
    I.g.G = (int)c.ghost;
    I.g.p = dims_of(S.desc[0]);
    I.g.u = dims_of(S.desc[1]);
    I.g.v = dims_of(S.desc[2]);
    I.g.w = dims_of(S.desc[3]);
    if (!batch_config_fits(c, err)) {
        S = SlotHost();
        return -1;
    }
    I.fpx = FastDiv((unsigned)I.g.p.nx);
    I.fpy = FastDiv((unsigned)I.g.p.ny);
    I.ffx = FastDiv((unsigned)(I.g.NX + 1));
    I.ffy = FastDiv((unsigned)(I.g.NY + 1));
    I.ffz = FastDiv((unsigned)(I.g.NZ + 1));
    I.fnx = FastDiv((unsigned)I.g.NX);
    I.fny = FastDiv((unsigned)I.g.NY);
    {
        // bc_set_count of each (component, set), component-major: extents
        // (normal, first tangential, second tangential) per component.
        const long long N[3][3] = {{I.g.NX, I.g.NY, I.g.NZ}, {I.g.NY, I.g.NX, I.g.NZ}, {I.g.NZ, I.g.NX, I.g.NY}};
        long long acc = 0;
        for (int c = 0; c < 3; ++c)
            for (int set = 0; set < 3; ++set) {
                I.bc_off[3 * c + set] = (int)acc;
                const long long Nn = N[c][0], N1 = N[c][1], N2 = N[c][2];
                // Components 1 and 2 (V, W) have their first tangential
                // axis along x, the stride-1 one (bc_t1_first).
                unsigned d1, d2;
                bc_divisors((int)Nn, (int)N1, (int)N2, c != 0 && set == 2, set, &d1, &d2);
                I.bcd[3 * c + set][0] = FastDiv(d1);
                I.bcd[3 * c + set][1] = FastDiv(d2);
                acc += set == 0 ? 2 * N1 * N2 : (set == 1 ? 2 * (Nn + 1) * N2 : 2 * (Nn + 1) * (N1 + 2));
            }
        I.bc_off[9] = (int)acc;
    }
    I.nlev = plan_levels(I.g.NX, I.g.NY, I.g.NZ, I.lev, &I.coarse_sweeps);
    I.tail = plan_tail(I.lev, I.nlev, &I.tail_floats, b->per_level);
    const int lim = I.tail >= 0 ? I.tail : I.nlev - 1;
    // Fused red-black pairs need an even sweep count (the ping-pong returns
    // the result to e) and run on every level below the tail.  The batch's
    // sweep count is the first slot's; a slot joining a batch that sweeps an
    // odd number of times smooths in place.
    bool others = false;
    for (int i = 0; i < b->cap; ++i)
        if (i != s && b->slots[i].used) others = true;
    const int batch_nu = others ? b->nu : (int)c.inner_sweeps;
    const bool fused = c.inner_sweeps % 2 == 0 && batch_nu % 2 == 0 && b->pairs;
    auto pair_level = [&](int l) { return fused && l < lim; };
    const size_t arena_bytes = ((size_t)off + 255) & ~(size_t)255;
    const size_t b_bytes = ((size_t)S.desc[0].count * 8 + 255) & ~(size_t)255;
    size_t sh_bytes[3];
    for (int k = 0; k < 3; ++k) {
        const af_field_desc& d = S.desc[1 + k];
        I.shp[k] = (int)((d.nx + 3) / 4 * 4);
        sh_bytes[k] = ((size_t)I.shp[k] * d.ny * d.nz * 4 + 255) & ~(size_t)255;
    }
    {
        // Shadow conversion: (row, quad) items per component.
        int acc = 0;
        for (int k = 0; k < 3; ++k) {
            const af_field_desc& d = S.desc[1 + k];
            I.shq[k] = acc;
            I.fsq[k] = FastDiv((unsigned)(I.shp[k] / 4));
            acc += (int)(d.ny * d.nz * (I.shp[k] / 4));
        }
        I.shq[3] = acc;
        // Staged sweep tiles: x, y and z tiles from G covering the largest
        // component extent along each axis (a U row's extra face belongs to
        // its last x tile), three components per spatial tile.
        const int ntx = (I.g.NX + kSwTX - 1) / kSwTX;
        const int nty = (I.g.NY + 1 + kSwTY - 1) / kSwTY;
        const int ntz = (I.g.NZ + 1 + kSwTZ - 1) / kSwTZ;
        I.swx = FastDiv((unsigned)ntx);
        I.swy = FastDiv((unsigned)nty);
        I.sw_tiles = 3 * ntx * nty * ntz;
    }
    size_t mg = 0;
    for (int l = 0; l < I.nlev; ++l) mg += (pair_level(l) ? 3 : 2) * (size_t)lvl_cells(I.lev[l]) * sizeof(float);
    mg = (mg + 255) & ~(size_t)255;
    S.external_arena = arena != nullptr;
    S.mem_bytes = (arena ? 0 : arena_bytes) + b_bytes + sh_bytes[0] + sh_bytes[1] + sh_bytes[2] + mg;
    if (b->use_pool) {
        S.mem = b->pool.alloc(S.mem_bytes);
        if (!S.mem) {
            *err = "aeroflux: batch device pool exhausted";
            S = SlotHost();
            return -1;
        }
    } else if (cudaMalloc(&S.mem, S.mem_bytes) != cudaSuccess) {
        cudaGetLastError();
        *err = "aeroflux: batch slot allocation failed";
        S = SlotHost();
        return -1;
    }
    char* p = S.mem;
    char* base = arena;
    if (!arena) {
        base = p;
        p += arena_bytes;
        cudaMemsetAsync(base, 0, arena_bytes, b->stream);  // MAC.Zero, grid.go:158-163
    }
    for (int f = 0; f < 8; ++f) I.slot[f] = (double*)(base + S.desc[f].off);
    I.b = (double*)p;
    p += b_bytes;
    for (int k = 0; k < 3; ++k) {
        I.sh[k] = (float*)p;
        p += sh_bytes[k];
    }
    I.tmap = b->d_tmaps + 12 * (size_t)s;
    b->tmaps_dirty = true;
    if (b->tma_sweep && !encode_slot_maps(I, &b->h_tmaps[12 * (size_t)s])) {
        // No tensor maps for this slot: the whole batch sweeps with the row kernel.
        b->tma_sweep = false;
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
    }
    float* fp = (float*)p;
    for (int l = 0; l < I.nlev; ++l) {
        const long long n = lvl_cells(I.lev[l]);
        I.lev[l].e = fp;
        I.lev[l].r = fp + n;
        fp += 2 * n;
        I.lev[l].e2 = nullptr;
        if (pair_level(l)) {
            I.lev[l].e2 = fp;
            fp += n;
        }
    }
    cudaMemsetAsync(p, 0, mg, b->stream);
    I.pmap = b->d_pmaps + 3 * kMaxLev * (size_t)s;
    encode_pair_maps(I, &b->h_pmaps[3 * kMaxLev * (size_t)s]);
    const double half = c.dt * 0.5;  // aeroflux.go:353
    const double invH = 1.0 / c.h;
    I.dt_invh = (float)(half * invH);
    I.lam = (float)(c.viscosity * half * invH * invH);  // stencil.go:73
    I.div_scale = c.density / (c.dt * c.h);             // project.go:49
    I.h2 = c.h * c.h;                                   // project.go:107
    I.grad_scale = c.dt / (c.density * c.h);            // project.go:179
    I.res_scale = c.dt / (c.density * c.h * c.h);
    I.thresh = 0.5 * c.div_tol;
    I.max_refine = (unsigned)c.max_refine;
    I.parity = 0;
    I.warm = b->cold ? 0 : 1;
    cudaMemsetAsync(b->d_ctl + s, 0, sizeof(Ctl), b->stream);  // no measured V-cycle factor yet
    // Smoothing sweeps per level are a property of the batch's step graph:
    // the first slot of an empty batch sets them.
    b->nu = batch_nu;
    S.used = true;
    S.active = true;
    b->tables_dirty = true;
    return s;
}

void batch_release(Batch* b, int s) {
    SlotHost& S = b->slots[s];
    if (!S.used) return;
    cudaStreamSynchronize(b->stream);
    if (b->use_pool) b->pool.release(S.mem, S.mem_bytes);
    else cudaFree(S.mem);
    S = SlotHost();
    b->tables_dirty = true;
}

void batch_set_active(Batch* b, int s, bool active) {
    if (b->slots[s].active != active) {
        b->slots[s].active = active;
        b->tables_dirty = true;
    }
}

af_field_desc batch_field(const Batch* b, int s, int field, double** dev) {
    const SlotHost& S = b->slots[s];
    int f = field;
    if (S.d.parity && field != 0 && field != 4) f = field <= 3 ? field + 4 : field - 4;
    if (dev) *dev = S.d.slot[f];
    return S.desc[f];
}

const Geom& batch_geom(const Batch* b, int s) { return b->slots[s].d.g; }
cudaStream_t batch_stream(Batch* b) { return b->stream; }

cudaError_t batch_step(Batch* b, int64_t nsteps, std::string* err, const std::vector<int64_t>* stop_at) {
    cudaError_t rc;
    if ((rc = prepare(b)) != cudaSuccess) {
        *err = std::string("aeroflux: cuda: preparing the batched step: ") + cudaGetErrorString(rc);
        return rc;
    }
    if ((rc = reset_status(b, stop_at, nsteps)) != cudaSuccess) return rc;
    for (int64_t i = 0; i < nsteps; ++i)
        if ((rc = cudaGraphLaunch(b->graph, b->stream)) != cudaSuccess) {
            *err = std::string("aeroflux: cuda: cudaGraphLaunch: ") + cudaGetErrorString(rc);
            return rc;
        }
    return cudaSuccess;
}

cudaError_t batch_prepare_capture(Batch* b) {
    cudaError_t rc;
    default_pair_variants(b);
    if (b->tables_dirty && (rc = upload_tables(b)) != cudaSuccess) return rc;
    if (max_levels(b) > b->graph_levels && b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->graph_levels = std::max(b->graph_levels, max_levels(b));
    b->graph_big |= big_coarse_levels(b);
    b->graph_pair |= pair_levels(b, false);
    b->graph_pairn |= pair_levels(b, true);
    b->graph_single |= single_levels(b);
    b->tail_smem = std::max(b->tail_smem, tail_smem_bytes(b));
    if ((rc = cudaFuncSetAttribute(kb_vtail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->tail_smem)) !=
        cudaSuccess)
        return rc;
    size_grids(b);
    return cudaSuccess;
}

int64_t batch_enqueue_project(Batch* b, int parity, int gate, cudaStream_t s) {
    const int64_t before = b->launches;
    const bool prof = b->profiling;
    b->profiling = false;
    enq_project(b, parity, gate, s);
    b->profiling = prof;
    return b->launches - before;
}

cudaError_t batch_capture_error(Batch* b) {
    const cudaError_t rc = b->capture_err;
    b->capture_err = cudaSuccess;
    return rc;
}

Status* batch_status(Batch* b, int slot) { return b->d_st + slot; }

cudaError_t batch_project(Batch* b, std::string* err) {
    cudaError_t rc;
    if ((rc = batch_prepare_capture(b)) != cudaSuccess) return rc;
    if ((rc = reset_status(b)) != cudaSuccess) return rc;
    cudaGraphExec_t g = nullptr;
    const bool prof = b->profiling;
    b->profiling = false;
    rc = capture(b, [&] { enq_project(b, 0, 0, b->stream); }, &g);
    b->profiling = prof;
    if (rc != cudaSuccess) {
        *err = std::string("aeroflux: cuda: capturing the projection: ") + cudaGetErrorString(rc);
        return rc;
    }
    rc = cudaGraphLaunch(g, b->stream);
    cudaStreamSynchronize(b->stream);
    cudaGraphExecDestroy(g);
    return rc;
}

cudaError_t batch_velocity_bc(Batch* b) {
    cudaError_t rc;
    if (b->tables_dirty && (rc = upload_tables(b)) != cudaSuccess) return rc;
    if ((rc = reset_status(b)) != cudaSuccess) return rc;
    cudaStream_t s = b->stream;
    enq_bc(b, 0, 0, s);
    return cudaGetLastError();
}

cudaError_t batch_sweep(Batch* b, int axis, double dt) {
    cudaError_t rc;
    // A sweep at a caller-chosen dt: the per-slot sweep constants change for
    // this launch only.
    std::vector<std::pair<float, float>> keep;
    for (auto& S : b->slots) {
        keep.emplace_back(S.d.dt_invh, S.d.lam);
        if (!S.used) continue;
        const double invH = 1.0 / S.cfg.h;
        S.d.dt_invh = (float)(dt * invH);
        S.d.lam = (float)(S.cfg.viscosity * dt * invH * invH);
    }
    if ((rc = upload_tables(b)) != cudaSuccess) return rc;
    if ((rc = reset_status(b)) != cudaSuccess) return rc;
    cudaStream_t s = b->stream;
    enq_sweep(b, axis, 0, 0, s);
    rc = cudaGetLastError();
    for (int i = 0; i < b->cap; ++i) {
        b->slots[i].d.dt_invh = keep[i].first;
        b->slots[i].d.lam = keep[i].second;
    }
    b->tables_dirty = true;
    if (rc != cudaSuccess) return rc;
    if ((rc = cudaStreamSynchronize(s)) != cudaSuccess) return rc;
    std::vector<Status> st(b->cap);
    cudaMemcpy(st.data(), b->d_st, sizeof(Status) * b->cap, cudaMemcpyDeviceToHost);
    for (int i = 0; i < b->cap; ++i)
        if (b->slots[i].used && b->slots[i].active && st[i].fault_gate == kNoFault) b->slots[i].d.parity ^= 1;
    b->tables_dirty = true;
    return cudaSuccess;
}

cudaError_t batch_seed(Batch* b, int s, double amp, double noise, uint64_t seed, uint64_t stream) {
    SlotHost& S = b->slots[s];
    if (!S.used) return cudaErrorInvalidValue;
    // The fields start from zero (as after New), then the write ranges are set.
    for (int f = 1; f <= 3; ++f) cudaMemsetAsync(S.d.slot[f], 0, (size_t)S.desc[f].count * 8, b->stream);
    for (int f = 5; f <= 7; ++f) cudaMemsetAsync(S.d.slot[f], 0, (size_t)S.desc[f].count * 8, b->stream);
    S.d.parity = 0;
    b->tables_dirty = true;
    return seed_tg_fields(S.d.g, S.d.slot[1], S.d.slot[2], S.d.slot[3], S.cfg.h, amp, noise, seed, stream, b->stream);
}

cudaError_t seed_tg_fields(const Geom& g, double* u, double* v, double* w, double h, double amp, double noise,
                           uint64_t seed, uint64_t stream, cudaStream_t s) {
    // pcg32_srandom_r(seed, stream): state 0, one step, add the seed, one step.
    const unsigned long long inc = (stream << 1u) | 1u;
    unsigned long long st = inc;
    st += seed;
    st = st * 6364136223846793005ull + inc;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_seed_tg<<<sms * 4, 256, 0, s>>>(g, u, v, w, (float)h, st, inc, amp, noise);
    return cudaGetLastError();
}

int batch_collect_faults(Batch* b, std::string* msg, int* first_slot) {
    std::vector<Status> st(b->cap);
    cudaStreamSynchronize(b->stream);
    cudaMemcpy(st.data(), b->d_st, sizeof(Status) * b->cap, cudaMemcpyDeviceToHost);
    int n = 0;
    *first_slot = -1;
    for (int s = 0; s < b->cap; ++s) {
        SlotHost& S = b->slots[s];
        if (!S.used || !status_faulted(st[s])) continue;
        if (n++ == 0) {
            *first_slot = s;
            *msg = fault_message_for(S.d.g, st[s].fault_gate, st[s].fault_key);
        }
        // The faulting step returned before commitVelocity of the faulting
        // sweep: `phase` commits happened in it.
        S.d.parity ^= (int)((st[s].fault_gate % 8u) & 1u);
        b->tables_dirty = true;
    }
    return n;
}

bool batch_debug_bounds(unsigned long long* first, unsigned* count, bool reset) {
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

bool batch_device_error(Batch* b, std::string* msg) {
    unsigned v = 0;
    cudaStreamSynchronize(b->stream);
    cudaMemcpy(&v, b->d_diag, sizeof v, cudaMemcpyDeviceToHost);
    if (!v) return false;
    cudaMemset(b->d_diag, 0, sizeof v);
    *msg = (v & 4u)   ? "aeroflux: cuda: the staged pair's shared-memory rings are not 128-byte aligned; the step's "
                        "results are invalid"
           : (v & 2u) ? "aeroflux: cuda: the TMA-staged pair ran on a level without tensor maps; the step's results "
                        "are invalid"
                      : "aeroflux: cuda: a staged kernel gave up waiting for its tile transfer; the step's results "
                        "are invalid";
    return true;
}

bool batch_slot_faulted(const Batch* b, int s, std::string* msg) {
    Status st;
    cudaMemcpy(&st, b->d_st + s, sizeof st, cudaMemcpyDeviceToHost);
    if (!status_faulted(st)) return false;
    *msg = fault_message_for(b->slots[s].d.g, st.fault_gate, st.fault_key);
    return true;
}

void batch_slot_projection(Batch* b, int s, int64_t* passes, double* max_div, int64_t* vcycles) {
    Ctl c;
    cudaStreamSynchronize(b->stream);
    cudaMemcpy(&c, b->d_ctl + s, sizeof c, cudaMemcpyDeviceToHost);
    *passes = c.passes;
    *max_div = c.last_div;
    if (vcycles) *vcycles = c.vtotal;
}

cudaError_t batch_profile(Batch* b, bool on) {
    if (on == b->profiling) return cudaSuccess;
    cudaStreamSynchronize(b->stream);
    if (on)
        for (auto& ev : b->ev)
            if (!ev) {
                cudaError_t rc = cudaEventCreate(&ev);
                if (rc != cudaSuccess) return rc;
            }
    b->profiling = on;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return cudaSuccess;
}

cudaError_t batch_last_profile(Batch* b, double* step_ms, double* sweep_ms, double* proj_ms, int64_t* launches) {
    if (!b->profiling) return cudaErrorInvalidValue;
    cudaError_t rc = cudaStreamSynchronize(b->stream);
    if (rc != cudaSuccess) return rc;
    auto ms = [&](int a, int c) {
        float t = 0;
        rc = cudaEventElapsedTime(&t, b->ev[a], b->ev[c]);
        return (double)t;
    };
    *step_ms = ms(kEvStart, kEvEnd);
    *sweep_ms = 0;
    for (int k = 0; k < 6; ++k) *sweep_ms += ms(kEvSweep + 2 * k, kEvSweep + 2 * k + 1);
    *proj_ms = ms(kEvProj, kEvProj + 1) + ms(kEvProj + 2, kEvProj + 3);
    *launches = b->launches;
    return rc;
}

// ---------------------------------------------------------------------------
// Autotuner: for every stage that has work, time each candidate shape on the
// current slots (each launch is idempotent or acts on scratch that the next
// projection reinitialises; run it before uploading fields, or between
// steps) and keep the fastest.
// ---------------------------------------------------------------------------
std::string batch_tune(Batch* b, int reps) {
    const Shape cands[] = {{128, 1, 8}, {256, 1, 8}, {512, 1, 4}, {256, 2, 8}, {256, 4, 8},
                           {128, 4, 16}, {256, 1, 16}, {512, 2, 4}, {1024, 1, 2}};
    std::string report = "{";
    for (int& gz : b->grid_sz) gz = 0;
    reps = std::max(1, reps);
    std::vector<cudaEvent_t> rev(2 * (size_t)reps);
    for (auto& ev : rev) cudaEventCreate(&ev);
    cudaStream_t s = b->stream;
    // The control records must see the slots as they are now (a slot
    // assigned since the last upload would read as inactive, and every
    // multigrid stage would be timed as a no-op).
    if (b->tables_dirty) upload_tables(b);
    kb_init<<<1, 256, 0, s>>>(b->d_inst, b->d_ctl, b->cap);
    reset_status(b);
    const int L = max_levels(b);
    auto run = [&](int st) {
        const Tab t = tab(b, st);
        const int gsz = grid(b, st), tpb = b->shape[st].tpb;
        if (st == S_BC) kb_bc<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_st, t, 0, 0);
        else if (st == S_SWEEP) kb_sweep<0><<<gsz, tpb, 0, s>>>(b->d_inst, b->d_st, t, 0, 0);
        else if (st == S_SHADOW) kb_shadow<<<gsz, tpb, 0, s>>>(b->d_inst, t, 0);
        else if (st == S_DIV) kb_div<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_st, t, 0, 0);
        else if (st == S_INT) kb_residual<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_st, b->d_ctl, t, 0, 0);
        else if (st == S_PBC) kb_pbc<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_st, t, 0);
        else if (st == S_GRAD) kb_grad<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_st, t, 0, 0, 1);
        else if (st >= S_SMOOTH && st < S_RESTRICT) kb_smooth<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_ctl, t, st - S_SMOOTH, 0, 0);
        else if (st >= S_RESTRICT && st < S_PROLONG)
            kb_restrict<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_ctl, t, st - S_RESTRICT, 0);
        else if (st >= S_PROLONG && st < S_BIGCOARSE)
            kb_prolong<<<gsz, tpb, 0, s>>>(b->d_inst, b->d_ctl, t, st - S_PROLONG, 0);
        else if (st >= S_PAIR && st < S_PAIRN) launch_pair(b, st, st - S_PAIR, 0, 0, s);
        else if (st >= S_PAIRN && st < S_PAIRN + kMaxLev) launch_pair(b, st, st - S_PAIRN, 0, 0, s);
    };
    std::vector<int> stages = {S_BC, S_SHADOW, S_DIV, S_INT, S_PBC, S_GRAD};
    if (!b->tma_sweep) stages.push_back(S_SWEEP);  // the staged sweep keeps its fixed tile shape
    for (int l = 0; l + 1 < L; ++l) {
        stages.push_back(S_SMOOTH + l);
        stages.push_back(S_RESTRICT + l);
        stages.push_back(S_PROLONG + l);
    }
    bool first = true;
    // Fused pairs: one of three tile variants per level and tile column.
    for (int l = 0; l < L; ++l) {
        stages.push_back(S_PAIR + l);
        stages.push_back(S_PAIRN + l);
    }
    default_pair_variants(b);
    b->pair_chosen = true;
    const Shape pair_cands[2][4] = {{pair_shape(true, 0), pair_shape(true, 1), pair_shape(true, 2), pair_shape(true, 4)},
                                    {pair_shape(false, 0), pair_shape(false, 1), pair_shape(false, 2), pair_shape(false, 4)}};
    for (int st : stages) {
        long long items = 0;
        for (auto& S : b->slots) items += stage_items(S, st, b->shape[st]);
        if (!items) continue;
        Shape best = b->shape[st];
        float best_ms = 1e30f;
        const bool pair_st = st >= S_PAIR && st < S_PAIRN + kMaxLev;
        if (pair_st && b->force_pair_var >= 0) continue;
        std::vector<Shape> cs(cands, cands + sizeof cands / sizeof cands[0]);
        if (pair_st) {
            cs.assign(pair_cands[st >= S_PAIRN], pair_cands[st >= S_PAIRN] + 4);
            if (st < S_PAIRN && pair_tma_ok(b, st - S_PAIR)) cs.push_back(pair_shape(true, 3));
        }
        std::string tried;  // fused-pair stages: every tile variant's time
        for (const Shape& c : cs) {
            b->shape[st] = c;
            upload_tables(b);
            run(st);  // warm-up
            // Each repetition timed on its own; the median of them stands
            // for the candidate (one disturbed launch does not decide).
            for (int r = 0; r < reps; ++r) {
                cudaEventRecord(rev[2 * r], s);
                run(st);
                cudaEventRecord(rev[2 * r + 1], s);
            }
            cudaEventSynchronize(rev[2 * reps - 1]);
            std::vector<float> t(reps);
            for (int r = 0; r < reps; ++r) cudaEventElapsedTime(&t[r], rev[2 * r], rev[2 * r + 1]);
            std::nth_element(t.begin(), t.begin() + reps / 2, t.end());
            const float ms = t[reps / 2] * reps;  // per-launch median, scaled like the report's sum
            const bool ok = cudaGetLastError() == cudaSuccess;
            if (ok && ms < best_ms) {
                best_ms = ms;
                best = c;
            }
            if (pair_st) {
                char t[48];
                snprintf(t, sizeof t, "%s\"%d\": %.2f", tried.empty() ? "" : ", ", c.var, ok ? 1e3 * ms / reps : -1.0);
                tried += t;
            }
        }
        b->shape[st] = best;
        char buf[160];
        snprintf(buf, sizeof buf,
                 "%s\"stage_%d\": {\"tpb\": %d, \"ept\": %d, \"blocks_per_sm\": %d, \"variant\": %d, \"us\": %.2f",
                 first ? "" : ", ", st, best.tpb, best.ept, best.bpsm, best.var, 1e3 * best_ms / reps);
        report += buf;
        if (pair_st) report += ", \"variants_us\": {" + tried + "}";
        report += "}";
        first = false;
    }
    report += "}";
    for (auto& ev : rev) cudaEventDestroy(ev);
    upload_tables(b);
    kb_init<<<1, 256, 0, s>>>(b->d_inst, b->d_ctl, b->cap);
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    cudaStreamSynchronize(s);
    return report;
}

// Contained-fault text of the reference (arena.go:230-243 around Go's
// bounds-check panic) for a NaN backtrace at fault key `key` in sweep phase
// gate%8: the tap indices follow from the face, component, axis and strides.
std::string fault_message_for(const Geom& g, unsigned gate, unsigned long long key) {
    const int phase = (int)(gate % 8u);
    const int axis = phase < 3 ? kFwd[phase] : kRev[phase - 3];
    const int comp = (int)(key >> 60);
    const unsigned long long z = (key >> 40) & 0xFFFFF, y = (key >> 20) & 0xFFFFF, x = key & 0xFFFFF;
    const Dims& d = comp == 0 ? g.u : (comp == 1 ? g.v : g.w);
    unsigned long long x0 = x, y0 = y, z0 = z;
    const unsigned long long nan_int = 0x8000000000000000ull;
    if (axis == 0) x0 = nan_int;
    if (axis == 1) y0 = nan_int;
    if (axis == 2) z0 = nan_int;
    const unsigned long long sy = (unsigned long long)d.sy, sz = (unsigned long long)d.sz;
    const unsigned long long i000 = x0 + y0 * sy + z0 * sz;
    const unsigned long long taps[8] = {i000, i000 + 1, i000 + sy, i000 + sy + 1,
                                        i000 + sz, i000 + sz + 1, i000 + sz + sy, i000 + sz + sy + 1};
    char buf[200];
    for (unsigned long long t : taps) {
        const long long idx = (long long)t;
        if (idx < 0) {
            snprintf(buf, sizeof buf, "aeroflux: guard-page fault contained: runtime error: index out of range [%lld]", idx);
            return buf;
        }
        if (idx >= d.count) {
            snprintf(buf, sizeof buf,
                     "aeroflux: guard-page fault contained: runtime error: index out of range [%lld] with length %lld",
                     idx, (long long)d.count);
            return buf;
        }
    }
    return "aeroflux: guard-page fault contained: runtime error: index out of range";
}

}  // namespace af
