// af_internal.h -- types shared by the engine (af_engine.cu) and the kernels
// (af_fp64.cu, af_mixed.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace af {

// Field geometry on the device: padded extents and strides of grid.go:12-21.
// Indices inside one field fit in int32 up to ~1280^3; row bases are formed
// in 64 bits so larger grids stay correct.
struct Dims {
    int nx, ny, nz;
    long long sy, sz, count;
};

// Grid geometry shared by every stage.
struct Geom {
    int NX, NY, NZ, G;   // interior extents and ghost thickness
    Dims p, u, v, w;     // P (= Div shape), U (= Tmp0), V (= Tmp1), W (= Tmp2)
};

// Device status block of one engine.
//  fault_gate: step*8 + sweep phase (0..5) of the first contained fault,
//              0xFFFFFFFF when none.  Every kernel of a later phase returns at
//              entry, so the state freezes where the reference's Step returns.
//  step:       device step counter, bumped at the end of each captured step.
//  fault_key:  min over the faults of that phase of (component, z, y, x),
//              the order the reference's single-worker loop meets them.
struct Status {
    unsigned int fault_gate;
    unsigned int step;
    unsigned long long fault_key;
};

constexpr unsigned int kNoFault = 0xFFFFFFFFu;
constexpr unsigned long long kNoKey = ~0ull;

__host__ __device__ inline unsigned long long fault_key(int comp, int x, int y, int z) {
    return ((unsigned long long)comp << 60) | ((unsigned long long)(unsigned)z << 40) |
           ((unsigned long long)(unsigned)y << 20) | (unsigned long long)(unsigned)x;
}

// Pointers of the eight arena fields (current descriptor slots).
struct Fields {
    double* p;
    double* u;
    double* v;
    double* w;
    double* div;
    double* t0;
    double* t1;
    double* t2;
};

// --- FP64 plain-form stage launchers (af_fp64.cu) ---------------------------
// `gate` is the step-relative phase index a kernel belongs to: it returns at
// entry when a fault was recorded at an earlier (step, phase).
void launch_velocity_bc(const Geom& g, double* u, double* v, double* w, Status* st, int gate, cudaStream_t s);
void launch_sweep_fp64(const Geom& g, int axis, const Fields& f, double dt, double invH, double lam,
                       Status* st, int phase, cudaStream_t s);
// MacCormack form of the same sweep: forward semi-Lagrangian step into
// fwd.t0..t2 (fwd.u/v/w = f.u/v/w), then the limited correction plus the
// directional diffusion into f.t0..t2.  Two launches.
void launch_maccormack_fp64(const Geom& g, int axis, const Fields& f, const Fields& fwd, double dt, double invH,
                            double lam, Status* st, int phase, cudaStream_t s);
// zero_p also zeroes all of P, as solvePressureRedBlack does first (project.go:81-83).
void launch_divergence_fp64(const Geom& g, const Fields& f, double* b, double scale, double h2, bool zero_p,
                            Status* st, int gate, cudaStream_t s);
void launch_rbgs_fp64(const Geom& g, double* p, const double* b, int color, Status* st, int gate,
                      cudaStream_t s);
void launch_pressure_bc_fp64(const Geom& g, double* p, Status* st, int gate, cudaStream_t s);
void launch_gradient_fp64(const Geom& g, const Fields& f, double scale, Status* st, int gate, cudaStream_t s);
void launch_step_tick(Status* st, cudaStream_t s);
void launch_b_from_div(const Geom& g, const double* div, double* b, double h2, cudaStream_t s);

// Diagnostics (af_fp64.cu).  `out` receives the bit pattern of a
// non-negative double (max) or the fixed-order sum; `scratch` holds one
// partial per z-plane for the sum.
void launch_max_divergence(const Geom& g, const double* u, const double* v, const double* w, double invH,
                           unsigned long long* out, cudaStream_t s);
void launch_max_abs3(const double* u, long long nu, const double* v, long long nv, const double* w, long long nw,
                     unsigned long long* out, cudaStream_t s);
void launch_kinetic_energy(const Geom& g, const double* u, const double* v, const double* w, double* partials,
                           double* out, cudaStream_t s);

// The reference's contained-fault text for a NaN backtrace recorded with
// fault gate `gate` (step*8 + sweep phase) and fault key `key`.
std::string fault_message_for(const Geom& g, unsigned gate, unsigned long long key);

// Writes the seeded Taylor-Green + PCG32 noise initial field into the write
// ranges of u, v, w (device, af_batch.cu).
cudaError_t seed_tg_fields(const Geom& g, double* u, double* v, double* w, double h, double amp, double noise,
                           uint64_t seed, uint64_t stream, cudaStream_t s);

// Compares both exact /6 forms with IEEE division on n random bit patterns
// (af_fp64.cu); false on a CUDA error.
bool selftest_div6(unsigned long long n, unsigned long long seed, unsigned long long* mismatches);
// Compares the integer-pipe binary64 add and subtract with the native ones.
bool selftest_dadd(unsigned long long n, unsigned long long seed, unsigned long long* mismatches);

// Debug build (AEROFLUX_DEBUG_BOUNDS): the first out-of-buffer access each
// kernel unit recorded -- (kernel << 56) | (slot << 40) | offset, ~0 when
// none -- and how many there were; reset clears them.  Product build: none.
bool fp64_debug_bounds(unsigned long long* first, unsigned* count, bool reset);
bool batch_debug_bounds(unsigned long long* first, unsigned* count, bool reset);
// Both units together; true with *msg set when the debug build recorded a
// violation (the record is then cleared).
bool debug_bounds_error(std::string* msg);

// Binary64 FMA issue rate of the current device (independent chains, timed
// with events); false on a CUDA error.
bool measure_fp64_rate(double* fma_per_s);

}  // namespace af
