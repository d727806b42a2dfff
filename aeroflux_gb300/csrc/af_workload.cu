// af_workload.cu -- host-side synthetic inputs for the engine: the seeded
// Taylor-Green initial field used by every benchmark configuration.
//
// The reference's own tests seed a trigonometric field straight into arena
// views (seedVortex, engine_test.go:302-335) and then apply the velocity BC;
// this generator writes the same index ranges in the same field and loop
// order (U, V, W; z, y, x) with a Taylor-Green vortex sampled at the staggered
// face positions plus i.i.d. uniform noise from PCG32.
#include "../../include/aeroflux_cuda.h"

#include <math.h>
#include <string.h>

namespace {

// PCG32, XSH-RR 64/32 (M.E. O'Neill, "PCG: A Family of Simple Fast
// Space-Efficient Statistically Good Algorithms for Random Number
// Generation", 2014), seeded as pcg32_srandom_r(initstate, initseq).
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    Pcg32(uint64_t initstate, uint64_t initseq) {
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // 53-bit uniform double in [0, 1) from two outputs.
    double uniform() {
        const uint32_t a = next() >> 5, b = next() >> 6;
        return ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
    }
};

}  // namespace

extern "C" int af_seed_taylor_green(const af_config* cfg, double amp, double noise, uint64_t seed, uint64_t stream,
                                    double* u, double* v, double* w) {
    if (!cfg || !u || !v || !w || cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1 || cfg->ghost < 1 || !(cfg->h > 0))
        return AF_ERR_ARG;
    const int64_t g = cfg->ghost, NX = cfg->nx, NY = cfg->ny, NZ = cfg->nz;
    const int64_t cx = NX + 2 * g, cy = NY + 2 * g, cz = NZ + 2 * g;
    // Padded extents of U, V, W (grid.go:121-123).
    const int64_t usy = cx + 1, usz = (cx + 1) * cy;
    const int64_t vsy = cx, vsz = cx * (cy + 1);
    const int64_t wsy = cx, wsz = cx * cy;
    memset(u, 0, sizeof(double) * (size_t)((cx + 1) * cy * cz));
    memset(v, 0, sizeof(double) * (size_t)(cx * (cy + 1) * cz));
    memset(w, 0, sizeof(double) * (size_t)(cx * cy * (cz + 1)));
    const double h = cfg->h;
    const double twopi = 6.283185307179586;
    Pcg32 rng(seed, stream);
    auto jitter = [&]() { return noise * (2.0 * rng.uniform() - 1.0); };
    for (int64_t z = g; z < g + NZ; ++z)
        for (int64_t y = g; y < g + NY; ++y)
            for (int64_t x = g; x <= g + NX; ++x) {
                const double X = (double)(x - g) * h, Y = ((double)(y - g) + 0.5) * h, Z = ((double)(z - g) + 0.5) * h;
                u[x + y * usy + z * usz] = amp * sin(twopi * X) * cos(twopi * Y) * cos(twopi * Z) + jitter();
            }
    for (int64_t z = g; z < g + NZ; ++z)
        for (int64_t y = g; y <= g + NY; ++y)
            for (int64_t x = g; x < g + NX; ++x) {
                const double X = ((double)(x - g) + 0.5) * h, Y = (double)(y - g) * h, Z = ((double)(z - g) + 0.5) * h;
                v[x + y * vsy + z * vsz] = -amp * cos(twopi * X) * sin(twopi * Y) * cos(twopi * Z) + jitter();
            }
    for (int64_t z = g; z <= g + NZ; ++z)
        for (int64_t y = g; y < g + NY; ++y)
            for (int64_t x = g; x < g + NX; ++x) w[x + y * wsy + z * wsz] = 0.0 + jitter();
    return AF_OK;
}
