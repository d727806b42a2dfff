/*
 * aeroflux_oracle.h -- CPU restatement of AeroFlux's fractional-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle the CUDA path is
 * checked against.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it; the product library never links or calls it.
 *
 * Parity pin status: the reference (a Go package) ships no golden vectors and
 * no known-answer test for this path, and Go is not available to run it, so
 * bit-level parity with the reference itself is UNPINNED.  The restatement is
 * checked against every property the reference's own tests assert and against
 * the magnitudes its README publishes (see tests/test_oracle_*.py).
 *
 * Every function cites the reference file:line it restates (paths inside the
 * AeroFlex module).  Arithmetic follows Go's amd64 semantics: left-to-right
 * evaluation, no fused multiply-add (build with -ffp-contract=off), IEEE
 * division, and CVTTSD2SQ float->int conversion (NaN -> INT64_MIN) so a NaN
 * backtrace produces the same contained-fault error text Go's bounds check
 * would.
 */
#ifndef AEROFLUX_ORACLE_H
#define AEROFLUX_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Config, aeroflux.go:14-41.  Go `int` is 64-bit on every supported target. */
typedef struct orc_config {
    int64_t nx, ny, nz;
    int64_t ghost;
    double h;
    double viscosity;
    double density;
    double dt;
    int64_t workers;
    int64_t gauss_seidel_iters;
    int32_t use_sparse_solver;
    int32_t lock;
} orc_config;

/* Field, grid.go:12-21.  off is a byte offset, like Go's Field.Off. */
typedef struct orc_field {
    int64_t off, nx, ny, nz, sy, sz, count;
} orc_field;

enum { ORC_P = 0, ORC_U, ORC_V, ORC_W, ORC_DIV, ORC_TMP0, ORC_TMP1, ORC_TMP2, ORC_NFIELDS };

typedef struct orc_engine orc_engine;

/* (*Config).Normalize, aeroflux.go:47-113.  Returns 0 or -1 with Go's text in err. */
int orc_normalize(orc_config* c, char* err, size_t errlen);
/* MACBytes, grid.go:138-144 (0 when the extents are invalid). */
int64_t orc_mac_bytes(int64_t nx, int64_t ny, int64_t nz, int64_t ghost);
/* New, aeroflux.go:176-213.  NULL plus Go's text in err on failure. */
orc_engine* orc_new(const orc_config* c, char* err, size_t errlen);
/* Close, aeroflux.go:419-439.  Safe on NULL. */
void orc_close(orc_engine* e);
/* Normalized config the engine runs with. */
void orc_get_config(const orc_engine* e, orc_config* out);
/* Current descriptor of field id (descriptors swap during a step) and its data. */
double* orc_field_data(orc_engine* e, int id, orc_field* desc);
/* Whole arena (layout of grid.go:101-134), MACBytes long. */
unsigned char* orc_arena(orc_engine* e, int64_t* bytes);

/* Advection scheme of the sweeps (the engine's SetAdvection): 0 the
 * reference's semi-Lagrangian sweep, 1 MacCormack.  0 or -1. */
enum { ORC_ADVECTION_SEMI_LAGRANGIAN = 0, ORC_ADVECTION_MACCORMACK = 1 };
int orc_set_advection(orc_engine* e, int scheme);

/* Step, aeroflux.go:348-409.  0 or -1 with the first contained fault in err. */
int orc_step(orc_engine* e, char* err, size_t errlen);
/* project, project.go:12-34 (the reference's tests call it directly). */
int orc_project(orc_engine* e, char* err, size_t errlen);
/* Phase hooks for stage-level parity tests. */
void orc_apply_velocity_bc(orc_engine* e);                 /* stencil.go:246-315 */
int orc_sweep(orc_engine* e, int axis, double dt, char* err, size_t errlen); /* dispatch(sweep) + commit */
void orc_compute_divergence(orc_engine* e);                /* project.go:42-62 */
void orc_solve_pressure_red_black(orc_engine* e);          /* project.go:73-100 */
void orc_apply_pressure_bc(orc_engine* e);                 /* project.go:139-163 */
void orc_subtract_gradient(orc_engine* e);                 /* project.go:172-205 */
void orc_commit_velocity(orc_engine* e);                   /* commitVelocity, stencil.go:230-235 */

/* Diagnostics. */
double orc_max_divergence(orc_engine* e);  /* project.go:210-232 */
double orc_kinetic_energy(orc_engine* e);  /* project.go:238-258 */
double orc_max_velocity(orc_engine* e);    /* stencil.go:319-331 */
double orc_cfl(orc_engine* e);             /* stencil.go:336-338 */

/* The reference's test inputs. */
void orc_seed_vortex(orc_engine* e, double amp);  /* engine_test.go:302-335 */
void orc_seed_shear_layer(orc_engine* e);         /* example_test.go:34-47 */
/* The benchmark's seeded Taylor-Green + PCG32 field (no BC applied). */
void orc_seed_taylor_green(orc_engine* e, double amp, double noise, uint64_t seed, uint64_t stream);

/* Planted mistakes for the oracle's self-checks (0: none): 1 runs the u
 * z-ghost reflection (stencil.go:285-290) before the y-ghost one (279-284);
 * 2 contracts the trilinear x-lerps into fused multiply-adds; 3 sweeps black
 * before red (project.go:88-97); 4 mirrors the pressure z-ghosts before the
 * x- and y-ghosts (project.go:139-163); 5 pairs the red-black neighbour sum
 * instead of Go's left-to-right order (project.go:125).  Process-wide;
 * tests only. */
void orc_set_mutation(int m);

/* Go strconv.FormatFloat(v, 'g', -1, 64), i.e. fmt's %v / %g for float64. */
void orc_go_format_float(double v, char* out, size_t outlen);

#ifdef __cplusplus
}
#endif
#endif
