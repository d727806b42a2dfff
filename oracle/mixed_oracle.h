/*
 * mixed_oracle.h -- CPU restatement of the mixed-precision form's arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY, like aeroflux_oracle.h: tests/ load it to check
 * the CUDA mixed, batched and served forms bit for bit.  The product library
 * never links or calls it.
 *
 * The mixed form has no counterpart in the reference; what it restates is the
 * reference's step (aeroflux.go:348-409) with the sweep's arithmetic
 * (stencil.go:44-225) in binary32 and the projection (project.go:12-205)
 * solved by binary64 iterative refinement around binary32 multigrid.  Every
 * binary32 operation is written with an explicit rounding (fmaf for a fused
 * multiply-add, plain operators otherwise, built with -ffp-contract=off), in
 * the order the CUDA kernels evaluate it, so the two agree bit for bit on any
 * IEEE host.  Binary64 stages that the mixed form shares with the FP64 form
 * (velocity BC, divergence, pressure BC, gradient) come from
 * aeroflux_oracle.c.
 */
#ifndef AEROFLUX_MIXED_ORACLE_H
#define AEROFLUX_MIXED_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* binary64 -> binary32 as the mixed form converts: round half away from zero
 * on the magnitude, results below FLT_MIN flush to signed zero, Inf/NaN kept
 * (a NaN becomes the quiet NaN with the same sign). */
float mxo_f64_to_f32(double d);
/* binary32 -> binary64, exact; subnormal inputs flush to signed zero. */
double mxo_f32_to_f64(float f);

/* One binary32 axis sweep of U, V, W (the current fields, padded MAC layout
 * of an NX x NY x NZ grid with ghost G) into tu, tv, tw over the reference's
 * write ranges (stencil.go:21-25, 63-67); nothing else of tu, tv, tw is
 * written.  dt_invh = (float)(dt/H), lam = (float)(nu dt/H^2).  Returns the
 * number of faces whose backtrace was NaN (a contained fault; those faces are
 * not written). */
int64_t mxo_sweep(int64_t NX, int64_t NY, int64_t NZ, int64_t G, int axis, float dt_invh, float lam,
                  const double* u, const double* v, const double* w, double* tu, double* tv, double* tw);

typedef struct mxo_solver mxo_solver;

/* Multigrid hierarchy and refinement state of one grid.  nu: red-black
 * smoothing pairs per level before and after each coarse correction;
 * max_refine: pass cap; vcycles: V-cycles per pass at most; div_tol: target
 * max|div|; pass_floor: 0, or the max|r| reduction one pass can reach. */
mxo_solver* mxo_solver_new(int64_t NX, int64_t NY, int64_t NZ, int64_t nu, int64_t max_refine, int64_t vcycles,
                           double div_tol, double dt, double density, double h, double pass_floor);
void mxo_solver_free(mxo_solver* s);
/* Levels of the hierarchy and, per level, extents, coarsening flags and
 * binary32 weights (out arrays of at least 16 entries); the first level of
 * the one-block tail (-1: none) and the coarsest sweep count. */
int mxo_solver_levels(const mxo_solver* s, int32_t* nx, int32_t* ny, int32_t* nz, int32_t* cx, int32_t* cy,
                      int32_t* cz, float* wx, float* wy, float* wz, int32_t* tail, int32_t* coarse_sweeps);

/* The refinement solve of one projection: p (the padded binary64 pressure,
 * interior updated in place) toward L p = b (b padded like p, interior
 * read).  fixed_passes > 0 runs that many passes (a stopped grid skips
 * them) instead of looping while the grid is unconverged.  Returns the
 * refinement passes; *vcycles gets the V-cycles run, *last_div the last
 * estimate dt/(rho h^2) max|r|. */
int64_t mxo_refine(mxo_solver* s, int64_t G, double* p, const double* b, int64_t fixed_passes, int64_t* vcycles,
                   double* last_div);

/* One V-cycle on level 0 arrays (compact NX x NY x NZ binary32 e and r):
 * e is improved in place toward L e = r. */
void mxo_vcycle(mxo_solver* s, float* e, const float* r);

/* Mutations for the oracle's self-checks (0: none).  Each plants one
 * mistake into the restatement so a test can show that the bit-level
 * comparisons catch it: 1 swaps the colour order of the smoother, 2 rounds
 * the relaxation's fused multiply-add in two steps, 3 sums the face velocity
 * in another order, 4 drops the zero-weight axis rule of a level. */
void mxo_set_mutation(int m);

#ifdef __cplusplus
}
#endif
#endif
