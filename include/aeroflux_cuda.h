/*
 * aeroflux_cuda.h -- C ABI of libaeroflux_cuda, the GB300 (sm_103a) engine for
 * AeroFlux's fractional-step timestep: semi-Lagrangian advection, axis-swept
 * explicit diffusion and red-black Gauss-Seidel pressure projection.
 *
 * The ABI is what a cgo shim binds to keep the Go API of the reference
 * package `aeroflux` (module AeroFlex) as a drop-in:
 *
 *   aeroflux.New(cfg)      -> af_create            (aeroflux.go:176-213)
 *   (*Engine).Step()       -> af_step(e, 1)        (aeroflux.go:348-409)
 *   (*Engine).MaxDivergence-> af_max_divergence    (project.go:210-232)
 *   (*Engine).Close()      -> af_close/af_destroy  (aeroflux.go:419-439)
 *   Mesh.Data(&f) views    -> af_field_download / af_field_upload in the
 *                             padded MAC layout of grid.go:79-134
 *
 * Conventions
 *   - Every function returns AF_OK (0) or a negative af_status.  No C++
 *     exception crosses the ABI.  af_last_error(e) returns the message of the
 *     engine's last failure; af_create reports into the caller's buffer.
 *   - Messages reproduce the reference's Go error text, "aeroflux: ..." prefix
 *     included.
 *   - The engine owns all device memory.  Fields live in one device
 *     allocation laid out exactly like the reference's arena (grid.go:101-134:
 *     P, U, V, W, Div, Tmp0, Tmp1, Tmp2, each rounded up to 128 bytes, x unit
 *     stride, SY = padded nx, SZ = padded nx*ny).
 *   - One engine is driven by one host thread at a time; it owns one CUDA
 *     stream.  Calls are synchronous: they return once the device work they
 *     enqueue has finished.  Results are bit-identical run to run.
 */
#ifndef AEROFLUX_CUDA_H
#define AEROFLUX_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AF_ABI_VERSION 1

typedef enum af_status {
    AF_OK = 0,
    AF_ERR_CONFIG = -1,      /* Normalize rejected the configuration */
    AF_ERR_CUDA = -2,        /* CUDA runtime failure or no usable device */
    AF_ERR_FAULT = -3,       /* contained fault: the device-side analogue of the
                                reference's guard-page fault (a NaN backtrace
                                coordinate driving an index out of range) */
    AF_ERR_ARG = -4,         /* bad argument: NULL, unknown field, wrong count */
    AF_ERR_UNSUPPORTED = -5, /* feature not available (the Darwin direct solver) */
    AF_ERR_CLOSED = -6,      /* engine already closed */
    AF_ERR_NOMEM = -7        /* device or host allocation failed */
} af_status;

/* Arithmetic form of the step.  AF_PRECISION_FP64 is the reference's
 * algorithm in binary64 with bit-identical results; AF_PRECISION_MIXED runs
 * advection, diffusion and the inner pressure sweeps in binary32 inside
 * binary64 iterative refinement. */
typedef enum af_precision {
    AF_PRECISION_FP64 = 0,
    AF_PRECISION_MIXED = 1
} af_precision;

/* Config, aeroflux.go:14-41.  Go ints are 64-bit.  Fields after `lock` are
 * GB300 extensions; zero selects the reference's behaviour. */
typedef struct af_config {
    int64_t nx, ny, nz;          /* interior cell counts */
    int64_t ghost;               /* halo thickness, default 1 */
    double h;                    /* cell size, default 1/max(nx,ny,nz) */
    double viscosity;            /* kinematic viscosity nu */
    double density;              /* rho, default 1 */
    double dt;                   /* fixed timestep, default from Normalize */
    int64_t workers;             /* accepted and normalized like the reference;
                                    results never depend on it */
    int64_t gauss_seidel_iters;  /* red-black sweep pairs per projection, default 24 */
    int32_t use_sparse_solver;   /* the Darwin direct solver: never available */
    int32_t lock;                /* residency request: device memory is always resident */
    /* --- extensions --- */
    int32_t precision;           /* af_precision */
    int32_t device;              /* CUDA device ordinal the engine lives on */
    double div_tol;              /* MIXED: stop refining once max|div| <= div_tol (0: 1e-10) */
    int64_t inner_sweeps;        /* MIXED: red-black smoothing pairs per level before and after
                                    each coarse correction (0: 2) */
    int64_t max_refine;          /* MIXED: cap on refinement passes per projection (0: 30) */
} af_config;

/* Field, grid.go:12-21.  off is the byte offset inside the engine arena. */
typedef struct af_field_desc {
    int64_t off, nx, ny, nz, sy, sz, count;
} af_field_desc;

/* Field ids in arena order, grid.go:60-67. */
typedef enum af_field {
    AF_FIELD_P = 0,
    AF_FIELD_U = 1,
    AF_FIELD_V = 2,
    AF_FIELD_W = 3,
    AF_FIELD_DIV = 4,
    AF_FIELD_TMP0 = 5,
    AF_FIELD_TMP1 = 6,
    AF_FIELD_TMP2 = 7
} af_field;

typedef struct af_engine af_engine;

/* Debug build only (no counterpart in the reference): libaeroflux_cuda_debug,
 * built with AEROFLUX_DEBUG_BOUNDS=1, checks every device load and store of
 * the kernels against the buffer it addresses and, instead of faulting,
 * records the first violation -- (kernel id << 56) | (slot << 40) | element
 * offset (40-bit two's complement) -- and counts them; the next synchronising
 * call then fails with AF_ERR_CUDA and the location in its error text.  This
 * reads (and with reset != 0 clears) the record: *enabled is 1 in the debug
 * build and 0 in the product build, which records nothing. */
int af_debug_bounds(int32_t* enabled, uint64_t* first, uint32_t* violations, int32_t reset);

/* Library ABI version (AF_ABI_VERSION of the build). */
int af_abi_version(void);

/* (*Config).Normalize, aeroflux.go:47-113: fills defaults in place and
 * validates.  On rejection returns AF_ERR_CONFIG and writes the reference's
 * message into err (if non-NULL). */
int af_config_normalize(af_config* cfg, char* err, size_t errlen);

/* MACBytes, grid.go:138-144: arena footprint in bytes, 0 for invalid extents. */
int64_t af_mac_bytes(int64_t nx, int64_t ny, int64_t nz, int64_t ghost);

/* New, aeroflux.go:176-213: normalize, allocate the device arena, zero every
 * field (grid.go:158-163).  *out is NULL on failure and err holds the text. */
int af_create(const af_config* cfg, af_engine** out, char* err, size_t errlen);

/* Engine.Cfg after Normalize. */
int af_get_config(const af_engine* e, af_config* out);

/* Current descriptor of a field.  Descriptors swap during a step
 * (commitVelocity, stencil.go:230-235) and return to their slots after every
 * complete step. */
int af_field_info(const af_engine* e, int field, af_field_desc* out);

/* Mesh.Data(&f) (grid.go:147-149) as explicit copies of the whole padded
 * field: count must equal the descriptor's count. */
int af_field_upload(af_engine* e, int field, const double* host, size_t count);
int af_field_download(af_engine* e, int field, double* host, size_t count);

/* applyVelocityBC, stencil.go:246-315 (callers seed, then apply the BC). */
int af_apply_velocity_bc(af_engine* e);

/* Step, aeroflux.go:348-409, nsteps times.  Stops at the first step that
 * contains a fault and returns AF_ERR_FAULT with the reference's message
 * ("aeroflux: guard-page fault contained: runtime error: ..."); the state is
 * then partly advanced, as in the reference. */
int af_step(af_engine* e, int64_t nsteps);

/* project, project.go:12-34 (the reference's tests call it directly). */
int af_project(af_engine* e);

/* Diagnostics: MaxDivergence (project.go:210-232, exact), KineticEnergy
 * (project.go:238-258, fixed-order tree sum), MaxVelocity and CFL
 * (stencil.go:319-338, exact). */
int af_max_divergence(af_engine* e, double* out);
int af_kinetic_energy(af_engine* e, double* out);
int af_max_velocity(af_engine* e, double* out);
int af_cfl(af_engine* e, double* out);

/* EnableSparseSolver (sparse_fallback.go:17-19 on non-Darwin): always
 * AF_ERR_UNSUPPORTED with the reference's fallback message. */
int af_enable_sparse_solver(af_engine* e);

/* The GPU analogue of EnableSparseSolver on Darwin (sparse_darwin.go:26-132,
 * used by project.go:19-27): from the next projection on, the FP64 engine
 * solves the pressure Poisson problem to max|div| <= div_tol (0 selects
 * 1e-12, "exact projection") by binary64 iterative refinement around
 * binary32 multigrid V-cycles instead of GaussSeidelIters red-black sweeps;
 * where the binary64 residual's round-off floor (about |h^2*Div| * 2^-53,
 * scaled by dt/(rho h^2)) lies above div_tol, refinement stops at the floor
 * (a pass that removes less than a tenth of max|r|).
 * The sweeps stay bit-identical to the reference; P is the refined solution
 * (its additive constant differs from the pinned-cell Cholesky solution,
 * which the gradient does not see).  Idempotent like EnableSparseSolver;
 * AF_ERR_UNSUPPORTED for the mixed-precision form (which already projects
 * this way).  af_last_projection_stats reports its passes. */
int af_enable_multigrid_solver(af_engine* e, double div_tol);

/* Advection scheme of the FP64 form's sweeps.  SEMI_LAGRANGIAN is the
 * reference's (stencil.go:44-119), bit-exact.  MACCORMACK is the higher-order
 * form the reference names as the remedy for its numerical dissipation
 * (README "Known limitations"): per axis sweep the reference's
 * semi-Lagrangian step, a backward trace through its result, the
 * error-compensating correction limited to the range of the sampled source
 * values (Selle et al. 2008), then the reference's directional diffusion.
 * Two launches per sweep and three extra face fields of device memory.
 * AF_ERR_UNSUPPORTED for MACCORMACK in the mixed-precision form. */
typedef enum af_advection {
    AF_ADVECTION_SEMI_LAGRANGIAN = 0,
    AF_ADVECTION_MACCORMACK = 1
} af_advection;
int af_set_advection(af_engine* e, int scheme);

/* Phase hooks, one reference phase each, for stage-level parity tests:
 * dispatch(sweepFn)+commitVelocity for one axis (0=x,1=y,2=z) at dt
 * (stencil.go:21-25,230-235), computeDivergence (project.go:42-62),
 * solvePressureRedBlack (project.go:73-100), applyPressureBC
 * (project.go:139-163), subtractGradient (project.go:172-205). */
int af_phase_sweep(af_engine* e, int axis, double dt);
int af_phase_divergence(af_engine* e);
int af_phase_red_black(af_engine* e);
int af_phase_pressure_bc(af_engine* e);
int af_phase_subtract_gradient(af_engine* e);

/* Statistics of the last projection of a MIXED engine: refinement passes
 * and the FP64 max|div| reached.  FP64 engines report 0 passes. */
int af_last_projection_stats(af_engine* e, int64_t* passes, double* max_div);
/* Multigrid V-cycles the last refined projection ran in total (its passes
 * run up to four each, fewer when the measured reduction predicts them
 * enough); 0 for the red-black form. */
int af_last_projection_vcycles(af_engine* e, int64_t* vcycles);

/* Device-time profile of the last Step, from event nodes the step graph
 * carries while profiling is on (af_profile).  No counterpart in the
 * reference, which reports only wall-clock Mcell/s (bench_test.go:26-32). */
typedef struct af_step_profile {
    double step_ms;           /* whole step */
    double sweep_ms;          /* the six advection/diffusion sweeps (BC passes excluded) */
    double rbgs_ms;           /* FP64: the red-black sweeps of both projections;
                                 MIXED: both projections (refinement included) */
    int64_t rbgs_launches;    /* FP64: red-black kernel launches per step */
    int64_t kernel_launches;  /* kernel launches per step */
} af_step_profile;

/* Turns event-node profiling of the step graph on or off (rebuilds it). */
int af_profile(af_engine* e, int enable);
int af_last_step_profile(af_engine* e, af_step_profile* out);

/* Self-test of the red-black update's correctly rounded x/6 (the integer
 * form the kernel uses and the FMA-remainder form) against IEEE division on
 * n random binary64 bit patterns from `seed`; *mismatches counts differing
 * results (NaN compared by NaN-ness). */
int af_selftest_div6(int device, int64_t n, uint64_t seed, int64_t* mismatches);

/* Self-test of the integer-pipe binary64 add/subtract the red-black update
 * uses against the native ones, on n pairs built from `seed` (random bit
 * patterns, cancellations, exact ties, far exponents). */
int af_selftest_dadd(int device, int64_t n, uint64_t seed, int64_t* mismatches);

/* Measures the device's binary64 FMA issue rate (independent DFMA chains),
 * in FMA instructions per second, for the FP64 roofline. */
int af_device_fp64_rate(int device, double* fma_per_s);

/* ---------------------------------------------------------------------------
 * Batched and served form (no counterpart in the reference, which steps one
 * grid per Engine): many MIXED-precision grids of uneven sizes in one batch.
 * Every stage of a step is one persistent launch over device-side work lists
 * covering all active slots, and the whole step is one CUDA graph with one
 * refinement loop for the batch.  A slot computes the same bits alone (an
 * af_create'd MIXED engine) and in any batch, under any tuning.  Slots can be
 * assigned, released, activated and deactivated between steps without
 * recapturing the graph, which is what continuous batching needs.
 * ------------------------------------------------------------------------- */
typedef struct af_batch af_batch;

/* capacity slots on `device`; pool_bytes > 0 reserves one device pool of
 * that size for all slot memory (the admission budget), 0 allocates per slot. */
int af_batch_create(int64_t capacity, int64_t pool_bytes, int32_t device, af_batch** out, char* err, size_t errlen);
/* Device bytes a slot with this config needs (after Normalize). */
int af_batch_slot_bytes(const af_config* cfg, int64_t* bytes);
/* Normalizes cfg (precision must be AF_PRECISION_MIXED) into a free slot;
 * AF_ERR_NOMEM when the pool or the slots are exhausted.  Fields start zero. */
int af_batch_assign(af_batch* b, const af_config* cfg, int64_t* slot);
int af_batch_release(af_batch* b, int64_t slot);
int af_batch_set_active(af_batch* b, int64_t slot, int active);
int af_batch_get_config(const af_batch* b, int64_t slot, af_config* out);
int af_batch_field_info(const af_batch* b, int64_t slot, int field, af_field_desc* out);
int af_batch_field_upload(af_batch* b, int64_t slot, int field, const double* host, size_t count);
int af_batch_field_download(af_batch* b, int64_t slot, int field, double* host, size_t count);
/* applyVelocityBC of every active slot. */
int af_batch_apply_velocity_bc(af_batch* b);
/* nsteps Steps of every active slot.  Returns AF_OK when the batch ran,
 * also if some slots faulted: query them with af_batch_slot_status. */
int af_batch_step(af_batch* b, int64_t nsteps);
/* faulted = 1 and the reference's message when the slot's last step faulted. */
int af_batch_slot_status(af_batch* b, int64_t slot, int32_t* faulted, char* msg, size_t msglen);
int af_batch_max_divergence(af_batch* b, int64_t slot, double* out);
int af_batch_projection_stats(af_batch* b, int64_t slot, int64_t* passes, double* max_div);
/* Autotuner: times candidate launch shapes of every stage on the current
 * slots (run before uploading fields or between steps) and keeps the
 * fastest; writes a JSON report, per stage "stage_<n>": {"tpb", "ept",
 * "blocks_per_sm", "variant", "us"}, and for the fused red-black pair
 * stages also "variants_us": every tile variant's time.  Results are
 * bit-identical under any shape or variant. */
int af_batch_tune(af_batch* b, int32_t reps, char* report, size_t len);
int af_batch_profile(af_batch* b, int enable);
int af_batch_last_step_profile(af_batch* b, af_step_profile* out);
/* Writes a slot's initial field on the device: the Taylor-Green vortex of
 * amplitude amp (binary32 sinpi/cospi) plus uniform [-noise, noise] from
 * PCG32(seed, stream) in af_seed_taylor_green's draw order; apply the
 * velocity BC afterwards. */
int af_batch_seed(af_batch* b, int64_t slot, double amp, double noise, uint64_t seed, uint64_t stream);
void af_batch_destroy(af_batch* b);
const char* af_batch_last_error(const af_batch* b);

/* ---------------------------------------------------------------------------
 * Serving: a continuous-batching request loop over a batch (no counterpart
 * in the reference).  Requests queue in arrival order; each round admits
 * queued requests while a slot and enough of the device budget are free
 * (state created by af_batch_seed and kept resident), advances every
 * resident request by the same number of Steps (at most max_round_steps) in
 * one batched graph launch, and retires finished requests with their
 * max|div| read back.  A request's bits do not depend on what else is
 * resident.  retain != 0 keeps finished requests resident (inactive) until
 * af_server_release so their fields can be downloaded.
 * ------------------------------------------------------------------------- */
typedef struct af_server af_server;

typedef struct af_request_result {
    int64_t id;
    int32_t status;            /* AF_OK or AF_ERR_FAULT */
    int32_t reserved;
    int64_t cells;             /* interior cells */
    int64_t steps;             /* Steps performed */
    int64_t refinement_passes; /* of the last projection */
    double arrival_s, admitted_s, completed_s;  /* server clock */
    double max_divergence;     /* MaxDivergence of the result */
} af_request_result;

typedef struct af_server_stats {
    int64_t queued, resident, retained;
    int64_t budget_bytes, used_bytes;
    int64_t executed_cell_steps;
    double now_s;
} af_server_stats;

/* max_resident_cells > 0 also caps the interior cells resident at once (the
 * work one round advances), so under overload requests finish instead of all
 * crawling; one request is always admitted when none is running. */
int af_server_create(int64_t budget_bytes, int64_t max_slots, int64_t max_resident_cells, int32_t device,
                     int32_t max_round_steps, int32_t retain, af_server** out, char* err, size_t errlen);
/* Seconds since creation (the clock of arrival/admission/completion times). */
int af_server_now(af_server* s, double* seconds);
/* cfg must be MIXED; arrival_s < 0 stamps the current time. */
int af_server_submit(af_server* s, const af_config* cfg, int64_t steps, uint64_t seed, double arrival_s, int64_t* id);
int af_server_round(af_server* s, int64_t* completed_now, int64_t* resident, int64_t* queued);
/* Moves up to cap finished requests' results out; *n gets how many. */
int af_server_results(af_server* s, af_request_result* out, int64_t cap, int64_t* n);
int af_server_download(af_server* s, int64_t id, int field, double* host, size_t count);
int af_server_release(af_server* s, int64_t id);
/* Drops every request not yet admitted (resident ones keep stepping);
 * *cancelled gets how many. */
int af_server_cancel_queued(af_server* s, int64_t* cancelled);
int af_server_get_stats(af_server* s, af_server_stats* out);
/* The batch autotuner on the requests currently resident. */
int af_server_tune(af_server* s, int32_t reps, char* report, size_t len);
void af_server_destroy(af_server* s);
const char* af_server_last_error(const af_server* s);

/* Synthetic input (no counterpart in the reference API; its tests seed a
 * trigonometric field straight into arena views, engine_test.go:302-335).
 * Fills host arrays u, v, w -- the padded counts of U, V, W for the
 * normalized cfg -- with a Taylor-Green vortex of amplitude amp sampled at the
 * staggered faces plus i.i.d. uniform [-noise, noise] from PCG32 (initstate
 * seed, stream `stream`), over seedVortex's index ranges and in its field and
 * loop order; every other element is zero.  Apply the velocity BC after
 * uploading. */
int af_seed_taylor_green(const af_config* cfg, double amp, double noise, uint64_t seed, uint64_t stream,
                         double* u, double* v, double* w);

/* KineticEnergy of caller-owned device fields, allocating nothing.  No
 * counterpart in the reference.  For callers that cannot allocate device
 * memory while they run (hosts that hand all device memory to their own pool
 * up front, loops that cannot afford cudaMalloc/cudaFree's implicit device
 * synchronisation).  u, v, w are device pointers to the padded U, V, W fields
 * of the MAC layout described by cfg (nx, ny, nz, ghost, h; other fields
 * unused) on the current device; the sum is the fixed-order tree of
 * af_kinetic_energy.  Its scratch is a static 128 KiB device array held by
 * every GPU that loads the library until exit, so nz is limited to 16384
 * z-planes, and nx, ny and ghost to below 2^20 (larger grids are rejected
 * with AF_ERR_ARG and a message in err).  The first call on a device
 * resolves the array's address there (a one-time set-up); make that first
 * call before any stream capture.  The call is synchronous: it enqueues on
 * `stream` (a cudaStream_t, NULL for the default stream), waits for that
 * stream and copies the result to *out (host), so it must not be made while
 * `stream` is being captured.  All calls share the one array: calls that
 * overlap on the GPU race. */
int af_kinetic_energy_noalloc(const af_config* cfg, const double* u, const double* v, const double* w,
                              void* stream, double* out, char* err, size_t errlen);

/* The same synthetic field written on the device (no counterpart in the
 * reference): Taylor-Green of amplitude amp with binary32 sinpi/cospi plus
 * uniform [-noise, noise] from PCG32(seed, stream) in af_seed_taylor_green's
 * draw order; U, V, W and Tmp0-2 are zeroed first.  Apply the BC after. */
int af_seed_device(af_engine* e, double amp, double noise, uint64_t seed, uint64_t stream);

/* Close, aeroflux.go:419-439: release device memory.  Idempotent. */
int af_close(af_engine* e);
/* Close (if needed) and free the handle.  Safe on NULL. */
void af_destroy(af_engine* e);

/* Message of the engine's last failure ("" when none). */
const char* af_last_error(const af_engine* e);

#ifdef __cplusplus
}
#endif
#endif /* AEROFLUX_CUDA_H */
