// af_batch.h -- batched mixed-precision engine: many independent grids of
// uneven sizes stepping together, one persistent launch per stage and one
// CUDA graph per step.  The single-grid mixed engine is a batch of one, so a
// grid computes the same bits alone and in a batch.  Internal to
// libaeroflux_cuda.
#pragma once

#include "../../include/aeroflux_cuda.h"
#include "af_internal.h"

#include <string>
#include <vector>

namespace af {

struct Batch;

// Creates an empty batch with `capacity` slots on the current device.
// pool_bytes > 0 reserves one device pool of that size for the slots' memory
// (the admission budget); 0 allocates each slot separately.
Batch* batch_create(int capacity, size_t pool_bytes, std::string* err);
void batch_destroy(Batch* b);

// Bytes of device memory one slot needs for a normalized MIXED config.
size_t batch_slot_bytes(const af_config& c);
// Whether a normalized config fits the 32-bit index arithmetic of a slot
// (face box < 2^32, each field and the velocity-BC write set < 2^31
// elements); otherwise false with the message in *err.  Host only.
bool batch_config_fits(const af_config& c, std::string* err);

// Puts a normalized MIXED config into a free slot.  `arena`, when non-NULL,
// is external field memory in the reference layout (the single-grid engine);
// otherwise the arena comes from the pool.  Returns the slot or -1.
int batch_assign(Batch* b, const af_config& c, char* arena, std::string* err);
void batch_release(Batch* b, int slot);
// Whether a slot steps (inactive slots keep their memory and state).
void batch_set_active(Batch* b, int slot, bool active);

// Field descriptor and device pointer of a slot's field (after swaps).
af_field_desc batch_field(const Batch* b, int slot, int field, double** dev);
const Geom& batch_geom(const Batch* b, int slot);

cudaStream_t batch_stream(Batch* b);

// Enqueues one Step of every active slot on the batch stream (graph
// replay); `nsteps` replays.  stop_at (optional, indexed by slot) limits a
// slot to its first stop_at[s] of them (0 or >= nsteps: all); the slot's
// later Steps are skipped by every kernel.  Returns a cudaError_t of the
// launch.
cudaError_t batch_step(Batch* b, int64_t nsteps, std::string* err, const std::vector<int64_t>* stop_at = nullptr);
// One projection (project.go:12-34) of every active slot, as a graph.
cudaError_t batch_project(Batch* b, std::string* err);
// A projection inside a caller's own graph (the FP64 engine's multigrid
// option): prepare before the caller begins capturing; enqueue on the
// caller's capturing stream with the caller's field parity and fault gate
// (returns the kernel launches it added); after capture, check the error the
// enqueue may have recorded.  Faults go to batch_status(b, slot).
cudaError_t batch_prepare_capture(Batch* b);
int64_t batch_enqueue_project(Batch* b, int parity, int gate, cudaStream_t s);
cudaError_t batch_capture_error(Batch* b);
Status* batch_status(Batch* b, int slot);
// applyVelocityBC of every active slot.
cudaError_t batch_velocity_bc(Batch* b);
// One sweep (dispatch + commit) of every active slot.
cudaError_t batch_sweep(Batch* b, int axis, double dt);

// Writes the seeded Taylor-Green + PCG32 noise initial field of a slot on
// the device (U, V, W zeroed first); apply the velocity BC afterwards.
cudaError_t batch_seed(Batch* b, int slot, double amp, double noise, uint64_t seed, uint64_t stream);

// Reads every slot's status after the enqueued work: returns the number of
// slots that faulted in it; `msg` gets the first faulting slot's message.
int batch_collect_faults(Batch* b, std::string* msg, int* first_slot);
bool batch_slot_faulted(const Batch* b, int slot, std::string* msg);
// Whether a kernel of the enqueued work gave up a bounded wait (the work's
// results are then invalid); clears the record and sets *msg.
bool batch_device_error(Batch* b, std::string* msg);
// Refinement passes, estimated max|div| and multigrid V-cycles of the slot's
// last projection.
void batch_slot_projection(Batch* b, int slot, int64_t* passes, double* max_div, int64_t* vcycles = nullptr);

// Times the candidate launch shapes of every stage on the current slots and
// keeps the fastest; returns a JSON report.  Results do not depend on it.
std::string batch_tune(Batch* b, int reps);

// Turns on event timing of the step (whole step, sweeps, projections).
cudaError_t batch_profile(Batch* b, bool on);
cudaError_t batch_last_profile(Batch* b, double* step_ms, double* sweep_ms, double* proj_ms, int64_t* launches);

}  // namespace af
