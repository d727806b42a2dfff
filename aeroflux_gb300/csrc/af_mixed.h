// af_mixed.h -- mixed-precision form (binary32 sweeps inside binary64
// iterative refinement).  Internal to libaeroflux_cuda.
#pragma once

#include "../../include/aeroflux_cuda.h"
#include "af_internal.h"

#include <string>

namespace af {

struct MixedState;

MixedState* mixed_create(const Geom& g, const af_config& c, cudaStream_t s, std::string* err);
void mixed_destroy(MixedState* m);
void launch_sweep_mixed(MixedState* m, const Geom& g, int axis, const Fields& f, double dt, double invH, double lam,
                        Status* st, int phase, cudaStream_t s);
void enqueue_project_mixed(MixedState* m, const Geom& g, const af_config& c, const Fields& f, Status* st, int gate,
                           cudaStream_t s);
void mixed_stats(MixedState* m, int64_t* passes, double* max_div);
// First CUDA error met while capturing the refinement loop (then cleared).
cudaError_t mixed_capture_error(MixedState* m);

}  // namespace af
