// af_mixed.cu -- mixed-precision form.  Placeholder until the form lands.
#include "af_mixed.h"

namespace af {

struct MixedState {};

MixedState* mixed_create(const Geom&, const af_config&, cudaStream_t, std::string* err) {
    *err = "aeroflux: mixed precision form is not available in this build";
    return nullptr;
}
void mixed_destroy(MixedState* m) { delete m; }
void launch_sweep_mixed(MixedState*, const Geom&, int, const Fields&, double, double, double, Status*, int,
                        cudaStream_t) {}
void enqueue_project_mixed(MixedState*, const Geom&, const af_config&, const Fields&, Status*, int, cudaStream_t) {}
void mixed_stats(MixedState*, int64_t* passes, double* max_div) {
    *passes = 0;
    *max_div = 0;
}

}  // namespace af
