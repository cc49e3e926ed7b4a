// Host side of the GPU-program scheme (MAWEFD{cart,spher}{2D,3D}gpu.cu).
#include "awe_internal.h"
#include "plan_impl.h"

namespace awe {

awe_status planA_init(awe_plan *) {
    set_error("scheme of the GPU programs not built yet");
    return AWE_ERR_UNSUPPORTED;
}
awe_status planA_model(awe_plan *, const float *, const float *) { return AWE_ERR_UNSUPPORTED; }
awe_status planA_run(awe_plan *, const float *, int, float *, float *, cudaStream_t) { return AWE_ERR_UNSUPPORTED; }

}  // namespace awe
