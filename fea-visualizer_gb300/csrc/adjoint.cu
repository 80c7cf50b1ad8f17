// adjoint.cu -- hand-written adjoint of the explicit advection-diffusion step.
#include "fea_internal.cuh"

extern "C" int fea_adjoint_advdiff(fea_solver*, const float*, const float*, int64_t, int64_t, double*, float*,
                                   float*) {
    return fea::fail(FEA_ERR_UNSUPPORTED, "adjoint not built yet");
}
extern "C" int fea_adjoint_advdiff_device(fea_solver*, const void*, const void*, int64_t, int64_t, double*, void*,
                                          void*) {
    return fea::fail(FEA_ERR_UNSUPPORTED, "adjoint not built yet");
}
