// batched.cu -- many Gray-Scott instances stepped together.
#include "fea_internal.cuh"

extern "C" {
int fea_batch_create(const fea_instance_desc*, int, int, double, int, fea_batch** out) {
    if (out) *out = nullptr;
    return fea::fail(FEA_ERR_UNSUPPORTED, "batched solver not built yet");
}
int fea_batch_destroy(fea_batch*) { return FEA_OK; }
int fea_batch_set_fields(fea_batch*, int, const float*, const float*) { return FEA_ERR_UNSUPPORTED; }
int fea_batch_get_fields(fea_batch*, int, float*, float*) { return FEA_ERR_UNSUPPORTED; }
int fea_batch_advance_time(fea_batch*, int64_t) { return FEA_ERR_UNSUPPORTED; }
int fea_batch_synchronize(fea_batch*) { return FEA_ERR_UNSUPPORTED; }
int fea_batch_get_status(fea_batch*, uint32_t*, int32_t*) { return FEA_ERR_UNSUPPORTED; }
}
