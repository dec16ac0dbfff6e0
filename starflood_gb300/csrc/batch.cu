// batch.cu -- batched and adjoint forms (filled in below).
#include "internal.cuh"

extern "C" int sfgpu_batch_create(sfgpu_batch** out, uint32_t, const uint32_t*, const sfgpu_params*) {
    if (out) *out = nullptr;
    sf_set_error("batched form is not available in this build");
    return SFGPU_FAILURE;
}
extern "C" int sfgpu_batch_destroy(sfgpu_batch*) { return SFGPU_OK; }
extern "C" int sfgpu_batch_upload(sfgpu_batch*, const float*, const float*, const float*) { return SFGPU_FAILURE; }
extern "C" int sfgpu_batch_download(sfgpu_batch*, float*, float*, float*, float*) { return SFGPU_FAILURE; }
extern "C" int sfgpu_batch_solve(sfgpu_batch*) { return SFGPU_FAILURE; }
extern "C" int sfgpu_batch_run(sfgpu_batch*, uint32_t) { return SFGPU_FAILURE; }
extern "C" int sfgpu_batch_autotune(sfgpu_batch*, int*) { return SFGPU_FAILURE; }
extern "C" int sfgpu_batch_synchronize(sfgpu_batch*) { return SFGPU_FAILURE; }
extern "C" void* sfgpu_batch_stream(sfgpu_batch*) { return nullptr; }
extern "C" int sfgpu_batch_grad(sfgpu_batch*, uint32_t, uint32_t, float*, float*, double*) { return SFGPU_FAILURE; }
extern "C" int sfgpu_batch_force_vjp(sfgpu_batch*, const float*, float*) { return SFGPU_FAILURE; }
