// sph.cu -- SPH stage (filled in below).
#include "internal.cuh"

int sf_sph_alloc(sfgpu_sim* s) {
    (void)s;
    return SFGPU_OK;
}
void sf_sph_free(sfgpu_sim* s) { (void)s; }
int sf_stage_sph(sfgpu_sim* s) {
    (void)s;
    sf_set_error("SPH is not available in this build");
    return SFGPU_FAILURE;
}
