// sph_cubic.cu -- cubic-spline SPH (filled in below).
#include "internal.cuh"

int sf_sph_cubic_alloc(sfgpu_sim* s) {
    (void)s;
    sf_set_error("cubic-spline SPH is not available in this build");
    return SFGPU_FAILURE;
}
void sf_sph_cubic_free(sfgpu_sim* s) { (void)s; }
int sf_sph_cubic(sfgpu_sim* s) {
    (void)s;
    sf_set_error("cubic-spline SPH is not available in this build");
    return SFGPU_FAILURE;
}
