/*
 * grid_host.c -- the reference's grid_t surface (src/grid.h, src/grid.c)
 * and the particle-mesh deposit of solve_gravity_part_mesh
 * (src/gravity.c:116-238) over the device grid of grid.cu.
 *
 * grid_t keeps the reference's layout as built with ENABLE_FFT (the only
 * build that has grid_solve_fft): mem holds side^3 FP32 samples followed by
 * side^3 int32 deposit counts, as the reference's 2*side^3 reals
 * (grid.c:52-54, gravity.c:131-132); mem_fft0 holds the device grid (the
 * reference's FFTW buffers have no use here); mem_fft1 and mem_fft2 are NULL.
 * Every call leaves mem current.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "starflood_compat.h"

static sfgpu_grid* grid_dev(const grid_t* grid, const char* fn) {
    if (!grid || !grid->mem || !grid->mem_fft0) {
        fprintf(stderr, "%s error: grid_t was not created by grid_init()\n", fn);
        return NULL;
    }
    return (sfgpu_grid*)grid->mem_fft0;
}

int grid_init(grid_t* grid_ptr, unsigned int side_length, const real* bounds_min, const real* bounds_max) {
    if (!grid_ptr || !bounds_min || !bounds_max) return SFGPU_FAILURE;
    /* grid.c:29-35 */
    if (1u > side_length || 256u < side_length) return SFGPU_FAILURE;
    sfgpu_params p;
    sfgpu_compat_params(&p);
    grid_t g;
    memset(&g, 0, sizeof g);
    for (int i = 0; i < 3; i++) {
        g.dim[i] = side_length;
        g.bounds_min[i] = bounds_min[i];
        g.bounds_max[i] = bounds_max[i];
    }
    const size_t cells = (size_t)side_length * side_length * side_length;
    g.mem = calloc(2u * cells, sizeof(real));
    if (!g.mem) return SFGPU_FAILURE;
    sfgpu_grid* dev = NULL;
    if (sfgpu_grid_create(&dev, side_length, bounds_min, bounds_max, p.G, NULL) != SFGPU_OK) {
        fprintf(stderr, "%s error: %s\n", "grid_init()", sfgpu_last_error());
        free(g.mem);
        return SFGPU_FAILURE;
    }
    g.mem_fft0 = dev;
    *grid_ptr = g;
    return SFGPU_OK;
}

int grid_free(grid_t* grid_ptr) {
    if (!grid_ptr) return SFGPU_FAILURE;
    sfgpu_grid_destroy((sfgpu_grid*)grid_ptr->mem_fft0);
    free(grid_ptr->mem);
    memset(grid_ptr, 0, sizeof *grid_ptr);
    return SFGPU_OK;
}

real* grid_samp(const grid_t* grid_ptr) { return grid_ptr ? (real*)grid_ptr->mem : NULL; }

int grid_solve_fft(const grid_t* grid_ptr) {
    sfgpu_grid* dev = grid_dev(grid_ptr, "grid_solve_fft()");
    if (!dev) return SFGPU_FAILURE;
    if (sfgpu_grid_upload(dev, (const float*)grid_ptr->mem) != SFGPU_OK || sfgpu_grid_solve_fft(dev) != SFGPU_OK ||
        sfgpu_grid_download(dev, (float*)grid_ptr->mem, NULL) != SFGPU_OK) {
        fprintf(stderr, "%s error: %s\n", "grid_solve_fft()", sfgpu_last_error());
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

int solve_gravity_part_mesh(const sim_t* sim, grid_t* grid_ptr) {
    sfgpu_grid* dev = grid_dev(grid_ptr, "solve_gravity_part_mesh()");
    sfgpu_sim* s = sim ? sfgpu_compat_handle(sim) : NULL;
    if (!dev) return SFGPU_FAILURE;
    if (!s) {
        fprintf(stderr, "%s error: sim_t was not created by sim_init()\n", "solve_gravity_part_mesh()");
        return SFGPU_FAILURE;
    }
    const size_t cells = (size_t)grid_ptr->dim[0] * grid_ptr->dim[1] * grid_ptr->dim[2];
    real* poten = (real*)grid_ptr->mem;
    int32_t* accum = (int32_t*)(poten + cells);
    /* the host slab is the state of record between compat calls */
    if (sfgpu_upload_arrays(s, (const float*)sim->mem, 0u, 3u) != SFGPU_OK ||
        sfgpu_grid_deposit(dev, s, sim->step_number, 128u) != SFGPU_OK ||
        sfgpu_grid_download(dev, NULL, accum) != SFGPU_OK || sfgpu_grid_solve_fft(dev) != SFGPU_OK ||
        sfgpu_grid_download(dev, poten, NULL) != SFGPU_OK) {
        fprintf(stderr, "%s error: %s\n", "solve_gravity_part_mesh()", sfgpu_last_error());
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}
