/*
 * starflood_compat.h -- the reference's own function surface, implemented by
 * libsfgpu.so on the GPU.  A program written against Starflood's headers
 * (src/simulation.h, src/tree.h, src/gravity.h, src/sph.h) links against
 * libsfgpu.so instead of the reference objects and runs unchanged; this
 * header restates the same declarations for programs built without them.
 *
 * ABI (FP32 build of the reference, ENABLE_TREE defined as shipped):
 *   real = float, uint = uint32_t, node_t 80 bytes, tree_t, sim_t below.
 * The slab mem holds N * SIM_DOF reals (13, or 16 with SPH) in the order of
 * enum sim_conf; the library keeps an HBM copy per sim_t, keyed by mem.
 *
 * The reference fixes dt, eps, G, theta, the solver and SPH at compile time
 * (src/config.h); here they are run-time parameters set with
 * sfgpu_compat_configure() before sim_init (defaults: the shipped config.h).
 * Every call uploads what it reads and downloads what it writes, so host
 * arrays are current after each call, as with the reference.
 */
#ifndef STARFLOOD_COMPAT_H
#define STARFLOOD_COMPAT_H

#include <stdint.h>

#include "sfgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef STARFLOOD_COMPAT_NO_TYPES
typedef float real;  /* src/types.h:19-23 (FP32 build) */

/* src/simulation.h:17-51 */
enum sim_conf {
    _SIM_POS_0, _SIM_POS_1, _SIM_POS_2,
    _SIM_VEL_0, _SIM_VEL_1, _SIM_VEL_2,
    _SIM_ACC_0, _SIM_ACC_1, _SIM_ACC_2,
    SIM_MAS, SIM_POT, SIM_KEN, SIM_PEN,
    SIM_RAD, SIM_RHO, SIM_PRS,   /* present when SPH is enabled */
    SIM_POS = _SIM_POS_0, SIM_VEL = _SIM_VEL_0, SIM_ACC = _SIM_ACC_0
};

/* src/tree.h:16-25 */
typedef struct {
    uint32_t parent;
    uint32_t bodies;
    uint32_t branch[8];
    real bounds[6];
    real params[4];
} node_t;

/* src/tree.h:28-35 */
typedef struct {
    uint32_t max_nodes;
    uint32_t num_nodes;
    real bounds[6];
    node_t* node;
} tree_t;

/* src/simulation.h:53-67 (ENABLE_TREE defined, ENABLE_GRID not) */
typedef struct {
    unsigned int step_number;
    unsigned int N;
    void* mem;
    tree_t tree;
} sim_t;
#endif

/* Parameters used by every entry point below (process-wide). */
int sfgpu_compat_configure(const sfgpu_params* p);
void sfgpu_compat_params(sfgpu_params* out);
/* The device simulation behind a sim_t (NULL if none). */
sfgpu_sim* sfgpu_compat_handle(const sim_t* sim);
/* Copy the device state behind sim (ahead of sim->mem after resident calls
 * such as sfgpu_run on sfgpu_compat_handle(sim)) into sim->mem; 0 or -1. */
int sfgpu_sync_host(sim_t* sim);

/* src/simulation.c:33-53 */
real* sim_find(const sim_t* sim, enum sim_conf parameter);
/* src/simulation.c:55-187 */
int sim_init(sim_t* sim, unsigned int N);
/* src/simulation.c:189-228 */
int sim_free(sim_t* sim);
/* src/initcond.c:11-255: the reference's default initial conditions,
 * generated on the GPU; the host arrays are current on return. */
int initcond_generate(sim_t* sim);

/* src/visualization.h:10-27 */
typedef enum { IMAGE_FILETYPE_PFM, IMAGE_FILETYPE_PPM, IMAGE_FILETYPE_PNG, NUM_IMAGE_FILETYPE } image_filetype_t;
typedef struct {
    unsigned int sizex, sizey;
    void* mem;
    int32_t* atomic_buffer;
    float* render_buffer;
    void* binary_buffer;
} vis_t;
/* src/visualization.c:34-176 (plus device buffers for the GPU draw) */
int vis_init(vis_t* vis, unsigned int sizex, unsigned int sizey);
/* src/visualization.c:178-238 */
int vis_free(vis_t* vis);
/* src/visualization_io.c:170-330: PFM and PPM (PNG needs stb_image_write:
 * reported, as a reference build without ENABLE_STB_IMAGE_WRITE does). */
int vis_save(const vis_t* vis, const char* filename, image_filetype_t filetype);
/* src/visualization.c:258-740 on the GPU; buffers current on return. */
int vis_draw(const vis_t* vis, const sim_t* sim);

/* src/grid.h:11-24 as built with ENABLE_FFT.  mem: side^3 FP32 samples, then
 * side^3 int32 deposit counts; mem_fft0: the device grid (opaque);
 * mem_fft1, mem_fft2: unused (NULL). */
typedef struct {
    unsigned int dim[3];
    real bounds_min[3];
    real bounds_max[3];
    void* mem;
    void* mem_fft0;
    void* mem_fft1;
    void* mem_fft2;
} grid_t;
/* src/grid.c:26-159 (side 1..256, else -1); G from sfgpu_compat_configure */
int grid_init(grid_t* grid, unsigned int side_length, const real* bounds_min, const real* bounds_max);
/* src/grid.c:161-188 */
int grid_free(grid_t* grid);
/* src/grid.c:190-194 */
real* grid_samp(const grid_t* grid);
/* src/grid.c:197-536 on the GPU (cuFFT); grid_samp() current on return. */
int grid_solve_fft(const grid_t* grid);
/* src/gravity.c:116-238: deposit of the bodies' positions (128 jittered
 * samples each, seeded by sim->step_number) into the counts and samples,
 * then grid_solve_fft.  The reference compiles this function out and reads
 * the grid from sim_t (ENABLE_GRID); this sim_t has no grid member, so the
 * grid is an argument. */
int solve_gravity_part_mesh(const sim_t* sim, grid_t* grid);

/* src/simulation_io.c:16-79: the slab (N*SIM_DOF reals, no header) from a
 * file into sim->mem and the device; like the reference, a short read is
 * reported on stderr but not failed. */
int sim_read_raw(sim_t* sim, const char* filename);
/* src/simulation_io.c:81-149: sim->mem (current after every call) to a file. */
int sim_save_raw(const sim_t* sim, const char* filename);
/* src/simulation.c:230-345 (without SOLVER_VIS) */
int sim_solv(sim_t* sim);
/* src/simulation.c:347-519 (without SOLVER_VIS) */
int sim_step(sim_t* sim);
/* src/simulation.h:90-95, the SOLVER_VIS signatures; the render buffer is
 * ignored (tree-walk debug drawing is not part of this library). */
int sim_solv_vis(sim_t* sim, float* render_buffer, unsigned int sizex, unsigned int sizey);
int sim_step_vis(sim_t* sim, float* render_buffer, unsigned int sizex, unsigned int sizey);
/* src/tree.c:14-55 */
int tree_init(tree_t* tree, unsigned int max_nodes);
/* src/tree.c:57-72 */
int tree_free(tree_t* tree);
/* src/tree.c:74-318: builds on the GPU and writes the node_t array in the
 * reference's numbering; returns -1 on node or depth overflow. */
int tree_build(tree_t* tree, unsigned int num_parts, const real* pos, const real* mas);
/* src/gravity.c:242-663 */
int solve_gravity_part_tree(const sim_t* sim);
/* src/gravity.c:666-819 */
int solve_gravity_part_part(const sim_t* sim);
/* src/sph.c:14-282 */
int solve_sph(const sim_t* sim);

#ifdef __cplusplus
}
#endif
#endif
