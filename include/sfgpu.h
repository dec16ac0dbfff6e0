/*
 * sfgpu.h -- C ABI of starflood_gb300: Starflood's force-and-step path
 * (particle-particle gravity, Barnes-Hut octree build and walk, SPH, and the
 * kick-drift-kick leapfrog) as hand-written CUDA kernels for one GB300
 * (sm_103a), with particle state resident in HBM across steps.
 *
 * Two layers sit on this ABI:
 *   - this file: resident-mode handles (sfgpu_sim) plus the new precision,
 *     batched and adjoint forms;
 *   - starflood_compat.h: the reference's own function surface (sim_init,
 *     sim_solv, sim_step, tree_build, solve_gravity_part_*, solve_sph over
 *     sim_t) implemented on top of this one, for drop-in replacement.
 *
 * Conventions: every int-returning call returns SFGPU_OK (0) on success and
 * SFGPU_FAILURE (-1) on failure, like the reference's STARFLOOD_SUCCESS /
 * STARFLOOD_FAILURE (src/common.h:31-32); the reason is then available from
 * sfgpu_last_error().  Arrays follow the reference slab layout
 * (src/simulation.h:17-51): one block of N*dof floats where array k starts
 * at k*N, positions / velocities / accelerations are xyz-interleaved.
 * Calls on one sfgpu_sim are not re-entrant (like the reference, whose
 * sim_* functions share global logs, src/simulation.c:24-30).
 */
#ifndef SFGPU_H
#define SFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFGPU_OK 0
#define SFGPU_FAILURE (-1)

/* Which gravity solver sim_solv runs (reference: ENABLE_TREE, config.h:38). */
enum sfgpu_solver { SFGPU_SOLVER_PP = 0, SFGPU_SOLVER_TREE = 1 };

/* SPH (reference: ENABLE_SPH, config.h:190).  REFERENCE is the reference's
 * Gaussian-kernel SPH of src/sph.c; CUBIC is the cubic-spline SPH with an
 * ideal-gas equation of state and Monaghan artificial viscosity (new form,
 * no reference counterpart). */
enum sfgpu_sph { SFGPU_SPH_OFF = 0, SFGPU_SPH_REFERENCE = 1, SFGPU_SPH_CUBIC = 2 };

/* Arithmetic of the force kernels.
 *   EXACT: the reference's FP32 expressions and order (IEEE divide and square
 *          root, Kahan sums per interaction) -- bit-identical to the
 *          reference for PP and KDK.
 *   FAST:  hardware reciprocal square root and fused multiply-adds. */
enum sfgpu_math { SFGPU_MATH_FAST = 0, SFGPU_MATH_EXACT = 1 };

/* Precision form.  PLAIN keeps the reference's FP32 state.  COMPENSATED
 * keeps FP32 pair arithmetic but accumulates forces with two-sum
 * compensation per j-tile, holds positions and velocities in FP64 for the
 * leapfrog and centre-of-mass sums in FP64. */
enum sfgpu_form { SFGPU_FORM_PLAIN = 0, SFGPU_FORM_COMPENSATED = 1 };

/* What "acc" holds.  REFERENCE: acc_i = -G m_i sum_j m_j r_ij/(r^2+eps^2)^1.5,
 * the m_i-scaled force the reference integrates as an acceleration
 * (src/gravity.c:808-811).  PHYSICAL: the acceleration itself (no m_i). */
enum sfgpu_acc { SFGPU_ACC_REFERENCE = 0, SFGPU_ACC_PHYSICAL = 1 };

typedef struct {
    double   dt;          /* TIMESTEP_SIZE (config.h:159)                   */
    double   eps;         /* EPSILON, Plummer softening (config.h:162), > 0 */
    double   G;           /* G (config.h:167)                               */
    double   theta;       /* TREE_THETA, compared with (w/d)^2 (gravity.c:448) */
    int32_t  solver;      /* enum sfgpu_solver                              */
    int32_t  sph;         /* enum sfgpu_sph                                 */
    int32_t  math;        /* enum sfgpu_math                                */
    int32_t  form;        /* enum sfgpu_form                                */
    int32_t  acc_mode;    /* enum sfgpu_acc                                 */
    uint32_t leaf_cap;    /* bodies per leaf; 8 in the reference (tree.h:20), <= 16 */
    uint32_t depth_max;   /* TREE_DEPTH_MAX (config.h:41), <= 16            */
    uint32_t nodes_max;   /* TREE_NODES_MAX (config.h:44)                   */
    double   sph_gamma;   /* CUBIC: adiabatic index                         */
    double   sph_alpha;   /* CUBIC: Monaghan viscosity alpha                */
    double   sph_beta;    /* CUBIC: Monaghan viscosity beta                 */
    uint32_t flags;       /* SFGPU_FLAG_*                                   */
    uint32_t walk_split;  /* walk variant: 0 group walk over a stack of sibling groups (default), 32 the same
                             group walk over a stack of single cells, 1 thread per body, 8 thread per body
                             and root octant, 64 32-body group walk over 8 warps */
    uint32_t sph_path;    /* SPH neighbour passes on the cell grid.  CUBIC: the 3 x 3 rows of cells
                             of side 2h around each body, each row cut to the cells the 2h sphere
                             reaches: 0 one warp per 32 sorted bodies over the union of their rows,
                             candidates staged in shared memory (default); 2 one thread per body; 1
                             one thread per body over cells of side h; 3 by warps over cells of side
                             h.  REFERENCE (FAST): 0 by warps (default), 2 one thread per body.
                             Every path adds the same terms in the same order. */
    uint32_t walk_group;  /* bodies per warp of the group walk: 0 the default (16), 8, 16 or 32 */
    uint32_t spin_limit;  /* rounds a bounded device wait (the look-backs of the sort and of the
                             node scan) spins on an unpublished word before it gives up and sets
                             SFGPU_STATUS_SPIN; 0: the default, 2^24 */
    uint32_t walk_limit;  /* rounds of a warp's tree-walk loop before it stops and sets
                             SFGPU_STATUS_WALK; 0: the default, 2^24 */
    uint32_t reserved[2];
} sfgpu_params;

/* flags */
#define SFGPU_FLAG_STATS   0x1u  /* per-particle statistics: walk interactions and opening tests,
                                    SPH neighbour-set hashes */
#define SFGPU_FLAG_TIMING  0x2u  /* record CUDA-event times per stage            */
#define SFGPU_FLAG_NOGRAPH 0x4u  /* sfgpu_run launches kernels one by one         */
#define SFGPU_FLAG_EXPORT_TREE 0x8u /* compat sim_solv/sim_step also fill sim_t.tree.node */
#define SFGPU_FLAG_VERBOSE 0x10u /* compat sim_step prints the energies like the reference */

/* Device status word bits (sfgpu_status). */
#define SFGPU_STATUS_TREE_NODES   0x01u /* node capacity exceeded (tree.c:180)   */
#define SFGPU_STATUS_TREE_DEPTH   0x02u /* depth limit exceeded  (tree.c:186)    */
#define SFGPU_STATUS_TIES         0x04u /* too many bodies exactly on cell midplanes */
#define SFGPU_STATUS_SPIN         0x08u /* a bounded device wait gave up         */
#define SFGPU_STATUS_WALK         0x10u /* walk stack or iteration bound hit     */
#define SFGPU_STATUS_SPH_CELLS    0x20u /* a body beyond the SPH cell grid's 2^20 cells per axis */

/* The reference's compiled-in defaults (src/config.h): dt=1, eps=1e-3, G=1,
 * theta=0.5, tree on, SPH off, leaf 8, depth 16, 262144 nodes; FAST math,
 * PLAIN form, REFERENCE acc. */
void sfgpu_params_default(sfgpu_params* p);

/* Number of reals per particle in the slab: 13, or 16 with SPH
 * (SIM_DOF, src/simulation.h:46). */
uint32_t sfgpu_dof(const sfgpu_params* p);

/* Message for the last failure on the calling thread ("" if none). */
const char* sfgpu_last_error(void);

/* ---- resident simulations -------------------------------------------- */
typedef struct sfgpu_sim sfgpu_sim;

/* Replaces sim_init (src/simulation.c:55-187): allocates the device slab
 * (zeroed, like the reference's memset) and every work array. */
int sfgpu_create(sfgpu_sim** out, uint32_t n, const sfgpu_params* p);
/* Replaces sim_free (src/simulation.c:189-228). */
int sfgpu_destroy(sfgpu_sim* s);

/* Copy a whole host slab (N*dof floats, reference layout) to / from HBM.
 * Synchronous with respect to the host. */
int sfgpu_upload(sfgpu_sim* s, const float* slab);
int sfgpu_download(sfgpu_sim* s, float* slab);
/* Copy only arrays [first, first+count) of the slab (count*N floats). */
int sfgpu_upload_arrays(sfgpu_sim* s, const float* slab, uint32_t first, uint32_t count);
int sfgpu_download_arrays(sfgpu_sim* s, float* slab, uint32_t first, uint32_t count);

/* Replaces sim_solv (src/simulation.c:230-345): forces and potentials for the
 * current positions; the tree's root cube is jittered with step_number. */
int sfgpu_solve(sfgpu_sim* s, uint32_t step_number);
/* Replaces sim_step (src/simulation.c:347-519): kick, drift, solve, kick,
 * per-particle energies and their FP64 totals.  Asynchronous: returns once
 * the work is queued on the simulation's stream. */
int sfgpu_step(sfgpu_sim* s, uint32_t step_number);
/* nsteps consecutive sfgpu_step calls with step numbers first, first+1, ...
 * replayed from a captured CUDA graph (unless SFGPU_FLAG_NOGRAPH). */
int sfgpu_run(sfgpu_sim* s, uint32_t first_step, uint32_t nsteps);
/* Wait for queued work. */
int sfgpu_synchronize(sfgpu_sim* s);
/* FP64 kinetic and potential energy totals of the last step, as the
 * reference prints them (src/simulation.c:453-503): T = sum ken, V = sum pen.
 * Synchronises. */
int sfgpu_energies(sfgpu_sim* s, double* T, double* V);
/* Energy with the double counting and self terms removed:
 * E = T + V/2 - (1/2) sum_i G m_i^2 / eps  (REFERENCE acc) . Synchronises. */
int sfgpu_energies_corrected(sfgpu_sim* s, double* T, double* V, double* E);
/* Momentum diagnostics of the current state (no reference counterpart):
 * P = sum_i m_i v_i and L = sum_i m_i (x_i cross v_i), per body in FP64
 * (from the FP64 state in the precision form), summed in a fixed order.
 * Either pointer may be NULL.  Queued after the work on the simulation's
 * stream; synchronises. */
int sfgpu_momentum(sfgpu_sim* s, double P[3], double L[3]);
/* Device status word (SFGPU_STATUS_* bits) accumulated since the last call;
 * reading it clears it.  Synchronises. */
int sfgpu_status(sfgpu_sim* s, uint32_t* status);

/* The simulation's CUDA stream (a cudaStream_t) and its device slab. */
void* sfgpu_stream(sfgpu_sim* s);
float* sfgpu_device_slab(sfgpu_sim* s);

/* Stage timings (ms, summed since the last call) recorded with CUDA events
 * when SFGPU_FLAG_TIMING is set.  names/ms arrays of length cap; returns
 * the number of stages written. */
int sfgpu_stage_times(sfgpu_sim* s, const char** names, double* ms, uint32_t* launches, int cap);

/* Per-particle walk counters of the last tree solve (SFGPU_FLAG_STATS):
 * monopole interactions and opening tests, by particle index. */
int sfgpu_walk_stats(sfgpu_sim* s, uint32_t* interactions, uint32_t* opening_tests);
/* Totals of the same counters (no flag needed). */
int sfgpu_walk_totals(sfgpu_sim* s, uint64_t* interactions, uint64_t* opening_tests);

/* Replaces tree_build (src/tree.c:74-318) for the positions and masses
 * already on the device: builds in the given root cube (min xyz, max xyz).
 * The status word reports node or depth overflow (tree.c:179-189). */
int sfgpu_tree_build(sfgpu_sim* s, const float bounds[6]);
/* Replaces solve_gravity_part_tree (src/gravity.c:242-663): walks the last
 * built tree for the current positions. */
int sfgpu_gravity_tree(sfgpu_sim* s);
/* Replaces solve_gravity_part_part (src/gravity.c:666-819) on the slab. */
int sfgpu_gravity_part(sfgpu_sim* s);
/* Replaces solve_sph (src/sph.c:14-282), or runs the cubic-spline SPH. */
int sfgpu_solve_sph(sfgpu_sim* s);

/* Per-body neighbour counts of the last SPH solve: REFERENCE, the bodies
 * with fl(r^2) <= 1 in the momentum pass (src/sph.c:231, j = i included);
 * CUBIC, the bodies with fl(r^2) < fl((2h)^2). */
int sfgpu_sph_neighbours(sfgpu_sim* s, uint32_t* counts);
/* The same neighbour sets as order-independent hashes (no reference
 * counterpart; for comparing two searches set for set): per body, the sum
 * modulo 2^64 of splitmix64's output function applied to each member's body
 * index.  Needs a simulation created with SFGPU_FLAG_STATS. */
int sfgpu_sph_neighbour_hashes(sfgpu_sim* s, uint64_t* hashes);
/* CUBIC SPH: specific internal energy u per body (kicked with du/dt in the
 * leapfrog, like the velocities).  Set it after sfgpu_create; read it and the
 * last du/dt back (either pointer may be NULL). */
int sfgpu_sph_set_u(sfgpu_sim* s, const float* u);
int sfgpu_sph_get_u(sfgpu_sim* s, float* u, float* dudt);

/* ---- tree inspection ---------------------------------------------------- */
/* Sorted 48-bit octree keys (3 bits per level, level 0 most significant,
 * octant bit 0 = x, 1 = y, 2 = z), the particle index of each sorted slot,
 * the number of particles inside the root cube, and the root cube. */
int sfgpu_tree_keys(sfgpu_sim* s, uint64_t* keys, uint32_t* index, uint32_t* n_inside,
                    float bounds[6]);
/* Number of nodes of the last build (1 + 8 * splits). */
int sfgpu_tree_num_nodes(sfgpu_sim* s, uint32_t* num_nodes);
/* The last build in the reference's node_t numbering and meaning
 * (src/tree.h:16-25): parent, bodies, branch[8] (child node ids, or the
 * particle ids of a leaf in insertion order), bounds[6], params[4] =
 * {COM x, y, z, mass}.  Arrays hold num_nodes entries. */
int sfgpu_tree_export(sfgpu_sim* s, uint32_t* parent, uint32_t* bodies, uint32_t* branch8,
                      float* bounds6, float* params4);

/* ---- failure detection ------------------------------------------------- */
/* Checks the bounded device wait of the radix sort's decoupled look-back
 * without a GPU fault (no reference counterpart): sorts the n host keys on
 * their low 7 bits in one tile pass of 256-thread tiles (4 keys per thread
 * up to 2^17 keys, 8 above) in which tile `withheld_tile` never publishes
 * its look-back words (0xFFFFFFFF: every tile publishes).  The tiles after
 * it wait `spin_limit` rounds (0: the default 2^24) on a word that nothing
 * sets, then give up, set SFGPU_STATUS_SPIN and finish, so the call
 * returns.  Writes the sorted keys, the original index of each sorted slot
 * and the device status word (all host arrays); the order is right only if
 * no tile was withheld. */
int sfgpu_sort_withheld_check(const uint64_t* keys, uint32_t n, uint32_t withheld_tile, uint32_t spin_limit,
                              uint64_t* sorted, uint32_t* index, uint32_t* status);

/* The library's stable radix sort of (key, original index) pairs on the n
 * host keys of `bits` significant bits (1..64), through the dispatch the
 * tree build and the SPH cell grids use (up to 2^17 keys: one tile pass on
 * the top 7-bit digit, then one CTA per bucket; above: one tile pass per
 * digit).  A check of that sort on chosen key distributions (no reference
 * counterpart: the reference sorts nothing).  Writes the sorted keys, the
 * original index of each sorted slot and the device status word. */
int sfgpu_sort_keys(const uint64_t* keys, uint32_t n, int bits, uint64_t* sorted, uint32_t* index,
                    uint32_t* status);

/* A check of the paired FP32 decisions (no reference counterpart): the
 * walk's opening test for two cells at once and the SPH density pass's
 * neighbour test for two candidates at once, against their scalar forms
 * (the reference's FP32 expressions) on n random cases around the decision
 * boundaries, seeded by `seed`.  mismatches[0] walk, [1] SPH; both 0 when
 * the paired forms decide every case as the scalar ones. */
int sfgpu_paired_check(uint32_t n, uint32_t seed, uint64_t mismatches[2]);

/* ---- process utilities ------------------------------------------------- */
/* Kernel launches the host has issued through this library in this process.
 * Replays of a captured CUDA graph issue no host launches and are not
 * counted: a replayed step runs the kernels counted while capturing it. */
unsigned long long sfgpu_kernel_launches(void);
/* Page-lock a host range so that uploads / downloads run at full speed. */
int sfgpu_host_register(void* ptr, size_t bytes);
int sfgpu_host_unregister(void* ptr);
/* Overwrite a 256 MiB device buffer (larger than the L2) on a stream, so
 * that the next kernel starts with a cold L2. */
int sfgpu_flush_l2(void* stream);

/* One drop-in call on a host slab (page-locked for full speed), as
 * sim_solv / sim_step (src/simulation.c:230-519) make it: uploads the arrays
 * the call reads (pos, vel, acc, mas; rad with SPH), runs the solve
 * (solve_only != 0) or one step, downloads the whole slab and the device
 * status word (cleared), with a single host synchronisation.  For a
 * page-locked slab the copies and the step are one captured CUDA graph
 * (recaptured when the slab pointer or the call kind changes), so a call
 * is one graph launch. */
int sfgpu_host_step(sfgpu_sim* s, float* slab, uint32_t step_number, int solve_only, uint32_t* status);

/* initcond_generate (src/initcond.c:11-255) on the device: the reference's
 * default initial conditions (uniform unit ball, its mass formula, Gaussian
 * speeds of 1e-4 plus a 4e-3 sqrt(8 pi G / 3) expansion, rad 0.1 with SPH)
 * written into the device slab (pos, vel, mas, rad), queued on the stream. */
int sfgpu_initcond(sfgpu_sim* s);

/* ---- snapshots (src/simulation_io.c:16-149, the raw format) --------------- */
/* The raw format is the slab itself, N*dof floats with no header, as
 * sim_save_raw / sim_read_raw write and read it.  sfgpu_save_raw snapshots
 * the state left by the work queued so far without waiting for it: the slab
 * is copied to page-locked staging memory on the simulation's stream and a
 * writer thread writes the file while later steps run (at most two
 * snapshots in flight; a third call waits for a free buffer).
 * sfgpu_snapshot_wait blocks until every snapshot is written and returns -1
 * with the first write error.  sfgpu_read_raw loads a raw file (exactly
 * N*dof floats, else -1; the reference only prints a short read) and
 * uploads it. */
int sfgpu_save_raw(sfgpu_sim* s, const char* filename);
int sfgpu_snapshot_wait(sfgpu_sim* s);
int sfgpu_read_raw(sfgpu_sim* s, const char* filename);

/* ---- visualisation (src/visualization.c:258-740, vis_draw) -------------- */
/* The reference's compile-time camera and image settings (config.h). */
typedef struct sfgpu_vis_params {
    uint32_t samples;    /* SPATIAL_SAMPLES: jittered splats per body (128) */
    int32_t autoscaling; /* AUTOSCALING: projection divided by the mean radius (1) */
    int32_t tonemap;     /* tanh tonemapping, as for 0 < VIS_FILE_FORMAT (1) */
    int32_t reserved;
    double timestep;     /* TIMESTEP_SIZE of the camera clock; < 0: the simulation's dt */
    double exposure;     /* EXPOSURE: pixel scale 0.01 / samples * 2^exposure (-1) */
    double ortho_scale;  /* ORTHO_SCALE: projection scale 2^ortho_scale (-1) */
} sfgpu_vis_params;
void sfgpu_vis_params_default(sfgpu_vis_params* vp);
/* Splats the simulation's current state into d_atomic (int32 RGBA,
 * 4*sizex*sizey, cleared first; alpha counts samples) and finishes it into
 * d_render (float RGBA), both device buffers, queued on the simulation's
 * stream without a sync.  Camera time = timestep * step_number. */
int sfgpu_vis_draw(sfgpu_sim* s, const sfgpu_vis_params* vp, uint32_t step_number, uint32_t sizex,
                   uint32_t sizey, int32_t* d_atomic, float* d_render);
/* Device buffers of the right size for sfgpu_vis_draw, and their release. */
int sfgpu_vis_buffers_alloc(uint32_t sizex, uint32_t sizey, int32_t** d_atomic, float** d_render);
void sfgpu_vis_buffers_free(int32_t* d_atomic, float* d_render);
/* Copies either buffer (NULL to skip) to host memory after the draw. */
int sfgpu_vis_download(sfgpu_sim* s, uint32_t sizex, uint32_t sizey, const int32_t* d_atomic,
                       const float* d_render, int32_t* atomic_out, float* render_out);
/* The model matrix of vis_draw's camera at time t (visualization.c:367-411). */
void sfgpu_vis_model_matrix(double time, float out[16]);

/* ---- stateless solver calls on device arrays ---------------------------- */
/* All pointers are device pointers in the reference layout; stream is a
 * cudaStream_t (NULL = default stream).  Work space is allocated and cached
 * per calling thread and device. */
/* solve_gravity_part_part (src/gravity.c:666-819) */
int sfgpu_gravity_pp(const sfgpu_params* p, uint32_t n, const float* pos, const float* mas,
                     float* acc, float* pot, void* stream);
/* No counterpart in the reference.  The same PP force as sfgpu_gravity_pp
 * for callers that cannot allocate device memory: a host application whose
 * own memory pool has already reserved the GPU's memory (a cudaMalloc there
 * fails or fragments the pool), or a time-critical loop that cannot take the
 * implicit device-wide synchronisation of cudaMalloc / cudaFree.  It calls
 * neither: the work array for the j-split partial sums is a 16 MiB array
 * built into the library, which every GPU that loads the library holds until
 * the process exits.  With FAST math N is limited to 1,048,576 bodies
 * (524,288 in the compensated form); larger N fails with a message in
 * sfgpu_last_error().  EXACT math needs no work array and has no such limit.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it, so make that first call before any
 * stream capture, and do not call it again on a device after
 * cudaDeviceReset.  All calls share the one array and it keeps the last
 * call's partial sums: calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.  Each call writes
 * every partial it reads, so no state carries over between calls. */
int sfgpu_gravity_pp_noalloc(const sfgpu_params* p, uint32_t n, const float* pos, const float* mas,
                             float* acc, float* pot, void* stream);

/* ---- batched form ------------------------------------------------------- */
/* Many independent systems of uneven size in one launch per step.  Systems
 * are concatenated: system b owns particles [offset[b], offset[b+1]).
 * pos/vel/acc are (total, 3), mas/pot (total). */
typedef struct sfgpu_batch sfgpu_batch;
int sfgpu_batch_create(sfgpu_batch** out, uint32_t nsys, const uint32_t* offsets,
                       const sfgpu_params* p);
int sfgpu_batch_destroy(sfgpu_batch* b);
int sfgpu_batch_upload(sfgpu_batch* b, const float* pos, const float* vel, const float* mas);
int sfgpu_batch_download(sfgpu_batch* b, float* pos, float* vel, float* acc, float* pot);
/* Forces for all systems (one persistent launch). */
int sfgpu_batch_solve(sfgpu_batch* b);
/* nsteps KDK steps for all systems, replayed from one CUDA graph. */
int sfgpu_batch_run(sfgpu_batch* b, uint32_t nsteps);
/* Pick the tile shape by timing the candidates on this batch (autotuner);
 * returns the chosen configuration index. */
int sfgpu_batch_autotune(sfgpu_batch* b, int* chosen);
int sfgpu_batch_synchronize(sfgpu_batch* b);
void* sfgpu_batch_stream(sfgpu_batch* b);

/* ---- adjoint (VJP) form ------------------------------------------------- */
/* Reverse-mode gradient of loss = sum_b mean_i |x_i|^2 (final step) of the
 * batch trajectory with respect to the initial positions and velocities,
 * with checkpoints every `checkpoint` steps and recomputation in between.
 * The batch state is left at the final step; grads are (total, 3).
 * loss (may be NULL) receives the loss. */
int sfgpu_batch_grad(sfgpu_batch* b, uint32_t nsteps, uint32_t checkpoint, float* grad_pos,
                     float* grad_vel, double* loss);
/* Single VJP of the softened PP force: given cotangents abar (total, 3) of
 * the accelerations, accumulate xbar += (d acc / d pos)^T abar. Device ptrs. */
int sfgpu_batch_force_vjp(sfgpu_batch* b, const float* d_abar, float* d_xbar);

/* ---- particle-mesh grid (src/grid.c, src/gravity.c:116-238) -------------- */
/* A cubic grid of side^3 FP32 samples over [bounds_min, bounds_max], x
 * fastest (index side*side*z + side*y + x), resident in HBM.  The
 * reference's grid is a compile-time option (ENABLE_GRID / ENABLE_FFT,
 * config.h:48-55) whose deposit (solve_gravity_part_mesh) is compiled out. */
typedef struct sfgpu_grid sfgpu_grid;
/* Replaces grid_init (src/grid.c:26-159): side in [1, 256], else -1 as the
 * reference.  The stencil -G/|x| and its spectrum are computed here, once.
 * Every grid call is queued on `stream` (a cudaStream_t, NULL = default).
 * Needs cuFFT (libcufft.so.12), loaded on first use; without it the call
 * fails with a message and the rest of the library is unaffected. */
int sfgpu_grid_create(sfgpu_grid** out, uint32_t side, const float bounds_min[3], const float bounds_max[3],
                      double G, void* stream);
/* Replaces grid_free (src/grid.c:161-188). */
int sfgpu_grid_destroy(sfgpu_grid* g);
/* grid_samp (src/grid.c:190-194): the device array of side^3 samples. */
float* sfgpu_grid_samp(sfgpu_grid* g);
/* The device array of side^3 int32 deposit counts. */
int32_t* sfgpu_grid_accum(sfgpu_grid* g);
void* sfgpu_grid_stream(sfgpu_grid* g);
uint32_t sfgpu_grid_side(const sfgpu_grid* g);
/* The deposit of solve_gravity_part_mesh (src/gravity.c:137-227): each of
 * the n bodies (device pos, 3n floats) is sampled `samples` times (the
 * reference's GRID_SAMPLES: 128) with pcg4d-seeded Gaussian offsets of sigma
 * 0.5 cell; counts land in the accum array, samp = count / samples. */
int sfgpu_grid_deposit_arrays(sfgpu_grid* g, uint32_t n, const float* pos, uint32_t step_number,
                              uint32_t samples);
/* The same over a simulation's current positions, ordered after the
 * simulation's queued work (and its later work after the deposit). */
int sfgpu_grid_deposit(sfgpu_grid* g, sfgpu_sim* s, uint32_t step_number, uint32_t samples);
/* Replaces grid_solve_fft (src/grid.c:197-536): samp <- the real part of
 * the unnormalised inverse transform of DFT(samp) * DFT(stencil), rolled by
 * side/2 along every axis.  Asynchronous. */
int sfgpu_grid_solve_fft(sfgpu_grid* g);
/* Host copies of samp (and the counts; either may be NULL), synchronous. */
int sfgpu_grid_upload(sfgpu_grid* g, const float* samp);
int sfgpu_grid_download(sfgpu_grid* g, float* samp, int32_t* accum);
int sfgpu_grid_synchronize(sfgpu_grid* g);

#ifdef __cplusplus
}
#endif
#endif
