/*
 * oracle.h -- CPU restatement of Starflood's force-and-step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation in starflood_gb300/: only tests/, __graft_entry__.smoke()
 * and the cpu_baseline / reference arm of bench.py may load it.  Nothing in
 * the product links or calls it.
 *
 * The file is compiled twice: with ORC_REAL=float (liboracle_f32.so, the
 * reference's FP32 semantics, bit-for-bit) and with ORC_REAL=double
 * (liboracle_f64.so, the FP64 oracle).  Every routine cites the reference
 * file:line it restates (paths relative to the Starflood source tree).
 *
 * Floating-point contract: compiled with -ffp-contract=off and without
 * -ffast-math, expressions are written in the same association order as the
 * reference, so the FP32 build reproduces the reference's results exactly.
 */
#ifndef SF_ORACLE_H
#define SF_ORACLE_H

#include <stdint.h>

#ifndef ORC_REAL
#define ORC_REAL float
#endif
typedef ORC_REAL orc_real;

#ifdef __cplusplus
extern "C" {
#endif

/* Run-time counterpart of the reference's compile-time config.h macros. */
typedef struct {
    double   dt;          /* TIMESTEP_SIZE   (config.h)                   */
    double   eps;         /* EPSILON         (config.h), > 0              */
    double   G;           /* G               (config.h)                   */
    double   theta;       /* TREE_THETA      (config.h)                   */
    int32_t  use_tree;    /* ENABLE_TREE: 1 = BH walk, 0 = PP             */
    int32_t  use_sph;     /* ENABLE_SPH:  0 off, 1 = reference Gaussian SPH */
    int32_t  kahan;       /* ENABLE_KAHAN_SUMMATION_SOLVER/_ENERGY (1 = on) */
    uint32_t leaf_cap;    /* bodies per leaf (reference: 8, tree.h:20)    */
    uint32_t depth_max;   /* TREE_DEPTH_MAX (16)                          */
    uint32_t nodes_max;   /* TREE_NODES_MAX (262144)                      */
} orc_params;

/* Tree node.  Same meaning as the reference node_t (tree.h:16-25), with
 * room for leaf capacities above 8 (an extension used only by the leaf-16
 * variant).  params[] = {COM x, COM y, COM z, mass} after orc_tree_build. */
#define ORC_LEAF_MAX 16
typedef struct {
    uint32_t parent;
    uint32_t bodies;
    uint32_t branch[ORC_LEAF_MAX];
    orc_real bounds[6];
    orc_real params[4];
} orc_node;

/* Walk statistics per particle (no counterpart in the reference: it has no
 * interaction counter). */
typedef struct {
    uint32_t interactions;   /* monopole interactions accumulated */
    uint32_t opening_tests;  /* internal-node opening tests        */
} orc_walk_stats;

/* rng.h:13-40 */
void orc_pcg4d(uint32_t s[4]);

/* simulation.c:244-277: FP64 Kahan mean radius. */
double orc_mean_radius(uint32_t n, const orc_real* pos);

/* simulation.c:279-308: jittered root cube for a step number. */
void orc_root_bounds(uint32_t n, const orc_real* pos, uint32_t step_number,
                     orc_real bounds[6]);

/* tree.c:74-318: serial insertion build.  Returns 0, or -1 on node or depth
 * overflow (the tree is left partial, as in the reference).  *num_nodes gets
 * the node count (the reference forgets to store it, tree.c:77-79,315). */
int orc_tree_build(const orc_params* p, uint32_t n, const orc_real* pos,
                   const orc_real* mas, const orc_real bounds[6],
                   orc_node* nodes, uint32_t* num_nodes);

/* gravity.c:242-663: stackless DFS walk.  stats may be NULL. */
void orc_gravity_tree(const orc_params* p, uint32_t n, const orc_real* pos,
                      const orc_real* mas, const orc_node* nodes,
                      orc_real* acc, orc_real* pot, orc_walk_stats* stats);

/* gravity.c:666-819: all-pairs softened gravity with Kahan sums. */
void orc_gravity_pp(const orc_params* p, uint32_t n, const orc_real* pos,
                    const orc_real* mas, orc_real* acc, orc_real* pot);

/* orc_gravity_pp for the bodies idx[0..ni) only (outputs indexed like idx);
 * mag (may be NULL) receives G m_i sum_j |F_ij|. */
void orc_gravity_pp_subset(const orc_params* p, uint32_t n, const orc_real* pos, const orc_real* mas,
                           uint32_t ni, const uint32_t* idx, orc_real* acc, orc_real* pot, orc_real* mag);
/* orc_gravity_tree, also writing per body G m_i sum_k |F_k| into mag. */
void orc_gravity_tree_mag(const orc_params* p, uint32_t n, const orc_real* pos, const orc_real* mas,
                          const orc_node* nodes, orc_real* acc, orc_real* pot, orc_walk_stats* stats,
                          orc_real* mag);

/* sph.c:14-282: reference SPH (Gaussian, all pairs).  Adds the pressure
 * force into acc, writes rho and prs.  nbr (may be NULL) receives, per
 * particle, the size of the momentum-pass neighbour set {j: r2 <= 1}. */
void orc_sph_reference(const orc_params* p, uint32_t n, const orc_real* pos,
                       const orc_real* mas, const orc_real* rad, orc_real* rho,
                       orc_real* prs, orc_real* acc, uint32_t* nbr);

/* Cubic-spline SPH with ideal-gas pressure and Monaghan viscosity (no
 * reference counterpart; the FP64 oracle of the GPU's SFGPU_SPH_CUBIC).
 * Inputs are the FP32 state; rho, prs, acc (SPH part only), dudt in FP64;
 * nbr (may be NULL) gets the neighbour-set sizes (j = i included). */
void orc_sph_cubic(uint32_t n, const float* pos, const float* vel, const float* mas, const float* rad,
                   const float* u, double gamma, double alpha, double beta, double* rho, double* prs,
                   double* acc, double* dudt, uint32_t* nbr);

/* initcond_generate (src/initcond.c:11-255), FP64 with the host libm:
 * uniform unit ball from pcg4d, mass (4/3) pi / N (the reference's radius^2
 * formula at radius 1), Gaussian speeds (sigma 1e-4) plus the expansion
 * 4e-3 sqrt(8 pi G / 3) x; rad (may be NULL) = 0.1. */
void orc_initcond(uint32_t n, double G, float* pos, float* vel, float* mas, float* rad);

/* vis_draw's splat rasteriser (src/visualization.c:258-740) on FP32 state:
 * mean radius (FP64 Kahan), camera matrix at time = timestep * step,
 * `samples` pcg4d-jittered Gaussian splats per body added to the int32 RGBA
 * buffer accum (4*sizex*sizey, cleared here), then render = tanh(accum *
 * 0.01 / samples * 2^exposure) when tonemap is set.  Defaults of the
 * reference's config.h: samples 128, exposure -1, ortho_scale -1, autoscale
 * on, tonemap on.  Uses the host libm (cosf, sinf, logf, tanh). */
void orc_vis_draw(uint32_t n, const float* pos, const float* vel, const float* pot, uint32_t step,
                  double timestep, uint32_t sizex, uint32_t sizey, uint32_t samples, double exposure,
                  double ortho_scale, int autoscale, int tonemap, int32_t* accum, float* render);

/* The particle-mesh deposit of solve_gravity_part_mesh (src/gravity.c:116-230,
 * compiled out by #if 0 in the reference): `samples` samples per body, each
 * two pcg4d rounds of {0xB79ABC95+j, 0xE0DA3F84+i, 0xAB75F07B+step,
 * 0xCF52CA01} turned into a Gaussian offset of sigma 0.5 cell by Box-Muller
 * (host libm logf, cosf, sinf), counted into accum (side^3 int32, x
 * fastest); poten = (float)(count / samples).  FP32 as the reference. */
void orc_grid_deposit(uint32_t side, const float bmin[3], const float bmax[3], uint32_t n, const float* pos,
                      uint32_t step, uint32_t samples, int32_t* accum, float* poten);
/* grid.c:281-315: the stencil -G / |x| sampled at the cell corners, FP32. */
void orc_grid_stencil(uint32_t side, const float bmin[3], const float bmax[3], double G, float* out);
/* grid_solve_fft (src/grid.c:197-536) in FP64 by the DFT's definition:
 * IDFT(DFT(samp) * DFT(stencil)) unnormalised (FFTW_BACKWARD), rolled by
 * side/2 along every axis, real part. */
void orc_grid_solve_fft(uint32_t side, const float bmin[3], const float bmax[3], double G, const float* samp,
                        double* out);

/* Simulation over one slab in the reference layout (simulation.h:17-51):
 * pos[3N] vel[3N] acc[3N] mas[N] pot[N] ken[N] pen[N] (+ rad rho prs). */
typedef struct {
    uint32_t  step_number;
    uint32_t  N;
    orc_real* mem;          /* caller-owned slab of N * dof reals          */
    orc_node* nodes;        /* caller-owned, p->nodes_max entries (tree)    */
    uint32_t  num_nodes;    /* out: nodes of the last build                 */
    int32_t   tree_status;  /* out: return of the last tree build           */
    orc_real  bounds[6];    /* out: root cube of the last build             */
} orc_sim;

uint32_t orc_sim_dof(const orc_params* p);                 /* SIM_DOF */

/* simulation.c:230-345 */
int orc_sim_solv(const orc_params* p, orc_sim* s);
/* simulation.c:347-519; energies written to *T and *V (may be NULL). */
int orc_sim_step(const orc_params* p, orc_sim* s, double* T, double* V);

/* Informational: sizeof(orc_real). */
int orc_real_size(void);
/* Informational: OpenMP threads the parallel loops use. */
int orc_threads(void);

#ifdef __cplusplus
}
#endif
#endif
