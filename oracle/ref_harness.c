/*
 * ref_harness.c -- drives the unmodified Starflood reference (compiled in
 * place from its own sources by oracle/build.py) so that its results can
 * be captured as golden vectors.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled against the reference headers with a
 * generated config.h; nothing in the product links it.  Initial conditions
 * are written straight into the sim_find() arrays after sim_init(), so the
 * reference's own IC generator is not involved.
 */
#include <stdio.h>
#include <string.h>
#include <unistd.h>

#include "simulation.h"
#include "gravity.h"
#include "sph.h"
#ifndef STARFLOOD_DOUBLE_PRECISION
#include "initcond.h"
#include "visualization.h"
#endif
#ifdef ENABLE_TREE
#include "tree.h"
#endif

static sim_t g_sim;
static int g_quiet_fd = -1;

/* The reference prints per-step energies and per-build node counts to stdout;
 * silence them while it runs. */
static void mute(void) {
    fflush(stdout);
    g_quiet_fd = dup(1);
    FILE* devnull = fopen("/dev/null", "w");
    if (devnull) {
        dup2(fileno(devnull), 1);
        fclose(devnull);
    }
}
static void unmute(void) {
    fflush(stdout);
    if (g_quiet_fd >= 0) {
        dup2(g_quiet_fd, 1);
        close(g_quiet_fd);
        g_quiet_fd = -1;
    }
}

int refh_real_size(void) { return (int)sizeof(real); }
int refh_dof(void) { return (int)SIM_DOF; }
int refh_has_tree(void) {
#ifdef ENABLE_TREE
    return 1;
#else
    return 0;
#endif
}

int refh_init(unsigned int n) {
    memset(&g_sim, 0, sizeof(g_sim));
    mute();
    int rc = sim_init(&g_sim, n);
    unmute();
    return rc;
}

real* refh_mem(void) { return (real*)g_sim.mem; }

int refh_solv(unsigned int step_number) {
    g_sim.step_number = step_number;
    mute();
    int rc = sim_solv(&g_sim);
    unmute();
    return rc;
}

int refh_step(unsigned int step_number) {
    g_sim.step_number = step_number;
    mute();
    int rc = sim_step(&g_sim);
    unmute();
    return rc;
}

/* Direct solver entry points (gravity.h:13-22, sph.h:6). */
int refh_pp(void) { return solve_gravity_part_part(&g_sim); }
#ifdef ENABLE_SPH
int refh_sph(void) { return solve_sph(&g_sim); }
#endif

#ifdef ENABLE_TREE
/* tree_build() keeps its node count local (tree.c:77-79), so count the nodes
 * reachable from the root.  Returns -1 if the count exceeds max. */
static unsigned int count_nodes(const node_t* node, unsigned int at, unsigned int max, unsigned int depth) {
    unsigned int total = 1u;
    if (node[at].bodies > 8u && depth < 64u) {
        for (int o = 0; o < 8; o++) {
            unsigned int c = count_nodes(node, node[at].branch[o], max, depth + 1u);
            if (c > max) return max + 1u;
            total += c;
        }
    }
    return total;
}

unsigned int refh_tree_nodes(void) {
    return count_nodes(g_sim.tree.node, 0u, (unsigned int)TREE_NODES_MAX, 0u);
}

/* Copy node records 0..count-1 out as flat arrays.  Returns the copied count. */
unsigned int refh_tree_dump(unsigned int count, unsigned int* parent, unsigned int* bodies,
                            unsigned int* branch8, real* bounds6, real* params4) {
    const node_t* node = g_sim.tree.node;
    for (unsigned int i = 0; i < count; i++) {
        parent[i] = (unsigned int)node[i].parent;
        bodies[i] = (unsigned int)node[i].bodies;
        for (int k = 0; k < 8; k++) branch8[8u * i + (unsigned int)k] = (unsigned int)node[i].branch[k];
        for (int k = 0; k < 6; k++) bounds6[6u * i + (unsigned int)k] = node[i].bounds[k];
        for (int k = 0; k < 4; k++) params4[4u * i + (unsigned int)k] = node[i].params[k];
    }
    return count;
}

void refh_tree_bounds(real* out6) {
    for (int k = 0; k < 6; k++) out6[k] = g_sim.tree.bounds[k];
}

/* tree_build on caller arrays, as sim_solv does after setting the bounds. */
int refh_tree_build(unsigned int n, const real* bounds6) {
    for (int k = 0; k < 6; k++) g_sim.tree.bounds[k] = bounds6[k];
    mute();
    int rc = tree_build(&g_sim.tree, n, sim_find(&g_sim, SIM_POS), sim_find(&g_sim, SIM_MAS));
    unmute();
    return rc;
}

int refh_walk(void) { return solve_gravity_part_tree(&g_sim); }
#endif

#ifndef STARFLOOD_DOUBLE_PRECISION
/* src/simulation_io.c:16-149 on the harness's simulation (FP32 builds; the
 * FP64 build of simulation_io.c does not compile) */
int refh_save_raw(const char* filename) { return sim_save_raw(&g_sim, filename); }

/* src/initcond.c:11-255 on the harness's simulation */
int refh_initcond(void) { return initcond_generate(&g_sim); }

/* src/visualization_io.c:170-330: vis_save of a given render buffer (the
 * binary buffer is sized for the configured VIS_FILE_FORMAT, 8-bit here,
 * so only the PPM / PNG writers may be called) */
int refh_vis_save(const f32* render_in, unsigned int sizex, unsigned int sizey, const char* filename,
                  int filetype) {
    vis_t vis;
    mute();
    int rc = vis_init(&vis, sizex, sizey);
    if (rc == 0) {
        memcpy(vis.render_buffer, render_in, sizeof(f32) * 4u * sizex * sizey);
        rc = vis_save(&vis, filename, (image_filetype_t)filetype);
        vis_free(&vis);
    }
    unmute();
    return rc;
}

/* src/visualization.c:34-740: vis_draw of the harness's state at step_number
 * into copies of the accumulation and render buffers */
int refh_vis_draw(unsigned int step_number, unsigned int sizex, unsigned int sizey, i32* atomic_out,
                  f32* render_out) {
    vis_t vis;
    mute();
    int rc = vis_init(&vis, sizex, sizey);
    if (rc == 0) {
        g_sim.step_number = step_number;
        rc = vis_draw(&vis, &g_sim);
        memcpy(atomic_out, vis.atomic_buffer, sizeof(i32) * 4u * sizex * sizey);
        memcpy(render_out, vis.render_buffer, sizeof(f32) * 4u * sizex * sizey);
        vis_free(&vis);
    }
    unmute();
    return rc;
}
int refh_read_raw(const char* filename) { return sim_read_raw(&g_sim, filename); }
#endif

int refh_free(void) {
    mute();
    int rc = sim_free(&g_sim);
    unmute();
#ifdef ENABLE_TREE
    tree_free(&g_sim.tree);
#endif
    return rc;
}
