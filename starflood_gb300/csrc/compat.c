/*
 * compat.c -- the reference's function surface over sim_t
 * (src/simulation.h, src/tree.h, src/gravity.h, src/sph.h), implemented on
 * the sfgpu ABI.  Each sim_t is paired with a device simulation, found by the
 * address of its slab (sim_t.mem), so sizeof(sim_t) is unchanged.  Every call
 * uploads the arrays it reads and downloads those it writes: host arrays are
 * current on return, as they are with the reference.
 */
#define _POSIX_C_SOURCE 200112L
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "starflood_compat.h"

#define COMPAT_ALIGN 4194304u /* STARFLOOD_ALIGNMENT, src/config.h:230 */
#define MAX_SIMS 256

static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;
static sfgpu_params g_params;
static int g_have_params = 0;

typedef struct {
    const void* key;      /* sim_t.mem, or the tree_t* for tree_build */
    sfgpu_sim* dev;
    unsigned int n;
} slot_t;
static slot_t g_slots[MAX_SIMS];

static void params_now(sfgpu_params* p) {
    pthread_mutex_lock(&g_lock);
    if (!g_have_params) {
        sfgpu_params_default(&g_params);
        g_have_params = 1;
    }
    *p = g_params;
    pthread_mutex_unlock(&g_lock);
}

int sfgpu_compat_configure(const sfgpu_params* p) {
    if (!p) return SFGPU_FAILURE;
    pthread_mutex_lock(&g_lock);
    g_params = *p;
    g_have_params = 1;
    pthread_mutex_unlock(&g_lock);
    return SFGPU_OK;
}

void sfgpu_compat_params(sfgpu_params* out) { params_now(out); }

static sfgpu_sim* find_slot(const void* key, unsigned int* n) {
    sfgpu_sim* r = NULL;
    pthread_mutex_lock(&g_lock);
    for (int i = 0; i < MAX_SIMS; i++) {
        if (g_slots[i].key == key && key) {
            r = g_slots[i].dev;
            if (n) *n = g_slots[i].n;
            break;
        }
    }
    pthread_mutex_unlock(&g_lock);
    return r;
}

static int add_slot(const void* key, sfgpu_sim* dev, unsigned int n) {
    int ok = -1;
    pthread_mutex_lock(&g_lock);
    for (int i = 0; i < MAX_SIMS; i++) {
        if (!g_slots[i].key) {
            g_slots[i].key = key;
            g_slots[i].dev = dev;
            g_slots[i].n = n;
            ok = 0;
            break;
        }
    }
    pthread_mutex_unlock(&g_lock);
    return ok;
}

static sfgpu_sim* take_slot(const void* key) {
    sfgpu_sim* r = NULL;
    pthread_mutex_lock(&g_lock);
    for (int i = 0; i < MAX_SIMS; i++) {
        if (g_slots[i].key == key && key) {
            r = g_slots[i].dev;
            g_slots[i].key = NULL;
            g_slots[i].dev = NULL;
            break;
        }
    }
    pthread_mutex_unlock(&g_lock);
    return r;
}

static void fail_msg(const char* fn);
sfgpu_sim* sfgpu_compat_handle(const sim_t* sim) { return sim ? find_slot(sim->mem, NULL) : NULL; }

/* Resident work queued on the handle (sfgpu_run, sfgpu_step) leaves the
 * device state ahead of sim->mem; this copies it back (one synchronisation).
 * 0, or -1 with a message on stderr as the reference's calls do. */
int sfgpu_sync_host(sim_t* sim) {
    sfgpu_sim* s = sfgpu_compat_handle(sim);
    if (!s) {
        fprintf(stderr, "sfgpu_sync_host() error: no device simulation behind this sim_t\n");
        return SFGPU_FAILURE;
    }
    if (sfgpu_download(s, (float*)sim->mem) != SFGPU_OK) {
        fail_msg("sfgpu_sync_host()");
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

static uint32_t dof_now(void) {
    sfgpu_params p;
    params_now(&p);
    return sfgpu_dof(&p);
}

/* src/simulation.c:33-53 */
real* sim_find(const sim_t* sim, enum sim_conf parameter) {
    unsigned int k = (unsigned int)parameter;
    if (k >= dof_now()) return NULL;
    if (k <= 2u) k = 0u;
    else if (k <= 5u) k = 3u;
    else if (k <= 8u) k = 6u;
    return (real*)sim->mem + (size_t)sim->N * (size_t)k;
}

static void fail_msg(const char* fn) { fprintf(stderr, "%s error: %s\n", fn, sfgpu_last_error()); }

int tree_init(tree_t* tree, unsigned int max_nodes) {
    tree->max_nodes = 0u;
    tree->num_nodes = 0u;
    for (int i = 0; i < 6; i++) tree->bounds[i] = 0.0f;
    tree->node = NULL;
    void* mem = NULL;
    if (posix_memalign(&mem, COMPAT_ALIGN, sizeof(node_t) * (size_t)max_nodes) != 0 || !mem) {
        fprintf(stderr, "tree_init() error: allocation of %u nodes failed\n", max_nodes);
        return SFGPU_FAILURE;
    }
    memset(mem, 0, sizeof(node_t) * (size_t)max_nodes);
    tree->max_nodes = max_nodes;
    tree->node = (node_t*)mem;
    return SFGPU_OK;
}

int tree_free(tree_t* tree) {
    free(tree->node);
    sfgpu_sim* dev = take_slot(tree);
    if (dev) sfgpu_destroy(dev);
    tree->max_nodes = 0u;
    tree->num_nodes = 0u;
    for (int i = 0; i < 6; i++) tree->bounds[i] = 0.0f;
    tree->node = NULL;
    return SFGPU_OK;
}

int sim_init(sim_t* sim, unsigned int N) {
    sfgpu_params p;
    params_now(&p);
    const uint32_t dof = sfgpu_dof(&p);
    const size_t bytes = sizeof(real) * (size_t)N * dof;
    void* mem = NULL;
    if (posix_memalign(&mem, COMPAT_ALIGN, bytes) != 0 || !mem) {
        fprintf(stderr, "sim_init() error: allocation of %zu bytes failed\n", bytes);
        return SFGPU_FAILURE;
    }
    memset(mem, 0, bytes);
    sfgpu_sim* dev = NULL;
    if (sfgpu_create(&dev, N, &p) != SFGPU_OK) {
        fail_msg("sim_init()");
        free(mem);
        return SFGPU_FAILURE;
    }
    /* page-locked so that every call's transfers run at full bandwidth */
    sfgpu_host_register(mem, bytes);
    if (add_slot(mem, dev, N) != 0) {
        fprintf(stderr, "sim_init() error: too many live simulations\n");
        sfgpu_destroy(dev);
        free(mem);
        return SFGPU_FAILURE;
    }
    sim->step_number = 0u;
    sim->N = N;
    sim->mem = mem;
    if (p.solver == SFGPU_SOLVER_TREE && tree_init(&sim->tree, p.nodes_max) != SFGPU_OK)
        fprintf(stderr, "sim_init() error: tree_init() failed.\n");
    return SFGPU_OK;
}

int sim_free(sim_t* sim) {
    sfgpu_sim* dev = take_slot(sim->mem);
    if (dev) {
        sfgpu_destroy(dev);
        sfgpu_host_unregister(sim->mem);
    }
    free(sim->mem);
    sim->step_number = 0u;
    sim->N = 0u;
    sim->mem = NULL;
    return SFGPU_OK;
}

static sfgpu_sim* dev_of(const sim_t* sim, const char* fn) {
    sfgpu_sim* dev = find_slot(sim->mem, NULL);
    if (!dev) fprintf(stderr, "%s error: sim_t was not created by sim_init()\n", fn);
    return dev;
}

static int export_tree(sfgpu_sim* dev, tree_t* tree) {
    uint32_t nn = 0;
    if (sfgpu_tree_num_nodes(dev, &nn) != SFGPU_OK) return SFGPU_FAILURE;
    if (!tree->node || nn > tree->max_nodes) return SFGPU_FAILURE;
    uint32_t* parent = malloc(sizeof(uint32_t) * nn);
    uint32_t* bodies = malloc(sizeof(uint32_t) * nn);
    uint32_t* branch = malloc(sizeof(uint32_t) * 8 * (size_t)nn);
    float* bounds = malloc(sizeof(float) * 6 * (size_t)nn);
    float* params = malloc(sizeof(float) * 4 * (size_t)nn);
    int rc = SFGPU_FAILURE;
    if (parent && bodies && branch && bounds && params &&
        sfgpu_tree_export(dev, parent, bodies, branch, bounds, params) == SFGPU_OK) {
        for (uint32_t i = 0; i < nn; i++) {
            node_t* nd = &tree->node[i];
            nd->parent = parent[i];
            nd->bodies = bodies[i];
            memcpy(nd->branch, branch + 8 * (size_t)i, sizeof(nd->branch));
            memcpy(nd->bounds, bounds + 6 * (size_t)i, sizeof(nd->bounds));
            memcpy(nd->params, params + 4 * (size_t)i, sizeof(nd->params));
        }
        tree->num_nodes = nn;
        rc = SFGPU_OK;
    }
    free(parent);
    free(bodies);
    free(branch);
    free(bounds);
    free(params);
    return rc;
}

static int solv_common(sim_t* sim, int step) {
    const char* fn = step ? "sim_step()" : "sim_solv()";
    sfgpu_sim* dev = dev_of(sim, fn);
    if (!dev) return SFGPU_FAILURE;
    sfgpu_params p;
    params_now(&p);
    /* upload, solve or one graph-replayed step, download: one host sync */
    uint32_t status = 0;
    if (sfgpu_host_step(dev, (float*)sim->mem, sim->step_number, !step, &status) != SFGPU_OK) {
        fail_msg(fn);
        return SFGPU_FAILURE;
    }
    if (status & (SFGPU_STATUS_TREE_NODES | SFGPU_STATUS_TREE_DEPTH))
        fprintf(stderr, "tree_build() error: Exceeded maximum %s!\n",
                (status & SFGPU_STATUS_TREE_NODES) ? "number of tree nodes" : "tree depth");
    if (p.solver == SFGPU_SOLVER_TREE && (p.flags & SFGPU_FLAG_EXPORT_TREE)) export_tree(dev, &sim->tree);
    if (step && (p.flags & SFGPU_FLAG_VERBOSE)) {
        double T = 0.0, V = 0.0;
        sfgpu_energies(dev, &T, &V);
        printf("E (tot) = % .015f\nV (pot) = % .015f\nT (kin) = % .015f\n", V + T, V, T);
    }
    return SFGPU_OK;
}

int sim_solv(sim_t* sim) { return solv_common(sim, 0); }
int sim_step(sim_t* sim) { return solv_common(sim, 1); }

/* src/initcond.c:11-255 on the device, then the slab back to the host */
int initcond_generate(sim_t* sim) {
    sfgpu_sim* dev = dev_of(sim, "initcond_generate()");
    if (!dev) return SFGPU_FAILURE;
    if (sfgpu_upload(dev, (const float*)sim->mem) != SFGPU_OK || sfgpu_initcond(dev) != SFGPU_OK ||
        sfgpu_download(dev, (float*)sim->mem) != SFGPU_OK) {
        fail_msg("initcond_generate()");
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

/* src/simulation_io.c:16-79.  The raw format is the slab itself.  As in the
 * reference, a short read is reported but not failed; the device copy
 * follows on the next call (every call uploads the host slab). */
int sim_read_raw(sim_t* sim, const char* filename) {
    if (!filename) {
        fprintf(stderr, "%s error: filename is NULL!\n", "sim_read_raw()");
        return -1;
    }
    FILE* f = fopen(filename, "rb");
    if (!f) {
        fprintf(stderr, "%s error: fopen(\"%s\", \"%s\") ", "sim_read_raw()", filename, "rb");
        perror("failed");
        return -1;
    }
    const size_t len = (size_t)sim->N * (size_t)dof_now();
    if (len != fread(sim->mem, sizeof(real), len, f)) {
        fprintf(stderr, "%s error: fread(file) ", "sim_read_raw()");
        perror("failed");
    }
    if (fclose(f) != 0) {
        fprintf(stderr, "%s error: fclose(file) ", "sim_read_raw()");
        perror("failed");
        return -1;
    }
    return 0;
}

/* src/simulation_io.c:81-149: the host slab, current after every call. */
int sim_save_raw(const sim_t* sim, const char* filename) {
    if (!filename) {
        fprintf(stderr, "%s error: filename is NULL!\n", "sim_save_raw()");
        return -1;
    }
    FILE* f = fopen(filename, "wb");
    if (!f) {
        fprintf(stderr, "%s error: fopen(\"%s\", \"%s\") ", "sim_save_raw()", filename, "wb");
        perror("failed");
        return -1;
    }
    const size_t len = (size_t)sim->N * (size_t)dof_now();
    if (len != fwrite(sim->mem, sizeof(real), len, f)) {
        fprintf(stderr, "%s error: fwrite(file) ", "sim_save_raw()");
        perror("failed");
    }
    if (fclose(f) != 0) {
        fprintf(stderr, "%s error: fclose(file) ", "sim_save_raw()");
        perror("failed");
        return -1;
    }
    return 0;
}

int sim_solv_vis(sim_t* sim, float* render_buffer, unsigned int sizex, unsigned int sizey) {
    (void)render_buffer;
    (void)sizex;
    (void)sizey;
    return sim_solv(sim);
}

int sim_step_vis(sim_t* sim, float* render_buffer, unsigned int sizex, unsigned int sizey) {
    (void)render_buffer;
    (void)sizex;
    (void)sizey;
    return sim_step(sim);
}

/* tree_build on caller arrays: a tree-only device simulation is kept per
 * tree_t (recreated when the body count changes). */
int tree_build(tree_t* tree, unsigned int num_parts, const real* pos, const real* mas) {
    sfgpu_params p;
    params_now(&p);
    p.solver = SFGPU_SOLVER_TREE;
    p.sph = SFGPU_SPH_OFF;
    p.form = SFGPU_FORM_PLAIN;
    p.nodes_max = tree->max_nodes ? tree->max_nodes : p.nodes_max;
    unsigned int have = 0;
    sfgpu_sim* dev = find_slot(tree, &have);
    if (dev && have != num_parts) {
        take_slot(tree);
        sfgpu_destroy(dev);
        dev = NULL;
    }
    if (!dev) {
        if (sfgpu_create(&dev, num_parts, &p) != SFGPU_OK || add_slot(tree, dev, num_parts) != 0) {
            fail_msg("tree_build()");
            if (dev) sfgpu_destroy(dev);
            return SFGPU_FAILURE;
        }
    }
    const uint32_t dof = sfgpu_dof(&p);
    float* slab = calloc((size_t)num_parts * dof, sizeof(float));
    if (!slab) return SFGPU_FAILURE;
    memcpy(slab, pos, sizeof(float) * 3 * (size_t)num_parts);
    memcpy(slab + (size_t)9 * num_parts, mas, sizeof(float) * (size_t)num_parts);
    int rc = sfgpu_upload(dev, slab);
    free(slab);
    if (rc != SFGPU_OK || sfgpu_tree_build(dev, tree->bounds) != SFGPU_OK) {
        fail_msg("tree_build()");
        return SFGPU_FAILURE;
    }
    uint32_t status = 0;
    sfgpu_status(dev, &status);
    if (status & SFGPU_STATUS_TREE_NODES) {
        fprintf(stderr, "%s error: Exceeded maximum number of tree nodes!\n", "tree_build()");
        return SFGPU_FAILURE;
    }
    if (status & SFGPU_STATUS_TREE_DEPTH) {
        fprintf(stderr, "%s error: Exceeded maximum tree depth!\n", "tree_build()");
        return SFGPU_FAILURE;
    }
    if (export_tree(dev, tree) != SFGPU_OK) {
        fail_msg("tree_build()");
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

static int single_solver(const sim_t* sim, int which) {
    static const char* names[3] = {"solve_gravity_part_part()", "solve_gravity_part_tree()", "solve_sph()"};
    sfgpu_sim* dev = dev_of(sim, names[which]);
    if (!dev) return SFGPU_FAILURE;
    if (sfgpu_upload(dev, (const float*)sim->mem) != SFGPU_OK) {
        fail_msg(names[which]);
        return SFGPU_FAILURE;
    }
    int rc;
    if (which == 0) {
        rc = sfgpu_gravity_part(dev);
    } else if (which == 1) {
        rc = sfgpu_tree_build(dev, sim->tree.bounds);
        if (rc == SFGPU_OK) rc = sfgpu_gravity_tree(dev);
    } else {
        rc = sfgpu_solve_sph(dev);
    }
    if (rc != SFGPU_OK || sfgpu_download(dev, (float*)sim->mem) != SFGPU_OK) {
        fail_msg(names[which]);
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

int solve_gravity_part_part(const sim_t* sim) { return single_solver(sim, 0); }
int solve_gravity_part_tree(const sim_t* sim) { return single_solver(sim, 1); }
int solve_sph(const sim_t* sim) { return single_solver(sim, 2); }
