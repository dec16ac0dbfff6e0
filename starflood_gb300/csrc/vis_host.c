/*
 * vis_host.c -- host parts of the visualisation (src/visualization.c,
 * src/visualization_io.c): the model matrix of vis_draw's camera, the
 * reference's vis_t surface (vis_init / vis_free / vis_draw / vis_save) on
 * top of sfgpu_vis_draw, and the PFM / PPM writers.  Compiled with
 * -ffp-contract=off: the matrix and the PPM transfer curve round each FP32
 * operation as the reference does.
 */
#define _POSIX_C_SOURCE 200112L
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "starflood_compat.h"

#define VIS_TAU 6.28318530717958647692528676655900576839433879875021

/* src/visualization.c:367-411: intrinsic rotation, roll alp, pitch bet,
 * yaw gam, each advanced by tau * 1e-4 * time (FP32, libm cosf / sinf). */
void sfgpu_vis_model_matrix(double time_d, float out[16]) {
    const float time = (float)time_d;
    float alp = 0.0f;
    float bet = (float)VIS_TAU * 0.1250f;
    float gam = (float)VIS_TAU * 0.0625f;
    alp += (float)VIS_TAU * 1.000e-4f * time;
    bet += (float)VIS_TAU * 1.000e-4f * time;
    gam += (float)VIS_TAU * 1.000e-4f * time;
    const float ca = cosf(alp), sa = sinf(alp);
    const float cb = cosf(bet), sb = sinf(bet);
    const float cg = cosf(gam), sg = sinf(gam);
    const float m[16] = {
        ca * cb, ca * sb * sg - sa * cg, ca * sb * cg + sa * sg, 0.0f,
        sa * cb, sa * sb * sg + ca * cg, sa * sb * cg - ca * sg, 0.0f,
        -sb,     cb * sg,                cb * cg,                0.0f,
        0.0f,    0.0f,                   0.0f,                   1.0f,
    };
    memcpy(out, m, sizeof(m));
}

/* ---- vis_t surface (src/visualization.h) ------------------------------- */
typedef struct {
    const void* key;  /* vis_t.mem */
    int32_t* d_atomic;
    float* d_render;
} vis_slot_t;

#define MAX_VIS 64
static pthread_mutex_t g_vis_lock = PTHREAD_MUTEX_INITIALIZER;
static vis_slot_t g_vis[MAX_VIS];

/* src/visualization.c:34-176: one aligned block holding the int32 RGBA
 * accumulation buffer, the float RGBA render buffer and the 3-channel
 * binary buffer for image output (sized for the float PFM case, which also
 * holds the 8-bit PPM one). */
int vis_init(vis_t* vis, unsigned int sizex, unsigned int sizey) {
    if (!vis) return -1;
    const size_t px = (size_t)sizex * (size_t)sizey;
    const size_t bytes = sizeof(int32_t) * 4u * px + sizeof(float) * 4u * px + sizeof(float) * 3u * px;
    void* mem = NULL;
    if (posix_memalign(&mem, 4194304u, bytes ? bytes : 16) != 0 || !mem) {
        fprintf(stderr, "%s error: cannot allocate %zu bytes\n", "vis_init()", bytes);
        return -1;
    }
    memset(mem, 0, bytes);
    int32_t* d_atomic = NULL;
    float* d_render = NULL;
    if (sfgpu_vis_buffers_alloc(sizex, sizey, &d_atomic, &d_render) != SFGPU_OK) {
        fprintf(stderr, "%s error: %s\n", "vis_init()", sfgpu_last_error());
        free(mem);
        return -1;
    }
    pthread_mutex_lock(&g_vis_lock);
    int slot = -1;
    for (int i = 0; i < MAX_VIS; i++)
        if (!g_vis[i].key) {
            slot = i;
            break;
        }
    if (slot >= 0) {
        g_vis[slot].key = mem;
        g_vis[slot].d_atomic = d_atomic;
        g_vis[slot].d_render = d_render;
    }
    pthread_mutex_unlock(&g_vis_lock);
    if (slot < 0) {
        fprintf(stderr, "%s error: more than %d visualisations\n", "vis_init()", MAX_VIS);
        sfgpu_vis_buffers_free(d_atomic, d_render);
        free(mem);
        return -1;
    }
    vis->sizex = sizex;
    vis->sizey = sizey;
    vis->mem = mem;
    vis->atomic_buffer = (int32_t*)mem;
    vis->render_buffer = (float*)((char*)mem + sizeof(int32_t) * 4u * px);
    vis->binary_buffer = (char*)mem + sizeof(int32_t) * 4u * px + sizeof(float) * 4u * px;
    return 0;
}

static int take_vis(const void* key, int32_t** d_atomic, float** d_render, int remove) {
    int found = 0;
    pthread_mutex_lock(&g_vis_lock);
    for (int i = 0; i < MAX_VIS; i++)
        if (key && g_vis[i].key == key) {
            *d_atomic = g_vis[i].d_atomic;
            *d_render = g_vis[i].d_render;
            if (remove) memset(&g_vis[i], 0, sizeof(g_vis[i]));
            found = 1;
            break;
        }
    pthread_mutex_unlock(&g_vis_lock);
    return found;
}

int vis_free(vis_t* vis) {
    if (!vis) return -1;
    int32_t* d_atomic = NULL;
    float* d_render = NULL;
    if (take_vis(vis->mem, &d_atomic, &d_render, 1)) sfgpu_vis_buffers_free(d_atomic, d_render);
    free(vis->mem);
    vis->mem = NULL;
    vis->atomic_buffer = NULL;
    vis->render_buffer = NULL;
    vis->binary_buffer = NULL;
    return 0;
}

/* src/visualization.c:258-740: drawn on the GPU from the simulation's
 * current host slab; the accumulation and render buffers are current on
 * return, as with the reference. */
int vis_draw(const vis_t* vis, const sim_t* sim) {
    int32_t* d_atomic = NULL;
    float* d_render = NULL;
    if (!vis || !sim || !take_vis(vis->mem, &d_atomic, &d_render, 0)) {
        fprintf(stderr, "%s error: visualisation not initialised by vis_init\n", "vis_draw()");
        return -1;
    }
    sfgpu_sim* dev = sfgpu_compat_handle(sim);
    if (!dev) {
        fprintf(stderr, "%s error: simulation not initialised by sim_init\n", "vis_draw()");
        return -1;
    }
    sfgpu_vis_params vp;
    sfgpu_vis_params_default(&vp);
    if (sfgpu_upload(dev, (const float*)sim->mem) != SFGPU_OK ||
        sfgpu_vis_draw(dev, &vp, sim->step_number, vis->sizex, vis->sizey, d_atomic, d_render) != SFGPU_OK ||
        sfgpu_vis_download(dev, vis->sizex, vis->sizey, d_atomic, d_render, vis->atomic_buffer,
                           vis->render_buffer) != SFGPU_OK) {
        fprintf(stderr, "%s error: %s\n", "vis_draw()", sfgpu_last_error());
        return -1;
    }
    return 0;
}

/* src/visualization_io.c:20-80 */
static int write_image(const char* filename, const char* header, const void* data, size_t bytes) {
    FILE* f = fopen(filename, "wb");
    if (!f) {
        fprintf(stderr, "%s error: fopen(\"%s\", \"%s\") ", "image_write()", filename, "wb");
        perror("failed");
        return -1;
    }
    fputs(header, f);
    fwrite(data, 1, bytes, f);
    if (fclose(f) != 0) {
        fprintf(stderr, "%s error: fclose() ", "image_write()");
        perror("failed");
        return -1;
    }
    return 0;
}

/* src/visualization_io.c:170-330: PFM (float RGB, rows as rendered) or PPM
 * (BT.709 transfer curve, 8-bit, rows flipped).  PNG needs stb_image_write,
 * which this build does not carry: like a reference built without
 * ENABLE_STB_IMAGE_WRITE it reports the error.  The reference returns 0
 * even when the write failed; so does this. */
int vis_save(const vis_t* vis, const char* filename, image_filetype_t filetype) {
    if (!vis || !filename) return -1;
    const unsigned int w = vis->sizex, h = vis->sizey;
    const float* rb = vis->render_buffer;
    char header[64];
    int rc = 0;
    if (filetype == IMAGE_FILETYPE_PFM) {
        float* bin = (float*)vis->binary_buffer;
        for (size_t i = 0; i < (size_t)w * h; i++) {
            bin[3 * i + 0] = rb[4 * i + 0];
            bin[3 * i + 1] = rb[4 * i + 1];
            bin[3 * i + 2] = rb[4 * i + 2];
        }
        snprintf(header, sizeof header, "PF\n%zu %zu\n-1.0\n", (size_t)w, (size_t)h);
        rc = write_image(filename, header, bin, sizeof(float) * 3u * (size_t)w * h);
    } else if (filetype == IMAGE_FILETYPE_PPM) {
        unsigned char* bin = (unsigned char*)vis->binary_buffer;
        for (unsigned int y = 0; y < h; y++)
            for (unsigned int x = 0; x < w; x++) {
                for (int c = 0; c < 3; c++) {
                    float v = rb[4u * (w * y + x) + (unsigned)c];
                    v = 0.0f < v ? v : 0.0f;
                    v = 1.0f > v ? v : 1.0f;
                    v = 0.018053968510807f <= v ? 1.099296826809442f * powf(v, 0.45f) - 0.099296826809442f
                                                : 4.500f * v;
                    v = roundf(v * 255.0f);
                    v = 0.0f < v ? v : 0.0f;
                    v = 255.0f > v ? v : 255.0f;
                    bin[3u * (w * ((h - 1u) - y) + x) + (unsigned)c] = (unsigned char)v;
                }
            }
        snprintf(header, sizeof header, "P6\n%zu %zu %u\n", (size_t)w, (size_t)h, 255u);
        rc = write_image(filename, header, bin, 3u * (size_t)w * h);
    } else {
        fprintf(stderr, "%s error: PNG output needs stb_image_write, which this build does not include.\n",
                "image_write_png()");
        rc = -1;
    }
    if (rc != 0) fprintf(stderr, "%s error: image_write() failed.\n", "vis_save()");
    return 0;
}
