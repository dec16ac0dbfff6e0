// vis.cu -- vis_draw's particle splat rasteriser (src/visualization.c:258-740)
// into headless device buffers.
//
// Every body is splatted SPATIAL_SAMPLES times: sample s of body i at step t
// draws one pcg4d round of {0xB79ABC95+s, 0xE0DA3F84+i, 0xAB75F07B+t,
// 0xCF52CA01}, Box-Muller turns two of the four uniforms into a Gaussian
// offset (sigma 0.75 pixel), the orthographic camera (model rotation times
// a projection scaled by 2^ORTHO_SCALE / mean radius) places the body, and
// the colour (a cosine palette of 0.1 * potential, in hundredths) is added
// with integer atomics to an RGBA int32 buffer, the alpha channel counting
// samples.  The finish pass scales by 0.01 / samples * 2^EXPOSURE and
// tonemaps with tanh.
//
// Arithmetic follows the reference's FP32 expression order without
// contraction; the transcendental functions are CUDA's (logf, cosf, sinf,
// tanh), so a sample whose coordinate lies within an ulp of a pixel edge can
// land one pixel over from the host build's.
#include <algorithm>

#include "internal.cuh"

namespace {

constexpr double VIS_TAU = 6.28318530717958647692528676655900576839433879875021;
constexpr int SPLAT_THREADS = 128;

struct VisConsts {
    float mvp_m[16];     // model matrix (host libm, as the reference)
    double ortho;        // 2^ORTHO_SCALE
    int autoscale;
    uint32_t samples;
    uint32_t step;
    uint32_t sizex, sizey;
};

// x86 float->int conversion semantics ((int)x in the reference): NaN and
// out-of-range values give INT_MIN, which every bounds test rejects.
__device__ __forceinline__ int to_int(float v) {
    return (v >= -2147483648.0f && v < 2147483648.0f) ? (int)v : INT_MIN;
}

// sum of |x_i| (FP64, fixed order) -> last block: mean radius -> the MVP matrix
__global__ void __launch_bounds__(256) k_vis_camera(const float* __restrict__ pos, uint32_t n, VisConsts vc,
                                                    double* __restrict__ part, uint32_t* done,
                                                    float* __restrict__ mvp) {
    double r = 0.0;
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) {
        const double x = pos[3u * i], y = pos[3u * i + 1u], z = pos[3u * i + 2u];
        r += sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = r;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = sh[0];
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
        if (last) *done = 0u;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double sum = 0.0;
    for (uint32_t b = 0; b < gridDim.x; b++) sum += __ldcg(&part[b]);
    const double mean = n ? sum * (1.0 / (double)n) : 1.0;
    // visualization.c:413-423: P = scale on the 3x3 block
    float s = (float)vc.ortho;
    if (vc.autoscale) s = __fmul_rn(s, (float)(1.0 / mean));
    float P[16] = {1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) P[4 * i + j] = __fmul_rn(P[4 * i + j], s);
    // visualization.c:425-478: MVP = P (V M), V = identity, products summed
    // from the last term to the first as the reference writes them
    float VM[16], C[16];
    const float I[16] = {1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            VM[4 * i + j] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(I[4 * i + 3], vc.mvp_m[12 + j]),
                                                          __fmul_rn(I[4 * i + 2], vc.mvp_m[8 + j])),
                                                __fmul_rn(I[4 * i + 1], vc.mvp_m[4 + j])),
                                      __fmul_rn(I[4 * i + 0], vc.mvp_m[j]));
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            C[4 * i + j] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(P[4 * i + 3], VM[12 + j]),
                                                         __fmul_rn(P[4 * i + 2], VM[8 + j])),
                                               __fmul_rn(P[4 * i + 1], VM[4 + j])),
                                     __fmul_rn(P[4 * i + 0], VM[j]));
    for (int k = 0; k < 16; k++) mvp[k] = C[k];
}

// one block per body, one thread per sample
__global__ void __launch_bounds__(SPLAT_THREADS) k_splat(const float* __restrict__ pos, const float* __restrict__ vel,
                                                         const float* __restrict__ pot, uint32_t n, VisConsts vc,
                                                         const float* __restrict__ mvp, int32_t* __restrict__ accum) {
    const uint32_t idx = blockIdx.x;
    if (idx >= n) return;
    __shared__ float s_p[2];
    __shared__ int32_t s_col[3];
    if (threadIdx.x == 0) {
        // visualization.c:507-547: homogeneous position through the MVP;
        // 609-619: plus the (zero, no motion blur) time offset times the
        // velocity, which only matters for a non-finite velocity
        const float x[4] = {pos[3u * idx], pos[3u * idx + 1u], pos[3u * idx + 2u], 1.0f};
        for (int i = 0; i < 2; i++) {
            const float p = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(mvp[4 * i + 0], x[0]),
                                                          __fmul_rn(mvp[4 * i + 1], x[1])),
                                                __fmul_rn(mvp[4 * i + 2], x[2])),
                                      __fmul_rn(mvp[4 * i + 3], x[3]));
            s_p[i] = __fadd_rn(p, __fmul_rn(0.0f, vel[3u * idx + i]));
        }
    }
    if (threadIdx.x < 3) {
        // visualization.c:549-555: cosine palette of 0.1 * potential
        const float phase = __fmul_rn(1.000e-1f, pot[idx]);
        const float shift = (float)(VIS_TAU * ((double)threadIdx.x / 3.0));
        const float c = __fadd_rn(__fmul_rn(0.5f, cosf(__fsub_rn(__fmul_rn((float)VIS_TAU, phase), shift))), 0.5f);
        s_col[threadIdx.x] = (int32_t)__fmul_rn(100.0f, c);
    }
    __syncthreads();
    const float p0 = s_p[0], p1 = s_p[1];
    const float half_y = __fmul_rn(0.5f, (float)vc.sizey), half_x = __fmul_rn(0.5f, (float)vc.sizex);
    for (uint32_t samp = threadIdx.x; samp < vc.samples; samp += SPLAT_THREADS) {
        uint32_t s0 = 0xB79ABC95u + samp, s1 = 0xE0DA3F84u + idx, s2 = 0xAB75F07Bu + vc.step, s3 = 0xCF52CA01u;
        pcg4d(s0, s1, s2, s3);
        const float inv = (float)2.3283062977608182109179324470460414886474609375e-10;  // INV_PCG32_MAX
        const float r2 = __fmul_rn(inv, (float)s2);
        const float r3 = __fmul_rn(inv, (float)s3);
        // visualization.c:594-606: Box-Muller, sigma 0.75
        const float rad = sqrtf(__fmul_rn(-2.0f, logf(r2)));
        const float ang = __fmul_rn((float)VIS_TAU, r3);
        const float o0 = __fmul_rn(0.750f, __fmul_rn(rad, cosf(ang)));
        const float o1 = __fmul_rn(0.750f, __fmul_rn(rad, sinf(ang)));
        // visualization.c:666-669
        const int cx = to_int(__fadd_rn(__fadd_rn(__fadd_rn(o0, -0.5f), __fmul_rn(half_y, p0)), half_x));
        const int cy = to_int(__fadd_rn(__fadd_rn(__fadd_rn(o1, -0.5f), __fmul_rn(half_y, p1)), half_y));
        if (0 <= cx && cx < (int)vc.sizex && 0 <= cy && cy < (int)vc.sizey) {
            int32_t* px = accum + 4u * ((size_t)vc.sizex * (uint32_t)cy + (uint32_t)cx);
            atomicAdd(px + 0, s_col[0]);
            atomicAdd(px + 1, s_col[1]);
            atomicAdd(px + 2, s_col[2]);
            atomicAdd(px + 3, 1);
        }
    }
}

// visualization.c:683-737: accumulated integers -> RGBA floats
__global__ void k_vis_finish(const int32_t* __restrict__ accum, uint32_t pixels, double scale, int tonemap,
                             float* __restrict__ render) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pixels) return;
    const int4 a = reinterpret_cast<const int4*>(accum)[i];
    double v[3] = {scale * (double)a.x, scale * (double)a.y, scale * (double)a.z};
    if (tonemap)
        for (int c = 0; c < 3; c++) v[c] = tanh(v[c]);
    reinterpret_cast<float4*>(render)[i] = make_float4((float)v[0], (float)v[1], (float)v[2], 1.0f);
}

struct VisScratch {
    double* part = nullptr;
    uint32_t* done = nullptr;
    float* mvp = nullptr;
};
constexpr uint32_t CAM_BLOCKS = 256;

}  // namespace

extern "C" void sfgpu_vis_model_matrix(double time, float out[16]);

extern "C" void sfgpu_vis_params_default(sfgpu_vis_params* vp) {
    if (!vp) return;
    vp->samples = 128;      // SPATIAL_SAMPLES
    vp->timestep = -1.0;    // TIMESTEP_SIZE: the simulation's dt
    vp->exposure = -1.0;    // EXPOSURE
    vp->ortho_scale = -1.0; // ORTHO_SCALE
    vp->autoscaling = 1;    // AUTOSCALING
    vp->tonemap = 1;        // 0 < VIS_FILE_FORMAT
}

extern "C" int sfgpu_vis_buffers_alloc(uint32_t sizex, uint32_t sizey, int32_t** d_atomic, float** d_render) {
    sf_clear_error();
    const size_t px = (size_t)sizex * sizey;
    *d_atomic = nullptr;
    *d_render = nullptr;
    SF_CUDA(cudaMalloc(d_atomic, sizeof(int32_t) * 4 * (px ? px : 1)));
    SF_CUDA(cudaMalloc(d_render, sizeof(float) * 4 * (px ? px : 1)));
    return SFGPU_OK;
}

extern "C" void sfgpu_vis_buffers_free(int32_t* d_atomic, float* d_render) {
    cudaFree(d_atomic);
    cudaFree(d_render);
}

extern "C" int sfgpu_vis_draw(sfgpu_sim* s, const sfgpu_vis_params* vp_in, uint32_t step_number, uint32_t sizex,
                              uint32_t sizey, int32_t* d_atomic, float* d_render) {
    sf_clear_error();
    if (!s || !d_atomic || !d_render) {
        sf_set_error("sfgpu_vis_draw: NULL argument");
        return SFGPU_FAILURE;
    }
    sfgpu_vis_params vp;
    if (vp_in) vp = *vp_in;
    else sfgpu_vis_params_default(&vp);
    if (vp.samples == 0 || sizex == 0 || sizey == 0 || (uint64_t)sizex * sizey > (1ull << 31)) {
        sf_set_error("sfgpu_vis_draw: bad size %ux%u or sample count %u", sizex, sizey, vp.samples);
        return SFGPU_FAILURE;
    }
    if (!s->vis) {
        VisScratch* v = new VisScratch();
        if (cudaMalloc(&v->part, sizeof(double) * CAM_BLOCKS) != cudaSuccess ||
            cudaMalloc(&v->done, sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&v->mvp, sizeof(float) * 16) != cudaSuccess ||
            cudaMemset(v->done, 0, sizeof(uint32_t)) != cudaSuccess) {
            cudaFree(v->part);
            cudaFree(v->done);
            cudaFree(v->mvp);
            delete v;
            sf_set_error("sfgpu_vis_draw: device allocation failed");
            return SFGPU_FAILURE;
        }
        s->vis = v;
    }
    VisScratch* v = (VisScratch*)s->vis;
    VisConsts vc;
    const double dt = vp.timestep >= 0.0 ? vp.timestep : s->p.dt;
    sfgpu_vis_model_matrix(dt * (double)step_number, vc.mvp_m);
    vc.ortho = exp2(vp.ortho_scale);
    vc.autoscale = vp.autoscaling;
    vc.samples = vp.samples;
    vc.step = step_number;
    vc.sizex = sizex;
    vc.sizey = sizey;
    const size_t pixels = (size_t)sizex * sizey;
    cudaStream_t st = s->stream;
    SF_CUDA(cudaMemsetAsync(d_atomic, 0, sizeof(int32_t) * 4 * pixels, st));
    const uint32_t cb = std::max<uint32_t>(1u, std::min<uint32_t>(CAM_BLOCKS, sf_ceil_div(s->n, 256)));
    k_vis_camera<<<cb, 256, 0, st>>>(s->slab, s->n, vc, v->part, v->done, v->mvp);
    SF_CHECK_LAUNCH();
    if (s->n) {
        k_splat<<<s->n, SPLAT_THREADS, 0, st>>>(s->slab, s->slab + (size_t)3 * s->n, s->slab + (size_t)10 * s->n,
                                                s->n, vc, v->mvp, d_atomic);
        SF_CHECK_LAUNCH();
    }
    const double scale = 0.01 / (double)vp.samples * exp2(vp.exposure);
    k_vis_finish<<<sf_ceil_div(pixels, 256), 256, 0, st>>>(d_atomic, (uint32_t)pixels, scale, vp.tonemap, d_render);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

extern "C" int sfgpu_vis_download(sfgpu_sim* s, uint32_t sizex, uint32_t sizey, const int32_t* d_atomic,
                                  const float* d_render, int32_t* atomic_out, float* render_out) {
    sf_clear_error();
    if (!s) {
        sf_set_error("sfgpu_vis_download: simulation is NULL");
        return SFGPU_FAILURE;
    }
    const size_t pixels = (size_t)sizex * sizey;
    if (atomic_out)
        SF_CUDA(cudaMemcpyAsync(atomic_out, d_atomic, sizeof(int32_t) * 4 * pixels, cudaMemcpyDeviceToHost,
                                s->stream));
    if (render_out)
        SF_CUDA(cudaMemcpyAsync(render_out, d_render, sizeof(float) * 4 * pixels, cudaMemcpyDeviceToHost,
                                s->stream));
    SF_CUDA(cudaStreamSynchronize(s->stream));
    return SFGPU_OK;
}

void sf_vis_free(sfgpu_sim* s) {
    VisScratch* v = (VisScratch*)s->vis;
    if (!v) return;
    cudaFree(v->part);
    cudaFree(v->done);
    cudaFree(v->mvp);
    delete v;
    s->vis = nullptr;
}
