// grid.cu -- the particle-mesh grid: the deposit of solve_gravity_part_mesh
// (src/gravity.c:116-238, compiled out by #if 0 in the reference) and
// grid_solve_fft (src/grid.c:197-536), on a cubic grid of side <= 256.
//
// Deposit: every body is sampled `samples` times; sample j of body i at
// step t runs two pcg4d rounds of {0xB79ABC95+j, 0xE0DA3F84+i, 0xAB75F07B+t,
// 0xCF52CA01}, Box-Muller turns them into a Gaussian offset of sigma 0.5
// cell, and the sample is counted in the int32 cell it lands in.  One warp
// per body; lanes that land in the same cell merge their counts
// (__match_any_sync) so each distinct cell of a warp round costs one atomic.
// The counts become samp = count / samples.
//
// Solve: the reference convolves samp with the stencil -G/|x| sampled at
// the cell corners (the stencil's origin is the grid's centre for the
// symmetric bounds it uses) by three complex FFTs, an unnormalised inverse,
// a roll by side/2 along every axis and the real part.  Here the inputs are
// real, so the transforms are real-to-complex / complex-to-real (cuFFT,
// loaded at run time), the stencil's spectrum is computed once per grid, and
// the roll is folded into it as the shift phase exp(+2 pi i k.s / side),
// s = side/2 (exactly +-1 for even sides): one forward transform, one
// pointwise product and one inverse transform per solve, written straight
// into samp.  The result is the reference's up to FP32 FFT rounding.
#include <dlfcn.h>

#include <cufft.h>

#include "internal.cuh"

namespace {

constexpr double GRID_TAU = 6.28318530717958647692528676655900576839433879875021;
constexpr int DEPOSIT_THREADS = 256;

// x86 float->int conversion ((int)x in the reference): NaN and out-of-range
// values give INT_MIN, which the bounds test rejects.
__device__ __forceinline__ int grid_to_int(float v) {
    return (v >= -2147483648.0f && v < 2147483648.0f) ? (int)v : INT_MIN;
}

// gravity.c:150-219: one warp per body, lanes over the samples
__global__ void __launch_bounds__(DEPOSIT_THREADS) k_grid_deposit(const float* __restrict__ pos, uint32_t n,
                                                                  uint32_t side, float3 bmin, float3 wid,
                                                                  uint32_t step, uint32_t samples,
                                                                  int32_t* __restrict__ accum) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t i = blockIdx.x * (DEPOSIT_THREADS / 32) + (threadIdx.x >> 5);
    if (i >= n) return;
    const float fs = (float)side;
    const float pl[3] = {__fdiv_rn(__fsub_rn(pos[3u * i], bmin.x), wid.x),
                         __fdiv_rn(__fsub_rn(pos[3u * i + 1u], bmin.y), wid.y),
                         __fdiv_rn(__fsub_rn(pos[3u * i + 2u], bmin.z), wid.z)};
    const float base[3] = {__fmul_rn(fs, pl[0]), __fmul_rn(fs, pl[1]), __fmul_rn(fs, pl[2])};
    const float inv = (float)2.3283062977608182109179324470460414886474609375e-10;  // INV_PCG32_MAX
    const float tau = (float)GRID_TAU;
    for (uint32_t j0 = 0; j0 < samples; j0 += 32u) {
        const uint32_t j = j0 + lane;
        uint32_t key = 0xFFFFFFFFu;  // no cell
        if (j < samples) {
            uint32_t s0 = 0xB79ABC95u + j, s1 = 0xE0DA3F84u + i, s2 = 0xAB75F07Bu + step, s3 = 0xCF52CA01u;
            pcg4d(s0, s1, s2, s3);
            pcg4d(s0, s1, s2, s3);
            const float r0 = __fmul_rn(inv, (float)s0), r1 = __fmul_rn(inv, (float)s1);
            const float r2 = __fmul_rn(inv, (float)s2), r3 = __fmul_rn(inv, (float)s3);
            // Box-Muller (gravity.c:183-188)
            const float a = sqrtf(__fmul_rn(-2.0f, logf(r0)));
            const float b = sqrtf(__fmul_rn(-2.0f, logf(r2)));
            const float g[3] = {__fmul_rn(a, cosf(__fmul_rn(tau, r1))), __fmul_rn(a, sinf(__fmul_rn(tau, r1))),
                                __fmul_rn(b, cosf(__fmul_rn(tau, r3)))};
            int c[3];
            for (int k = 0; k < 3; k++) c[k] = grid_to_int(__fadd_rn(__fadd_rn(__fmul_rn(0.500f, g[k]), base[k]), 0.5f));
            if (0 <= c[0] && c[0] < (int)side && 0 <= c[1] && c[1] < (int)side && 0 <= c[2] && c[2] < (int)side)
                key = (side * (uint32_t)c[2] + (uint32_t)c[1]) * side + (uint32_t)c[0];
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        if (key != 0xFFFFFFFFu && (__ffs(peers) - 1) == (int)lane) atomicAdd(accum + key, __popc(peers));
    }
}

// gravity.c:224-227: counts -> FP32 samples.  With a power-of-two sample
// count the scale is exact in FP32 and (float)count * 2^-k equals the
// reference's (float)(count * 2^-k) in FP64.
__global__ void k_grid_counts(const int32_t* __restrict__ accum, size_t cells, float inv_f, double inv_d, int pow2,
                              float* __restrict__ samp) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < cells; c += (size_t)gridDim.x * blockDim.x) {
        const int32_t v = accum[c];
        samp[c] = pow2 ? __fmul_rn((float)v, inv_f) : (float)(inv_d * (double)v);
    }
}

// grid.c:281-315: -G / |x| at the cell corners, FP32 in the reference's order
__global__ void k_grid_stencil(uint32_t side, float3 bmin, float3 wid, float neg_g, float* __restrict__ out) {
    const size_t cells = (size_t)side * side * side;
    const float fs = (float)side;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < cells; c += (size_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(c % side), y = (uint32_t)((c / side) % side), z = (uint32_t)(c / side / side);
        const float px = __fadd_rn(__fmul_rn(wid.x, __fdiv_rn((float)x, fs)), bmin.x);
        const float py = __fadd_rn(__fmul_rn(wid.y, __fdiv_rn((float)y, fs)), bmin.y);
        const float pz = __fadd_rn(__fmul_rn(wid.z, __fdiv_rn((float)z, fs)), bmin.z);
        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py)), __fmul_rn(pz, pz));
        const float ir = 0.0f < r2 ? __fdiv_rn(1.0f, __fsqrt_rn(r2)) : 0.0f;
        out[c] = __fmul_rn(neg_g, ir);
    }
}

// The roll by side/2 (grid.c:500-521) as the shift phase of the stencil's
// half spectrum [z][y][x <= side/2].
__global__ void k_grid_phase(uint32_t side, float2* __restrict__ kern) {
    const uint32_t hx = side / 2u + 1u, sh = side / 2u;
    const size_t count = (size_t)side * side * hx;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < count; c += (size_t)gridDim.x * blockDim.x) {
        const uint32_t kx = (uint32_t)(c % hx), ky = (uint32_t)((c / hx) % side), kz = (uint32_t)(c / hx / side);
        const uint32_t m = (uint32_t)(((uint64_t)kx + ky + kz) * sh % side);
        double sn, cs;
        sincospi(2.0 * (double)m / (double)side, &sn, &cs);
        const float2 k = kern[c];
        kern[c] = make_float2((float)((double)k.x * cs - (double)k.y * sn), (float)((double)k.x * sn + (double)k.y * cs));
    }
}

// grid.c:444-475: the pointwise product, in place
__global__ void k_grid_mul(float2* __restrict__ spec, const float2* __restrict__ kern, size_t count) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < count; c += (size_t)gridDim.x * blockDim.x) {
        const float2 f = spec[c], s = kern[c];
        spec[c] = make_float2(__fsub_rn(__fmul_rn(f.x, s.x), __fmul_rn(f.y, s.y)),
                              __fadd_rn(__fmul_rn(f.x, s.y), __fmul_rn(f.y, s.x)));
    }
}

// side 1: the transforms are the identity and the roll is empty
__global__ void k_grid_single(float* samp, float kern) { samp[0] = __fmul_rn(samp[0], kern); }

// cuFFT, resolved at run time so that the rest of the library loads on a
// host without it; the grid calls fail with a message instead.
struct CufftApi {
    bool ok = false;
    char err[256] = {0};
    decltype(&cufftPlan3d) plan3d = nullptr;
    decltype(&cufftExecR2C) exec_r2c = nullptr;
    decltype(&cufftExecC2R) exec_c2r = nullptr;
    decltype(&cufftSetStream) set_stream = nullptr;
    decltype(&cufftDestroy) destroy = nullptr;
};

CufftApi load_cufft() {
    CufftApi a;
    void* h = nullptr;
    for (const char* name : {"libcufft.so.12", "libcufft.so.13", "libcufft.so"})
        if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
        snprintf(a.err, sizeof a.err, "cuFFT not found (dlopen libcufft.so.12: %s)", dlerror());
        return a;
    }
    a.plan3d = (decltype(a.plan3d))dlsym(h, "cufftPlan3d");
    a.exec_r2c = (decltype(a.exec_r2c))dlsym(h, "cufftExecR2C");
    a.exec_c2r = (decltype(a.exec_c2r))dlsym(h, "cufftExecC2R");
    a.set_stream = (decltype(a.set_stream))dlsym(h, "cufftSetStream");
    a.destroy = (decltype(a.destroy))dlsym(h, "cufftDestroy");
    a.ok = a.plan3d && a.exec_r2c && a.exec_c2r && a.set_stream && a.destroy;
    if (!a.ok) snprintf(a.err, sizeof a.err, "cuFFT: missing symbols");
    return a;
}

const CufftApi& cufft() {
    static const CufftApi api = load_cufft();
    return api;
}

unsigned grid_blocks(size_t items, int threads) {
    const size_t b = (items + threads - 1) / threads;
    return (unsigned)std::min<size_t>(std::max<size_t>(b, 1), 152u * 16u);
}

}  // namespace

struct sfgpu_grid {
    uint32_t side = 0;
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    double G = 1.0;
    cudaStream_t stream = nullptr;
    float* samp = nullptr;     // side^3, x fastest (grid_samp)
    int32_t* accum = nullptr;  // side^3 deposit counts
    float2* spec = nullptr;    // side * side * (side/2+1) half spectrum
    float2* kern = nullptr;    // the stencil's half spectrum times the roll phase
    float kern0 = 0.0f;        // side 1: the stencil's one value
    cufftHandle fwd = 0, inv = 0;
    bool have_fwd = false, have_inv = false;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};

namespace {

int grid_cufft(cufftResult r, const char* what) {
    if (r != CUFFT_SUCCESS) {
        sf_set_error("%s failed (cufftResult %d)", what, (int)r);
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

float3 grid_lo(const sfgpu_grid* g) { return make_float3(g->bmin[0], g->bmin[1], g->bmin[2]); }
float3 grid_wid(const sfgpu_grid* g) {
    return make_float3(g->bmax[0] - g->bmin[0], g->bmax[1] - g->bmin[1], g->bmax[2] - g->bmin[2]);
}

}  // namespace

extern "C" int sfgpu_grid_destroy(sfgpu_grid* g) {
    if (!g) return SFGPU_OK;
    if (g->stream) cudaStreamSynchronize(g->stream);
    else cudaDeviceSynchronize();
    if (g->have_fwd) cufft().destroy(g->fwd);
    if (g->have_inv) cufft().destroy(g->inv);
    cudaFree(g->samp);
    cudaFree(g->accum);
    cudaFree(g->spec);
    cudaFree(g->kern);
    if (g->ev_in) cudaEventDestroy(g->ev_in);
    if (g->ev_out) cudaEventDestroy(g->ev_out);
    delete g;
    return SFGPU_OK;
}

extern "C" int sfgpu_grid_create(sfgpu_grid** out, uint32_t side, const float bounds_min[3],
                                 const float bounds_max[3], double G, void* stream) {
    sf_clear_error();
    if (!out || !bounds_min || !bounds_max) {
        sf_set_error("sfgpu_grid_create: null argument");
        return SFGPU_FAILURE;
    }
    *out = nullptr;
    // grid.c:29-35
    if (side < 1u || side > 256u) {
        sf_set_error("sfgpu_grid_create: side_length %u outside [1, 256]", side);
        return SFGPU_FAILURE;
    }
    if (side > 1u && !cufft().ok) {
        sf_set_error("sfgpu_grid_create: %s", cufft().err);
        return SFGPU_FAILURE;
    }
    sfgpu_grid* g = new sfgpu_grid;
    g->side = side;
    for (int k = 0; k < 3; k++) {
        g->bmin[k] = bounds_min[k];
        g->bmax[k] = bounds_max[k];
    }
    g->G = G;
    g->stream = (cudaStream_t)stream;
    const size_t cells = (size_t)side * side * side;
    const size_t half = (size_t)side * side * (side / 2u + 1u);
    auto fail = [&]() {
        sfgpu_grid_destroy(g);
        return SFGPU_FAILURE;
    };
#define GRID_TRY(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            sf_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return fail();                                                                      \
        }                                                                                       \
    } while (0)
    GRID_TRY(cudaMalloc(&g->samp, sizeof(float) * cells));
    GRID_TRY(cudaMalloc(&g->accum, sizeof(int32_t) * cells));
    GRID_TRY(cudaMalloc(&g->spec, sizeof(float2) * half));
    GRID_TRY(cudaMalloc(&g->kern, sizeof(float2) * half));
    GRID_TRY(cudaEventCreateWithFlags(&g->ev_in, cudaEventDisableTiming));
    GRID_TRY(cudaEventCreateWithFlags(&g->ev_out, cudaEventDisableTiming));
    GRID_TRY(cudaMemsetAsync(g->samp, 0, sizeof(float) * cells, g->stream));
    GRID_TRY(cudaMemsetAsync(g->accum, 0, sizeof(int32_t) * cells, g->stream));
    // the stencil (into samp as scratch) and its spectrum
    k_grid_stencil<<<grid_blocks(cells, 256), 256, 0, g->stream>>>(side, grid_lo(g), grid_wid(g), (float)(-G),
                                                                    g->samp);
    GRID_TRY(cudaGetLastError());
    if (side == 1u) {
        GRID_TRY(cudaMemcpyAsync(&g->kern0, g->samp, sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    } else {
        const int n = (int)side;
        if (grid_cufft(cufft().plan3d(&g->fwd, n, n, n, CUFFT_R2C), "cufftPlan3d(R2C)")) return fail();
        g->have_fwd = true;
        if (grid_cufft(cufft().plan3d(&g->inv, n, n, n, CUFFT_C2R), "cufftPlan3d(C2R)")) return fail();
        g->have_inv = true;
        if (grid_cufft(cufft().set_stream(g->fwd, g->stream), "cufftSetStream")) return fail();
        if (grid_cufft(cufft().set_stream(g->inv, g->stream), "cufftSetStream")) return fail();
        if (grid_cufft(cufft().exec_r2c(g->fwd, g->samp, (cufftComplex*)g->kern), "cufftExecR2C(stencil)"))
            return fail();
        k_grid_phase<<<grid_blocks(half, 256), 256, 0, g->stream>>>(side, g->kern);
        GRID_TRY(cudaGetLastError());
    }
    GRID_TRY(cudaMemsetAsync(g->samp, 0, sizeof(float) * cells, g->stream));
    GRID_TRY(cudaStreamSynchronize(g->stream));
#undef GRID_TRY
    *out = g;
    return SFGPU_OK;
}

extern "C" float* sfgpu_grid_samp(sfgpu_grid* g) { return g ? g->samp : nullptr; }
extern "C" int32_t* sfgpu_grid_accum(sfgpu_grid* g) { return g ? g->accum : nullptr; }
extern "C" void* sfgpu_grid_stream(sfgpu_grid* g) { return g ? (void*)g->stream : nullptr; }
extern "C" uint32_t sfgpu_grid_side(const sfgpu_grid* g) { return g ? g->side : 0u; }

extern "C" int sfgpu_grid_deposit_arrays(sfgpu_grid* g, uint32_t n, const float* pos, uint32_t step_number,
                                         uint32_t samples) {
    sf_clear_error();
    if (!g || (n && !pos)) {
        sf_set_error("sfgpu_grid_deposit_arrays: null argument");
        return SFGPU_FAILURE;
    }
    const size_t cells = (size_t)g->side * g->side * g->side;
    SF_CUDA(cudaMemsetAsync(g->accum, 0, sizeof(int32_t) * cells, g->stream));
    if (n && samples) {
        const uint32_t wpb = DEPOSIT_THREADS / 32;
        k_grid_deposit<<<(n + wpb - 1) / wpb, DEPOSIT_THREADS, 0, g->stream>>>(pos, n, g->side, grid_lo(g),
                                                                               grid_wid(g), step_number, samples,
                                                                               g->accum);
        SF_CHECK_LAUNCH();
    }
    const bool pow2 = samples && (samples & (samples - 1u)) == 0u;
    const double inv_d = samples ? 1.0 / (double)samples : 0.0;
    k_grid_counts<<<grid_blocks(cells, 256), 256, 0, g->stream>>>(g->accum, cells, (float)inv_d, inv_d,
                                                                   pow2 ? 1 : 0, g->samp);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

extern "C" int sfgpu_grid_deposit(sfgpu_grid* g, sfgpu_sim* s, uint32_t step_number, uint32_t samples) {
    sf_clear_error();
    if (!g || !s) {
        sf_set_error("sfgpu_grid_deposit: null argument");
        return SFGPU_FAILURE;
    }
    // the grid's stream reads the simulation's positions after its queued
    // work, and the simulation's next work waits for the deposit
    SF_CUDA(cudaEventRecord(g->ev_in, s->stream));
    SF_CUDA(cudaStreamWaitEvent(g->stream, g->ev_in, 0));
    if (sfgpu_grid_deposit_arrays(g, s->n, s->slab, step_number, samples)) return SFGPU_FAILURE;
    SF_CUDA(cudaEventRecord(g->ev_out, g->stream));
    SF_CUDA(cudaStreamWaitEvent(s->stream, g->ev_out, 0));
    return SFGPU_OK;
}

extern "C" int sfgpu_grid_solve_fft(sfgpu_grid* g) {
    sf_clear_error();
    if (!g) {
        sf_set_error("sfgpu_grid_solve_fft: null grid");
        return SFGPU_FAILURE;
    }
    if (g->side == 1u) {
        k_grid_single<<<1, 1, 0, g->stream>>>(g->samp, g->kern0);
        SF_CHECK_LAUNCH();
        return SFGPU_OK;
    }
    const size_t half = (size_t)g->side * g->side * (g->side / 2u + 1u);
    if (grid_cufft(cufft().exec_r2c(g->fwd, g->samp, (cufftComplex*)g->spec), "cufftExecR2C")) return SFGPU_FAILURE;
    k_grid_mul<<<grid_blocks(half, 256), 256, 0, g->stream>>>(g->spec, g->kern, half);
    SF_CHECK_LAUNCH();
    if (grid_cufft(cufft().exec_c2r(g->inv, (cufftComplex*)g->spec, g->samp), "cufftExecC2R")) return SFGPU_FAILURE;
    return SFGPU_OK;
}

extern "C" int sfgpu_grid_upload(sfgpu_grid* g, const float* samp) {
    sf_clear_error();
    if (!g || !samp) {
        sf_set_error("sfgpu_grid_upload: null argument");
        return SFGPU_FAILURE;
    }
    const size_t cells = (size_t)g->side * g->side * g->side;
    SF_CUDA(cudaMemcpyAsync(g->samp, samp, sizeof(float) * cells, cudaMemcpyHostToDevice, g->stream));
    SF_CUDA(cudaStreamSynchronize(g->stream));
    return SFGPU_OK;
}

extern "C" int sfgpu_grid_download(sfgpu_grid* g, float* samp, int32_t* accum) {
    sf_clear_error();
    if (!g) {
        sf_set_error("sfgpu_grid_download: null grid");
        return SFGPU_FAILURE;
    }
    const size_t cells = (size_t)g->side * g->side * g->side;
    if (samp) SF_CUDA(cudaMemcpyAsync(samp, g->samp, sizeof(float) * cells, cudaMemcpyDeviceToHost, g->stream));
    if (accum)
        SF_CUDA(cudaMemcpyAsync(accum, g->accum, sizeof(int32_t) * cells, cudaMemcpyDeviceToHost, g->stream));
    SF_CUDA(cudaStreamSynchronize(g->stream));
    return SFGPU_OK;
}

extern "C" int sfgpu_grid_synchronize(sfgpu_grid* g) {
    sf_clear_error();
    if (!g) {
        sf_set_error("sfgpu_grid_synchronize: null grid");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(g->stream));
    return SFGPU_OK;
}
