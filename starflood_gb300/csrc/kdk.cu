// kdk.cu -- the leapfrog of sim_step (src/simulation.c:347-519) and the root
// cube of sim_solv (src/simulation.c:244-308), fused into three passes over
// the slab:
//
//   k_kick_drift   kick_0 and drift for one body per thread (each component
//                  rounded exactly as the reference: v + ((dt/2) a), x + dt v)
//                  and, for the tree, the body's distance from the origin (to
//                  FP64-like precision in float-float arithmetic) summed per
//                  block; the last block adds the
//                  block sums, takes the mean radius, hashes the step number
//                  with pcg4d and writes the jittered root cube in FP32;
//   k_kick_energy  kick_1, ken = (m/2) v^2, pen = m pot, per-block
//                  float-float sums of ken, pen and the corrected energies,
//                  added in block order by the last block.
//
// Bytes per body: kick/drift reads pos, vel, acc (36 B) and writes pos, vel
// (24 B); kick/energy reads vel, acc, mas, pot (32 B), writes vel, ken, pen
// (20 B).  All HBM-bound.
#include "internal.cuh"

namespace {

constexpr double K_INV_U32 = 2.3283062977608182109179324470460414886474609375e-10;  // rng.h:9

// Block sum of NV per-thread values in a fixed order: float-float within
// each warp (shuffles), then the 8 warp totals in FP64 by thread 0, which
// writes the NV block totals.  Only the last step touches the FP64 pipe.
template <int NV>
__device__ void block_sum(ff (&v)[NV], double* out) {
    __shared__ double wsum[NV][SF_RED_BLOCK / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ff_warp_sum<NV>(v);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) wsum[k][warp] = ff_to_double(v[k]);
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double t = 0.0;
            for (int w = 0; w < SF_RED_BLOCK / 32; w++) t += wsum[k][w];
            out[(size_t)blockIdx.x * NV + k] = t;
        }
    }
}

// simulation.c:253-260: sqrt((x*x)+(y*y)+(z*z)), the reference's FP64 value
// to about 46 bits, in float-float arithmetic on the FP32 pipe
__device__ __forceinline__ ff radius_ff(float x, float y, float z) {
    return ff_sqrt(ff_add(ff_add(ff_sqr(x), ff_sqr(y)), ff_sqr(z)));
}

// The last block to finish (ticket from an atomic counter, reset for the
// next launch) adds up the per-block partials in block order, so the totals
// are deterministic, and no separate single-block launch is needed.
__device__ bool last_block(uint32_t* done) {
    __shared__ bool s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t ticket = atomicAdd(done, 1u);
        s_last = ticket == gridDim.x - 1;
        if (s_last) *done = 0u;
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last;
}

template <int NV>
__device__ void sum_partials(const double* part, uint32_t nparts, double* out) {
    double v[NV];
    for (int k = 0; k < NV; k++) v[k] = 0.0;
    for (uint32_t b = threadIdx.x; b < nparts; b += SF_RED_BLOCK)
        for (int k = 0; k < NV; k++) v[k] += __ldcg(&part[(size_t)b * NV + k]);
    __shared__ double wsum[NV][SF_RED_BLOCK / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < NV; k++) {
        double x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) wsum[k][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) {
            double t = 0.0;
            for (int w = 0; w < SF_RED_BLOCK / 32; w++) t += wsum[k][w];
            out[k] = t;
        }
}

// simulation.c:276-301: mean radius -> jittered root cube
__device__ void root_cube(double sum, uint32_t n, uint32_t step, float* __restrict__ bounds, double* __restrict__ sums) {
    const double rbar = __dmul_rn(sum, 1.0 / (double)n);
    uint32_t a = 0x638FE17Bu + step, b = 0xB10BDCE7u, c = 0x7B8ADB9Bu, d = 0xD8C5850Eu;
    pcg4d(a, b, c, d);
    const uint32_t h[3] = {a, b, c};
    for (int k = 0; k < 3; k++) {
        const double j = __dsub_rn(__dmul_rn(2.0, __dmul_rn(K_INV_U32, (double)h[k])), 1.0);
        const double shift = __dmul_rn(__dmul_rn(0.5, j), rbar);
        bounds[k] = __double2float_rn(__dadd_rn(__dmul_rn(-2.000, rbar), shift));
        bounds[3 + k] = __double2float_rn(__dadd_rn(__dmul_rn(2.000, rbar), shift));
    }
    sums[4] = rbar;
}

__device__ void finish_bounds(const double* part, uint32_t n, const uint32_t* d_step, float* bounds, double* sums) {
    __shared__ double tot[1];
    sum_partials<1>(part, gridDim.x, tot);
    __syncthreads();
    if (threadIdx.x == 0) root_cube(tot[0], n, *d_step, bounds, sums);
}

__global__ void __launch_bounds__(SF_RED_BLOCK) k_kick_drift(float* __restrict__ slab, uint32_t n, float half_dt,
                                                             float dt, double* __restrict__ pos64,
                                                             double* __restrict__ vel64, double dt64,
                                                             int want_radius, double* __restrict__ part,
                                                             uint32_t* done, const uint32_t* __restrict__ d_step,
                                                             float* __restrict__ bounds, double* __restrict__ sums,
                                                             float* __restrict__ u, const float* __restrict__ dudt) {
    const uint32_t i = blockIdx.x * SF_RED_BLOCK + threadIdx.x;
    if (u && i < n) u[i] = fadd(u[i], fmul(half_dt, dudt[i]));  // SPH internal energy, kick_0
    float* pos = slab;
    float* vel = slab + (size_t)3 * n;
    const float* acc = slab + (size_t)6 * n;
    ff r[1] = {ff{0.0f, 0.0f}};
    if (i < n) {
        float x[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const size_t k = 3u * (size_t)i + c;
            if (pos64) {
                // precision form: FP64 state, FP32 copies for the force kernels
                const double v = vel64[k] + 0.5 * dt64 * (double)acc[k];
                const double xx = pos64[k] + dt64 * v;
                vel64[k] = v;
                pos64[k] = xx;
                vel[k] = (float)v;
                x[c] = (float)xx;
                pos[k] = x[c];
            } else {
                const float v = fadd(vel[k], fmul(half_dt, acc[k]));  // simulation.c:382
                x[c] = fadd(pos[k], fmul(dt, v));                      // simulation.c:394
                vel[k] = v;
                pos[k] = x[c];
            }
        }
        if (want_radius) r[0] = radius_ff(x[0], x[1], x[2]);
    }
    if (!want_radius) return;
    block_sum<1>(r, part);
    if (last_block(done)) finish_bounds(part, n, d_step, bounds, sums);
}

__global__ void __launch_bounds__(SF_RED_BLOCK) k_radius(const float* __restrict__ pos, uint32_t n,
                                                         double* __restrict__ part, uint32_t* done,
                                                         const uint32_t* __restrict__ d_step,
                                                         float* __restrict__ bounds, double* __restrict__ sums) {
    const uint32_t i = blockIdx.x * SF_RED_BLOCK + threadIdx.x;
    ff r[1] = {ff{0.0f, 0.0f}};
    if (i < n) r[0] = radius_ff(pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u]);
    block_sum<1>(r, part);
    if (last_block(done)) finish_bounds(part, n, d_step, bounds, sums);
}

__global__ void __launch_bounds__(SF_RED_BLOCK) k_kick_energy(float* __restrict__ slab, uint32_t n, float half_dt,
                                                              double* __restrict__ vel64, double dt64,
                                                              float g_over_eps, int physical,
                                                              double* __restrict__ part, uint32_t* done,
                                                              double* __restrict__ sums, uint32_t* d_step,
                                                              float* __restrict__ u, const float* __restrict__ dudt) {
    const uint32_t i = blockIdx.x * SF_RED_BLOCK + threadIdx.x;
    if (u && i < n) u[i] = fadd(u[i], fmul(half_dt, dudt[i]));  // SPH internal energy, kick_1
    float* vel = slab + (size_t)3 * n;
    const float* acc = slab + (size_t)6 * n;
    const float* mas = slab + (size_t)9 * n;
    const float* pot = slab + (size_t)10 * n;
    float* ken = slab + (size_t)11 * n;
    float* pen = slab + (size_t)12 * n;
    ff e[4] = {ff{0.f, 0.f}, ff{0.f, 0.f}, ff{0.f, 0.f}, ff{0.f, 0.f}};
    if (i < n) {
        float v[3];
        double v64[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const size_t k = 3u * (size_t)i + c;
            if (vel64) {
                v64[c] = vel64[k] + 0.5 * dt64 * (double)acc[k];
                vel64[k] = v64[c];
                v[c] = (float)v64[c];
            } else {
                v[c] = fadd(vel[k], fmul(half_dt, acc[k]));  // simulation.c:424
                v64[c] = v[c];
            }
            vel[k] = v[c];
        }
        const float m = mas[i];
        // simulation.c:443-450
        const float v2 = fadd(fadd(fmul(v[0], v[0]), fmul(v[1], v[1])), fmul(v[2], v[2]));
        const float k_i = fmul(fmul(0.5f, m), v2);
        const float p_i = fmul(m, pot[i]);
        ken[i] = k_i;
        pen[i] = p_i;
        // corrected totals: kinetic term of the integrated dynamics and the
        // pair potential without self terms, each pair once (FP32 per body;
        // FP64 velocities in the precision form)
        if (vel64) {
            const double v2d = v64[0] * v64[0] + v64[1] * v64[1] + v64[2] * v64[2];
            e[2] = ff_from_double(physical ? 0.5 * (double)m * v2d : 0.5 * v2d);
        } else {
            e[2] = ff_from(physical ? fmul(fmul(0.5f, m), v2) : fmul(0.5f, v2));
        }
        const float selfp = fmul(g_over_eps, m);  // G m_i / eps (the j = i term)
        e[3] = ff_from(fmul(fmul(0.5f, m), fadd(pot[i], selfp)));
        e[0] = ff_from(k_i);
        e[1] = ff_from(p_i);
    }
    block_sum<4>(e, part);
    if (last_block(done)) {
        // simulation.c:455-497: T = sum ken, V = sum pen (FP64)
        sum_partials<4>(part, gridDim.x, sums);
        if (threadIdx.x == 0) *d_step += 1u;
    }
}

// Momentum diagnostics of the current state: P = sum m v and
// L = sum m (x cross v), per body in FP64 (from the FP64 state in the
// precision form), summed in float-float within warps and FP64 across
// warps and blocks in a fixed order (last-block pattern), into out[0..5].
__global__ void __launch_bounds__(SF_RED_BLOCK) k_momentum(const float* __restrict__ slab, uint32_t n,
                                                           const double* __restrict__ pos64,
                                                           const double* __restrict__ vel64,
                                                           double* __restrict__ part, uint32_t* done,
                                                           double* __restrict__ out) {
    const uint32_t i = blockIdx.x * SF_RED_BLOCK + threadIdx.x;
    ff r[6];
#pragma unroll
    for (int k = 0; k < 6; k++) r[k] = ff{0.0f, 0.0f};
    if (i < n) {
        double x[3], v[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const size_t q = 3u * (size_t)i + c;
            x[c] = pos64 ? pos64[q] : (double)slab[q];
            v[c] = vel64 ? vel64[q] : (double)slab[(size_t)3 * n + q];
        }
        const double m = (double)slab[(size_t)9 * n + i];
#pragma unroll
        for (int c = 0; c < 3; c++) r[c] = ff_from_double(m * v[c]);
        r[3] = ff_from_double(m * (x[1] * v[2] - x[2] * v[1]));
        r[4] = ff_from_double(m * (x[2] * v[0] - x[0] * v[2]));
        r[5] = ff_from_double(m * (x[0] * v[1] - x[1] * v[0]));
    }
    block_sum<6>(r, part);
    if (!last_block(done)) return;
    __shared__ double tot[6];
    sum_partials<6>(part, gridDim.x, tot);
    __syncthreads();
    if (threadIdx.x < 6) out[threadIdx.x] = tot[threadIdx.x];
}

}  // namespace

static int ensure_red(sfgpu_sim* s, uint32_t entries) {
    if (s->red_cap >= entries) return SFGPU_OK;
    cudaFree(s->red);
    s->red = nullptr;
    SF_CUDA(cudaMalloc(&s->red, sizeof(double2) * entries));
    s->red_cap = entries;
    return SFGPU_OK;
}

int sf_stage_kick_drift(sfgpu_sim* s, bool want_radius) {
    const uint32_t nb = sf_ceil_div(s->n, SF_RED_BLOCK);
    if (ensure_red(s, nb * 4) != SFGPU_OK) return SFGPU_FAILURE;
    const float dt = (float)s->p.dt;
    k_kick_drift<<<nb, SF_RED_BLOCK, 0, s->stream>>>(s->slab, s->n, 0.5f * dt, dt, s->pos64, s->vel64, s->p.dt,
                                                     want_radius ? 1 : 0, (double*)s->red, s->d_done, s->d_step, s->d_bounds,
                                                     s->sums, s->u, s->dudt);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

int sf_stage_radius(sfgpu_sim* s) {
    const uint32_t nb = sf_ceil_div(s->n, SF_RED_BLOCK);
    if (ensure_red(s, nb * 4) != SFGPU_OK) return SFGPU_FAILURE;
    k_radius<<<nb, SF_RED_BLOCK, 0, s->stream>>>(s->slab, s->n, (double*)s->red, s->d_done, s->d_step, s->d_bounds, s->sums);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

int sf_stage_kick_energy(sfgpu_sim* s) {
    const uint32_t nb = sf_ceil_div(s->n, SF_RED_BLOCK);
    if (ensure_red(s, nb * 4) != SFGPU_OK) return SFGPU_FAILURE;
    const float dt = (float)s->p.dt;
    const float g_over_eps = (float)(s->p.G / s->p.eps);
    k_kick_energy<<<nb, SF_RED_BLOCK, 0, s->stream>>>(s->slab, s->n, 0.5f * dt, s->vel64, s->p.dt, g_over_eps,
                                                      s->p.acc_mode == SFGPU_ACC_PHYSICAL, (double*)s->red, s->d_done + 1,
                                                      s->sums, s->d_step, s->u, s->dudt);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

// sums[8..10] = P, sums[11..13] = L; ticket d_done[2]
int sf_stage_momentum(sfgpu_sim* s) {
    const uint32_t nb = sf_ceil_div(s->n, SF_RED_BLOCK);
    if (ensure_red(s, nb * 6) != SFGPU_OK) return SFGPU_FAILURE;
    k_momentum<<<nb, SF_RED_BLOCK, 0, s->stream>>>(s->slab, s->n, s->pos64, s->vel64, (double*)s->red,
                                                   s->d_done + 2, s->sums + 8);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}
