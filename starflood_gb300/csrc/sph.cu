// sph.cu -- SPH, solve_sph (src/sph.c:14-282) and the cubic-spline form.
//
// SFGPU_SPH_REFERENCE restates the reference:
//   density   rho_i = sum_j (W_i + W_j)/2 m_j over all j (j = i included),
//             W_k = (1/(sqrt(pi) h_k))^3 exp(-r^2/h_k^2)          sph.c:35-145
//   pressure  P_i = (0.1 rho_i)^2                                  sph.c:148-159
//   momentum  acc_i += -m_i sum_{j: fl(r^2) <= 1} (c_i + c_j) g_ij r_ij,
//             c = P/rho^2 (0 if rho = 0), g = (n_i + n_j)/2,
//             n_k = -2 exp(-r^2/h_k^2) / (pi^1.5 h_k^5)            sph.c:172-277
// Both passes are j-tiles staged in shared memory (x, y, z, m | h, rho, P)
// with one body i per thread; the neighbour test uses the reference's FP32
// r^2 = (dx^2 + dy^2) + dz^2 with IEEE rounding, so the neighbour sets (the
// per-body counts are kept) are bit-identical.  The exponentials use expf,
// so densities and forces match the reference to FP32 rounding, not bits.
#include "internal.cuh"

namespace {

constexpr int SPH_BS = 128;
constexpr double K_INV_SQRT_PI = 0.56418958354775628694807945156077258584405062932900;  // common.h:24
constexpr double K_PI_1_5 = 5.56832799683170784528481798211883570201362439028324;       // common.h:29

struct SphWork {
    uint32_t* nbr = nullptr;  // momentum-pass neighbour counts per body
};

__global__ void __launch_bounds__(SPH_BS) k_sph_density(const float* __restrict__ pos, const float* __restrict__ mas,
                                                        const float* __restrict__ rad, uint32_t n, int exact,
                                                        float* __restrict__ rho) {
    __shared__ float4 sj[SPH_BS];
    __shared__ float sh[SPH_BS];
    const uint32_t i = blockIdx.x * SPH_BS + threadIdx.x;
    const bool live = i < n;
    const float xi = live ? pos[3u * i] : 0.f, yi = live ? pos[3u * i + 1u] : 0.f, zi = live ? pos[3u * i + 2u] : 0.f;
    const float hi = live ? rad[i] : 1.f;
    const float inv_sqrt_pi = (float)K_INV_SQRT_PI;
    const float ai = fdiv(inv_sqrt_pi, hi);
    const float ai3 = fmul(fmul(ai, ai), ai);
    const float hi2 = fmul(hi, hi);
    KSum s{0.f, 0.f};
    float hsum = 0.f, lsum = 0.f;  // FAST: per-tile sums folded with two-sum
    for (uint32_t jt = 0; jt < n; jt += SPH_BS) {
        const uint32_t j = jt + threadIdx.x;
        __syncthreads();
        if (j < n) {
            sj[threadIdx.x] = make_float4(pos[3u * j], pos[3u * j + 1u], pos[3u * j + 2u], mas[j]);
            sh[threadIdx.x] = rad[j];
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)SPH_BS, n - jt);
        float t = 0.f;
        for (uint32_t jj = 0; jj < cnt; jj++) {
            const float4 q = sj[jj];
            const float hj = sh[jj];
            const float dx = fsub(xi, q.x), dy = fsub(yi, q.y), dz = fsub(zi, q.z);
            const float r2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
            const float aj = fdiv(inv_sqrt_pi, hj);
            const float wi = fmul(ai3, expf(fdiv(-r2, hi2)));
            const float wj = fmul(fmul(fmul(aj, aj), aj), expf(fdiv(-r2, fmul(hj, hj))));
            const float c = fmul(fmul(0.5f, fadd(wi, wj)), q.w);
            if (exact) s.add(c);
            else t += c;
        }
        if (!exact) {
            float e;
            two_sumf(hsum, t, hsum, e);
            lsum += e;
        }
    }
    if (live) rho[i] = exact ? s.s : hsum + lsum;
}

// sph.c:148-159: powf(0.1 rho, 2) is the correctly rounded square
__global__ void k_sph_eos(const float* __restrict__ rho, uint32_t n, float* __restrict__ prs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float t = fmul(0.1f, rho[i]);
    prs[i] = fmul(t, t);
}

__global__ void __launch_bounds__(SPH_BS) k_sph_momentum(const float* __restrict__ pos, const float* __restrict__ mas,
                                                         const float* __restrict__ rad, const float* __restrict__ rho,
                                                         const float* __restrict__ prs, uint32_t n, int exact,
                                                         float* __restrict__ acc, uint32_t* __restrict__ nbr) {
    __shared__ float4 sj[SPH_BS];
    __shared__ float4 sq[SPH_BS];  // (h, con, -, -)
    const uint32_t i = blockIdx.x * SPH_BS + threadIdx.x;
    const bool live = i < n;
    const float xi = live ? pos[3u * i] : 0.f, yi = live ? pos[3u * i + 1u] : 0.f, zi = live ? pos[3u * i + 2u] : 0.f;
    const float hi = live ? rad[i] : 1.f;
    const float rhoi = live ? rho[i] : 0.f;
    const float rhoi2 = fmul(rhoi, rhoi);
    const float ci = (0.0f < rhoi2) ? fdiv(live ? prs[i] : 0.f, rhoi2) : 0.0f;
    const float pi15 = (float)K_PI_1_5;
    const float hi2 = fmul(hi, hi);
    const float den_i = fmul(fmul(fmul(fmul(fmul(pi15, hi), hi), hi), hi), hi);
    KSum ax{0.f, 0.f}, ay{0.f, 0.f}, az{0.f, 0.f};
    uint32_t count = 0;
    for (uint32_t jt = 0; jt < n; jt += SPH_BS) {
        const uint32_t j = jt + threadIdx.x;
        __syncthreads();
        if (j < n) {
            sj[threadIdx.x] = make_float4(pos[3u * j], pos[3u * j + 1u], pos[3u * j + 2u], mas[j]);
            const float rj = rho[j];
            const float rj2 = fmul(rj, rj);
            sq[threadIdx.x] = make_float4(rad[j], (0.0f < rj2) ? fdiv(prs[j], rj2) : 0.0f, 0.f, 0.f);
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)SPH_BS, n - jt);
        for (uint32_t jj = 0; jj < cnt; jj++) {
            const float4 q = sj[jj];
            const float dx = fsub(xi, q.x), dy = fsub(yi, q.y), dz = fsub(zi, q.z);
            const float r2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
            if (r2 > 1.0f) continue;  // sph.c:231
            count++;
            const float4 e = sq[jj];
            const float hj = e.x;
            const float den_j = fmul(fmul(fmul(fmul(fmul(pi15, hj), hj), hj), hj), hj);
            const float ni = fdiv(fmul(-2.0f, expf(fdiv(-r2, hi2))), den_i);
            const float nj = fdiv(fmul(-2.0f, expf(fdiv(-r2, fmul(hj, hj)))), den_j);
            const float g = fmul(0.5f, fadd(ni, nj));
            const float cc = fadd(ci, e.y);
            const float fx = fmul(cc, fmul(g, dx)), fy = fmul(cc, fmul(g, dy)), fz = fmul(cc, fmul(g, dz));
            if (exact) {
                ax.add(fx);
                ay.add(fy);
                az.add(fz);
            } else {
                ax.s += fx;
                ay.s += fy;
                az.s += fz;
            }
        }
    }
    if (!live) return;
    const float mi = mas[i];
    // sph.c:274-276: acc += -m_i * sum
    acc[3u * i + 0u] = fadd(acc[3u * i + 0u], fmul(-mi, ax.s));
    acc[3u * i + 1u] = fadd(acc[3u * i + 1u], fmul(-mi, ay.s));
    acc[3u * i + 2u] = fadd(acc[3u * i + 2u], fmul(-mi, az.s));
    if (nbr) nbr[i] = count;
}

}  // namespace

int sf_sph_cubic_alloc(sfgpu_sim* s);
void sf_sph_cubic_free(sfgpu_sim* s);
int sf_sph_cubic(sfgpu_sim* s);

int sf_sph_alloc(sfgpu_sim* s) {
    SphWork* w = new SphWork();
    s->sph = w;
    SF_CUDA(cudaMalloc(&w->nbr, sizeof(uint32_t) * std::max<uint32_t>(s->n, 1)));
    SF_CUDA(cudaMemset(w->nbr, 0, sizeof(uint32_t) * std::max<uint32_t>(s->n, 1)));
    if (s->p.sph == SFGPU_SPH_CUBIC) return sf_sph_cubic_alloc(s);
    return SFGPU_OK;
}

void sf_sph_free(sfgpu_sim* s) {
    SphWork* w = (SphWork*)s->sph;
    if (!w) return;
    if (s->p.sph == SFGPU_SPH_CUBIC) sf_sph_cubic_free(s);
    cudaFree(w->nbr);
    delete w;
    s->sph = nullptr;
}

uint32_t* sf_sph_neighbour_counts(sfgpu_sim* s) { return s->sph ? ((SphWork*)s->sph)->nbr : nullptr; }

int sf_stage_sph(sfgpu_sim* s) {
    if (s->p.sph == SFGPU_SPH_CUBIC) return sf_sph_cubic(s);
    const uint32_t n = s->n;
    float* slab = s->slab;
    const float* pos = slab;
    float* acc = slab + (size_t)6 * n;
    const float* mas = slab + (size_t)9 * n;
    const float* rad = slab + (size_t)13 * n;
    float* rho = slab + (size_t)14 * n;
    float* prs = slab + (size_t)15 * n;
    const int exact = s->p.math == SFGPU_MATH_EXACT ? 1 : 0;
    const uint32_t grid = sf_ceil_div(n, SPH_BS);
    k_sph_density<<<grid, SPH_BS, 0, s->stream>>>(pos, mas, rad, n, exact, rho);
    SF_CHECK_LAUNCH();
    k_sph_eos<<<sf_ceil_div(n, 256), 256, 0, s->stream>>>(rho, n, prs);
    SF_CHECK_LAUNCH();
    k_sph_momentum<<<grid, SPH_BS, 0, s->stream>>>(pos, mas, rad, rho, prs, n, exact, acc,
                                                   ((SphWork*)s->sph)->nbr);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}
