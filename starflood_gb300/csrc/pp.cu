// pp.cu -- O(N^2) softened gravity, solve_gravity_part_part
// (src/gravity.c:666-819), three ways:
//
//   k_pp_exact  one thread per body, every j in index order, the reference's
//               FP32 expression tree with IEEE divide / square root and a
//               Kahan sum per component (bit-identical to the reference);
//   k_pp_tile2  j-tiles staged in shared memory and broadcast to the warp,
//               8 bodies per thread in registers on paired FP32 instructions
//               (fma/add/mul.f32x2), hardware rsqrt and reciprocal;
//               the j range is split over blockIdx.y so the grid covers the
//               152 SMs several times, partial sums land in a scratch array
//               and a second kernel adds them in a fixed order;
//   compensated the same tiles, but the partial sum of every four j-tiles
//               is added to a (hi, lo) pair with a paired two-sum (the
//               precision form), and the split partials are added in FP64.
#include <algorithm>

#include "internal.cuh"

namespace {

// ---- exact ----------------------------------------------------------------
constexpr int EXACT_BS = 128;

__global__ void __launch_bounds__(EXACT_BS) k_pp_exact(const float* __restrict__ pos, const float* __restrict__ mas,
                                                       uint32_t n, ForceConsts fc, float* __restrict__ acc,
                                                       float* __restrict__ pot) {
    __shared__ float4 sj[EXACT_BS];
    const uint32_t i = blockIdx.x * EXACT_BS + threadIdx.x;
    const bool live = i < n;
    const float xi = live ? pos[3u * i] : 0.f;
    const float yi = live ? pos[3u * i + 1u] : 0.f;
    const float zi = live ? pos[3u * i + 2u] : 0.f;
    const float mi = live ? mas[i] : 0.f;
    KSum ax{0.f, 0.f}, ay{0.f, 0.f}, az{0.f, 0.f}, ph{0.f, 0.f};
    for (uint32_t jt = 0; jt < n; jt += EXACT_BS) {
        const uint32_t j = jt + threadIdx.x;
        __syncthreads();
        if (j < n) sj[threadIdx.x] = make_float4(pos[3u * j], pos[3u * j + 1u], pos[3u * j + 2u], mas[j]);
        __syncthreads();
        const uint32_t cnt = min((uint32_t)EXACT_BS, n - jt);
        for (uint32_t jj = 0; jj < cnt; jj++) {
            const float4 q = sj[jj];
            // gravity.c:744-769: r_ij = r_i - r_j, r2 = (x^2 + y^2) + z^2
            const float dx = fsub(xi, q.x), dy = fsub(yi, q.y), dz = fsub(zi, q.z);
            const float r2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
            const float s = fadd(r2, fc.eps2);
            const float inv2 = fdiv(1.0f, s);
            const float inv1 = fdiv(1.0f, fsqrt(s));
            const float phi = fmul(q.w, inv1);
            const float f = fmul(phi, inv2);
            ax.add(fmul(f, dx));
            ay.add(fmul(f, dy));
            az.add(fmul(f, dz));
            ph.add(phi);
        }
    }
    if (!live) return;
    // gravity.c:808-811: acc = (-G) * m_i * sum, pot = (-G) * sum
    const float scale = fc.physical ? fc.neg_g : fmul(fc.neg_g, mi);
    acc[3u * i + 0u] = fmul(scale, ax.s);
    acc[3u * i + 1u] = fmul(scale, ay.s);
    acc[3u * i + 2u] = fmul(scale, az.s);
    pot[i] = fmul(fc.neg_g, ph.s);
}

// ---- fast / compensated ---------------------------------------------------
// Each thread owns IPT bodies i = ibase + k*BS + tid.  The sum accumulated is
// S_i = sum_j m_j (r_j - r_i) / (r^2 + eps^2)^1.5 = -sum_j F_ij, so the
// reference's acc = (-G) m_i sum F = G m_i S.
template <int BS, int IPT, bool COMP>
__global__ void __launch_bounds__(BS) k_pp_tile(const float* __restrict__ pos, const float* __restrict__ mas,
                                                const double* __restrict__ pos64, uint32_t n, float eps2,
                                                uint32_t jchunk, float4* __restrict__ part) {
    __shared__ float4 sj[BS];
    const uint32_t ibase = blockIdx.x * (BS * IPT);
    float xi[IPT], yi[IPT], zi[IPT];
    float ax[IPT], ay[IPT], az[IPT], ph[IPT];
    float hx[IPT], hy[IPT], hz[IPT], hp[IPT];  // compensated totals
    float lx[IPT], ly[IPT], lz[IPT], lp[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        const uint32_t i = ibase + k * BS + threadIdx.x;
        const bool live = i < n;
        xi[k] = live ? pos[3u * i] : 0.f;
        yi[k] = live ? pos[3u * i + 1u] : 0.f;
        zi[k] = live ? pos[3u * i + 2u] : 0.f;
        ax[k] = ay[k] = az[k] = ph[k] = 0.f;
        hx[k] = hy[k] = hz[k] = hp[k] = 0.f;
        lx[k] = ly[k] = lz[k] = lp[k] = 0.f;
    }
    const uint32_t j0 = blockIdx.y * jchunk;
    const uint32_t j1 = min(n, j0 + jchunk);
    for (uint32_t jt = j0; jt < j1; jt += BS) {
        const uint32_t j = jt + threadIdx.x;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);  // padding: zero mass
        if (j < j1) q = make_float4(pos[3u * j], pos[3u * j + 1u], pos[3u * j + 2u], mas[j]);
        __syncthreads();
        sj[threadIdx.x] = q;
        __syncthreads();
#pragma unroll 8
        for (int jj = 0; jj < BS; jj++) {
            const float4 s = sj[jj];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                const float dx = s.x - xi[k];
                const float dy = s.y - yi[k];
                const float dz = s.z - zi[k];
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                const float inv = rsqrtf(r2);
                const float mphi = s.w * inv;
                const float f = mphi * (inv * inv);
                ax[k] = fmaf(f, dx, ax[k]);
                ay[k] = fmaf(f, dy, ay[k]);
                az[k] = fmaf(f, dz, az[k]);
                ph[k] += mphi;
            }
        }
        if (COMP) {
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                float e;
                two_sumf(hx[k], ax[k], hx[k], e); lx[k] += e;
                two_sumf(hy[k], ay[k], hy[k], e); ly[k] += e;
                two_sumf(hz[k], az[k], hz[k], e); lz[k] += e;
                two_sumf(hp[k], ph[k], hp[k], e); lp[k] += e;
                ax[k] = ay[k] = az[k] = ph[k] = 0.f;
            }
        }
    }
    float4* out = part + (size_t)blockIdx.y * n * (COMP ? 2 : 1);
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        const uint32_t i = ibase + k * BS + threadIdx.x;
        if (i >= n) continue;
        if (COMP) {
            out[i] = make_float4(hx[k], hy[k], hz[k], hp[k]);
            out[(size_t)n + i] = make_float4(lx[k], ly[k], lz[k], lp[k]);
        } else {
            out[i] = make_float4(ax[k], ay[k], az[k], ph[k]);
        }
    }
    (void)pos64;
}

// The same tile loop on Blackwell's paired FP32 instructions (fma/add/mul
// .f32x2): two bodies per instruction, so one issue slot does two lanes'
// worth of FP32 work and the rsqrt (MUFU) and shared-memory loads no longer
// compete with the arithmetic for issue.  Every element is rounded exactly as
// in k_pp_tile (same operations, same order), so the results are identical.
// Each j is staged pre-duplicated as (x,x,y,y) and (z,z,w,w) so the paired
// operands come straight out of one 128-bit shared load.
// Paired two-sum (Knuth) on both elements: (h, l) += a, error term into l.
__device__ __forceinline__ void two_sum2(float2& h, float2 a, float2& l) {
    const float2 s = __fadd2_rn(h, a);
    const float2 bp = __fadd2_rn(s, make_float2(-h.x, -h.y));
    const float2 ap = __fadd2_rn(s, make_float2(-bp.x, -bp.y));
    const float2 e = __fadd2_rn(__fadd2_rn(h, make_float2(-ap.x, -ap.y)), __fadd2_rn(a, make_float2(-bp.x, -bp.y)));
    h = s;
    l = __fadd2_rn(l, e);
}
// The same on a (hi, lo) total kept in shared memory.
__device__ __forceinline__ void two_sum2_at(float2* hs, float2* ls, float2 a) {
    float2 h = *hs, l = *ls;
    two_sum2(h, a, l);
    *hs = h;
    *ls = l;
}

// j-tiles the compensated form sums plainly before each two-sum: 1024
// bodies, whose FP32 partial sum is far inside the 1e-6 bound (its error is
// a few ulps of a partial ~1/1000 of the total at N = 1,048,576).
constexpr int COMP_TILES = 8;

template <int BS, int PAIRS, bool COMP, int RSQ = 0, int MINB = 1>
__global__ void __launch_bounds__(BS, MINB) k_pp_tile2(const float* __restrict__ pos, const float* __restrict__ mas,
                                                 uint32_t n, float eps2, uint32_t jchunk,
                                                 float4* __restrict__ part) {
    __shared__ float4 sj[2][BS];
    // compensated totals, (hi, lo) of x, y, z, potential per pair of bodies,
    // in shared memory: touched once every COMP_TILES tiles, they would
    // otherwise take 8 registers per pair from the tile loop (and spill at
    // the 64-register budget of 8 blocks per SM)
    __shared__ float2 s_tot[COMP ? 8 * PAIRS : 1][COMP ? BS : 1];
    const uint32_t ibase = blockIdx.x * (BS * 2 * PAIRS);
    float2 nx[PAIRS], ny[PAIRS], nz[PAIRS];
    float2 ax[PAIRS], ay[PAIRS], az[PAIRS], ph[PAIRS];
    const float2 zero2 = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < PAIRS; q++) {
        const uint32_t i0 = ibase + (2 * q) * BS + threadIdx.x;
        const uint32_t i1 = i0 + BS;
        nx[q] = make_float2(i0 < n ? -pos[3u * i0] : 0.f, i1 < n ? -pos[3u * i1] : 0.f);
        ny[q] = make_float2(i0 < n ? -pos[3u * i0 + 1u] : 0.f, i1 < n ? -pos[3u * i1 + 1u] : 0.f);
        nz[q] = make_float2(i0 < n ? -pos[3u * i0 + 2u] : 0.f, i1 < n ? -pos[3u * i1 + 2u] : 0.f);
        ax[q] = ay[q] = az[q] = ph[q] = zero2;
        if (COMP)
#pragma unroll
            for (int c = 0; c < 8; c++) s_tot[8 * q + c][threadIdx.x] = zero2;
    }
    const float2 e2 = make_float2(eps2, eps2);
    const uint32_t j0 = blockIdx.y * jchunk;
    const uint32_t j1 = min(n, j0 + jchunk);
    // the compensated form runs the plain tile loop over spans of
    // COMP_TILES tiles and adds each span's partial sums into the (hi, lo)
    // totals with a paired two-sum (the plain form: one span)
    const uint32_t span = COMP ? (uint32_t)(BS * COMP_TILES) : j1 - j0;
    for (uint32_t js = j0; js < j1; js += span) {
        const uint32_t je = min(j1, js + span);
        for (uint32_t jt = js; jt < je; jt += BS) {
            const uint32_t j = jt + threadIdx.x;
            float x = 0.f, y = 0.f, z = 0.f, w = 0.f;  // padding: zero mass
            if (j < j1) {
                x = pos[3u * j];
                y = pos[3u * j + 1u];
                z = pos[3u * j + 2u];
                w = mas[j];
            }
            __syncthreads();
            sj[0][threadIdx.x] = make_float4(x, x, y, y);
            sj[1][threadIdx.x] = make_float4(z, z, w, w);
            __syncthreads();
#pragma unroll 8
            for (int jj = 0; jj < BS; jj++) {
                const float4 A = sj[0][jj];
                const float4 B = sj[1][jj];
                const float2 sx = make_float2(A.x, A.y), sy = make_float2(A.z, A.w);
                const float2 sz = make_float2(B.x, B.y), sw = make_float2(B.z, B.w);
#pragma unroll
                for (int q = 0; q < PAIRS; q++)
                    pp_pair_step<RSQ>(sx, sy, sz, sw, nx[q], ny[q], nz[q], e2, ax[q], ay[q], az[q], ph[q]);
            }
        }
        if (COMP) {
#pragma unroll
            for (int q = 0; q < PAIRS; q++) {
                float2* t = &s_tot[8 * q][threadIdx.x];  // rows 8q + (0..3 hi x y z p, 4..7 lo)
                two_sum2_at(t, t + 4 * BS, ax[q]);
                two_sum2_at(t + BS, t + 5 * BS, ay[q]);
                two_sum2_at(t + 2 * BS, t + 6 * BS, az[q]);
                two_sum2_at(t + 3 * BS, t + 7 * BS, ph[q]);
                ax[q] = ay[q] = az[q] = ph[q] = zero2;
            }
        }
    }
    float4* out = part + (size_t)blockIdx.y * n * (COMP ? 2 : 1);
#pragma unroll
    for (int q = 0; q < PAIRS; q++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const uint32_t i = ibase + (2 * q + h) * BS + threadIdx.x;
            if (i >= n) continue;
            if (COMP) {
                float2 v[8];
#pragma unroll
                for (int c = 0; c < 8; c++) v[c] = s_tot[8 * q + c][threadIdx.x];
                out[i] = h ? make_float4(v[0].y, v[1].y, v[2].y, v[3].y) : make_float4(v[0].x, v[1].x, v[2].x, v[3].x);
                out[(size_t)n + i] = h ? make_float4(v[4].y, v[5].y, v[6].y, v[7].y)
                                       : make_float4(v[4].x, v[5].x, v[6].x, v[7].x);
            } else {
                out[i] = h ? make_float4(ax[q].y, ay[q].y, az[q].y, ph[q].y)
                           : make_float4(ax[q].x, ay[q].x, az[q].x, ph[q].x);
            }
        }
    }
}

template <bool COMP>
__global__ void k_pp_reduce(const float4* __restrict__ part, uint32_t n, uint32_t nsplit,
                            const float* __restrict__ mas, ForceConsts fc, float* __restrict__ acc,
                            float* __restrict__ pot) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = -fc.neg_g;
    const float mi = mas[i];
    if (!COMP) {
        float4 s = part[i];
        for (uint32_t b = 1; b < nsplit; b++) {
            const float4 t = part[(size_t)b * n + i];
            s.x += t.x; s.y += t.y; s.z += t.z; s.w += t.w;
        }
        const float scale = fc.physical ? g : g * mi;
        acc[3u * i + 0u] = scale * s.x;
        acc[3u * i + 1u] = scale * s.y;
        acc[3u * i + 2u] = scale * s.z;
        pot[i] = fc.neg_g * s.w;
    } else {
        double sx = 0, sy = 0, sz = 0, sw = 0;
        for (uint32_t b = 0; b < nsplit; b++) {
            const float4 h = part[(size_t)b * 2 * n + i];
            const float4 l = part[(size_t)b * 2 * n + n + i];
            sx += (double)h.x + (double)l.x;
            sy += (double)h.y + (double)l.y;
            sz += (double)h.z + (double)l.z;
            sw += (double)h.w + (double)l.w;
        }
        const double scale = fc.physical ? (double)g : (double)g * (double)mi;
        acc[3u * i + 0u] = (float)(scale * sx);
        acc[3u * i + 1u] = (float)(scale * sy);
        acc[3u * i + 2u] = (float)(scale * sz);
        pot[i] = (float)((double)fc.neg_g * sw);
    }
}

// The production tile: 128 threads, 2 pairs (4 bodies) per thread at 64
// registers, 8 blocks (32 warps) per SM, rsqrt and 1/r^2 both from the MUFU
// (one FP32 multiply fewer per interaction: the FMA pipe is the bound),
// the j range split for about 16 waves.  Measured at N = 1,048,576 on GB300
// (CUDA events, one launch): 2.366e12 interactions/s plain and 2.33e12
// with the compensation every 4 tiles, against 2.253e12 for 4 pairs per
// thread at 128 registers (16 warps per SM, 8 waves), 2.36e12 for 1 pair
// at 32 registers, 2.28e12 for 3 pairs, and 1.92e12 for the scalar
// k_pp_tile<128,4>.
constexpr int FAST_BS = 128;
constexpr int FAST_PAIRS = 2;
constexpr int FAST_IPT = 2 * FAST_PAIRS;
constexpr int FAST_RSQ = 2;
constexpr int FAST_MINB = 8;
constexpr uint32_t FAST_WAVES = 16;

void launch_pp_tiles(bool comp, dim3 grid, const float* pos, const float* mas, uint32_t n, float eps2,
                     uint32_t jchunk, float4* part, cudaStream_t st) {
    if (comp) {
        // 8 blocks of 20 KB (tiles + totals) per SM: ask for the largest
        // shared-memory carve-out
        static bool carve = false;
        if (!carve) {
            cudaFuncSetAttribute(k_pp_tile2<FAST_BS, FAST_PAIRS, true, FAST_RSQ, FAST_MINB>,
                                 cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
            carve = true;
        }
        k_pp_tile2<FAST_BS, FAST_PAIRS, true, FAST_RSQ, FAST_MINB><<<grid, FAST_BS, 0, st>>>(pos, mas, n, eps2,
                                                                                           jchunk, part);
    }
    else
        k_pp_tile2<FAST_BS, FAST_PAIRS, false, FAST_RSQ, FAST_MINB><<<grid, FAST_BS, 0, st>>>(pos, mas, n, eps2,
                                                                                            jchunk, part);
}

}  // namespace

ForceConsts sf_force_consts(const sfgpu_params& p) {
    ForceConsts c;
    c.eps2 = (float)(p.eps * p.eps);
    c.neg_g = (float)(-p.G);
    c.theta = (float)p.theta;
    c.third = (float)(1.0 / 3.0);
    c.physical = p.acc_mode == SFGPU_ACC_PHYSICAL;
    c.walk_limit = p.walk_limit ? p.walk_limit : (1u << 24);
    return c;
}

namespace {
struct PPShape {
    uint32_t iblocks, nsplit, jchunk;
};
PPShape pp_shape(uint32_t n) {
    PPShape sh;
    sh.iblocks = sf_ceil_div(n, FAST_BS * FAST_IPT);
    // enough blocks for ~FAST_WAVES waves at FAST_MINB resident blocks per SM
    const uint32_t target = (uint32_t)sf_num_sms() * (uint32_t)FAST_MINB * FAST_WAVES;
    uint32_t nsplit = std::max<uint32_t>(1u, sf_ceil_div(target, sh.iblocks));
    uint32_t jchunk = sf_ceil_div(n, nsplit);
    jchunk = sf_ceil_div(jchunk, FAST_BS) * FAST_BS;
    sh.jchunk = jchunk;
    sh.nsplit = sf_ceil_div(n, jchunk);
    return sh;
}
}  // namespace

size_t sf_pp_scratch_need(const sfgpu_params& p, uint32_t n) {
    if (n == 0 || (p.math == SFGPU_MATH_EXACT && p.form == SFGPU_FORM_PLAIN)) return 0;
    const PPShape sh = pp_shape(n);
    return (size_t)sh.nsplit * n * (p.form == SFGPU_FORM_COMPENSATED ? 2 : 1);
}

int sf_pp_launch(const sfgpu_params& p, uint32_t n, const float* pos, const float* mas, float* acc, float* pot,
                 float4** part, size_t* part_cap, cudaStream_t st, const double* pos64) {
    if (n == 0) return SFGPU_OK;
    const ForceConsts fc = sf_force_consts(p);
    if (p.math == SFGPU_MATH_EXACT && p.form == SFGPU_FORM_PLAIN) {
        k_pp_exact<<<sf_ceil_div(n, EXACT_BS), EXACT_BS, 0, st>>>(pos, mas, n, fc, acc, pot);
        SF_CHECK_LAUNCH();
        return SFGPU_OK;
    }
    const bool comp = p.form == SFGPU_FORM_COMPENSATED;
    const PPShape sh = pp_shape(n);
    const uint32_t iblocks = sh.iblocks, nsplit = sh.nsplit, jchunk = sh.jchunk;
    const size_t need = sf_pp_scratch_need(p, n);
    if (*part_cap < need) {
        cudaFree(*part);
        *part = nullptr;
        *part_cap = 0;
        SF_CUDA(cudaMalloc(part, need * sizeof(float4)));
        *part_cap = need;
    }
    dim3 grid(iblocks, nsplit);
    launch_pp_tiles(comp, grid, pos, mas, n, fc.eps2, jchunk, *part, st);
    (void)pos64;
    SF_CHECK_LAUNCH();
    if (comp)
        k_pp_reduce<true><<<sf_ceil_div(n, 256), 256, 0, st>>>(*part, n, nsplit, mas, fc, acc, pot);
    else
        k_pp_reduce<false><<<sf_ceil_div(n, 256), 256, 0, st>>>(*part, n, nsplit, mas, fc, acc, pot);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

int sf_stage_gravity_pp(sfgpu_sim* s) {
    float* acc = s->slab + (size_t)6 * s->n;
    float* pot = s->slab + (size_t)10 * s->n;
    return sf_pp_launch(s->p, s->n, s->slab, s->slab + (size_t)9 * s->n, acc, pot, &s->pp_part, &s->pp_part_cap,
                        s->stream, s->pos64);
}

// ---------------------------------------------------------------------------
// PP force without allocation (sfgpu_gravity_pp_noalloc).
//
// For callers that cannot call cudaMalloc: the j-split partial sums that
// sfgpu_gravity_pp keeps in a cudaMalloc'd work buffer live instead in the
// file-scope array below, 16 MiB (NOALLOC_PARTS float4 entries), which every
// GPU that loads this library holds until the process exits.  The number of
// j-splits is lowered until the partials fit; N above NOALLOC_PARTS (plain
// form) or NOALLOC_PARTS/2 (compensated form) is rejected.  Nothing in the
// array needs clearing between calls: every partial that the reduction reads
// is written by the same call first.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {
constexpr size_t NOALLOC_PARTS = (size_t)1 << 20;
static __device__ __align__(256) float4 g_noalloc_parts[NOALLOC_PARTS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
float4* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {nullptr};

// Device address of g_noalloc_parts on the current device: looked up once
// per device (the host-side symbol is not a device address).
int noalloc_parts(float4** out) {
    int dev = 0;
    SF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        sf_set_error("sfgpu_gravity_pp_noalloc: device %d out of range", dev);
        return SFGPU_FAILURE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        SF_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_parts));
        g_noalloc_ptr[dev] = (float4*)ptr;
    }
    *out = g_noalloc_ptr[dev];
    return SFGPU_OK;
}
}  // namespace

extern "C" int sfgpu_gravity_pp_noalloc(const sfgpu_params* p, uint32_t n, const float* pos, const float* mas,
                                        float* acc, float* pot, void* stream) {
    sf_clear_error();
    if (!p) {
        sf_set_error("sfgpu_gravity_pp_noalloc: params is NULL");
        return SFGPU_FAILURE;
    }
    if (!(p->eps > 0.0)) {
        sf_set_error("sfgpu_gravity_pp_noalloc: eps must be > 0");
        return SFGPU_FAILURE;
    }
    if (p->math == SFGPU_MATH_EXACT && p->form == SFGPU_FORM_COMPENSATED) {
        sf_set_error("sfgpu_gravity_pp_noalloc: EXACT math applies to the PLAIN form only");
        return SFGPU_FAILURE;
    }
    if (n == 0) return SFGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const ForceConsts fc = sf_force_consts(*p);
    if (p->math == SFGPU_MATH_EXACT) {  // needs no work array at all, so no size limit
        k_pp_exact<<<sf_ceil_div(n, EXACT_BS), EXACT_BS, 0, st>>>(pos, mas, n, fc, acc, pot);
        SF_CHECK_LAUNCH();
        return SFGPU_OK;
    }
    const bool comp = p->form == SFGPU_FORM_COMPENSATED;
    const size_t per_split = (size_t)n * (comp ? 2 : 1);
    if (per_split > NOALLOC_PARTS) {
        sf_set_error("sfgpu_gravity_pp_noalloc: N = %u exceeds the maximum of %zu bodies (%s form) of the "
                     "built-in %zu MiB work array",
                     n, comp ? NOALLOC_PARTS / 2 : NOALLOC_PARTS, comp ? "compensated" : "plain",
                     (NOALLOC_PARTS * sizeof(float4)) >> 20);
        return SFGPU_FAILURE;
    }
    float4* parts = nullptr;
    if (noalloc_parts(&parts) != SFGPU_OK) return SFGPU_FAILURE;
    const PPShape sh = pp_shape(n);
    uint32_t nsplit = std::min<uint32_t>(sh.nsplit, (uint32_t)(NOALLOC_PARTS / per_split));
    uint32_t jchunk = sf_ceil_div(sf_ceil_div(n, nsplit), FAST_BS) * FAST_BS;
    nsplit = sf_ceil_div(n, jchunk);
    dim3 grid(sh.iblocks, nsplit);
    launch_pp_tiles(comp, grid, pos, mas, n, fc.eps2, jchunk, parts, st);
    SF_CHECK_LAUNCH();
    if (comp)
        k_pp_reduce<true><<<sf_ceil_div(n, 256), 256, 0, st>>>(parts, n, nsplit, mas, fc, acc, pot);
    else
        k_pp_reduce<false><<<sf_ceil_div(n, 256), 256, 0, st>>>(parts, n, nsplit, mas, fc, acc, pot);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}
