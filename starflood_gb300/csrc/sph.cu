// sph.cu -- SPH, solve_sph (src/sph.c:14-282) and the cubic-spline form.
//
// SFGPU_SPH_REFERENCE restates the reference:
//   density   rho_i = sum_j (W_i + W_j)/2 m_j over all j (j = i included),
//             W_k = (1/(sqrt(pi) h_k))^3 exp(-r^2/h_k^2)          sph.c:35-145
//   pressure  P_i = (0.1 rho_i)^2                                  sph.c:148-159
//   momentum  acc_i += -m_i sum_{j: fl(r^2) <= 1} (c_i + c_j) g_ij r_ij,
//             c = P/rho^2 (0 if rho = 0), g = (n_i + n_j)/2,
//             n_k = -2 exp(-r^2/h_k^2) / (pi^1.5 h_k^5)            sph.c:172-277
// The neighbour test is the reference's FP32 r^2 = (dx^2 + dy^2) + dz^2
// with IEEE rounding, so the momentum pass's neighbour sets are the
// reference's, bit for bit (each body's set is returned as a count and an
// order-independent hash of its members).
//
// EXACT arithmetic keeps the reference's order: all pairs j = 0..N-1 in
// index order with Kahan sums (j-tiles staged in shared memory, one body i
// per thread).
//
// FAST arithmetic finds the neighbours through a sorted cell grid of side
// 1/4 (the momentum radius is 1, so a body's set lies within 4 cells on
// every axis).  Per body, each cell within reach is classified by its box
// distance: beyond the radius (skipped), inside it (its bodies join the set
// whole: count from the cell's run of sorted slots, hash from a per-cell
// sum), or straddling it (each pair tested with the reference's FP32
// expression).  Pair terms are evaluated only where exp(-r^2/h^2) can be a
// normal FP32 number: r^2 < 88 h_max^2 (exp(-88) < FLT_MIN), so the terms
// left out are subnormal or zero.  The density uses the same grid with that
// cutoff as its radius when it reaches at most 4 cells (h_max <= 0.107),
// else the all-pairs tiles.
#include "internal.cuh"
#include "chunks.cuh"
#include "sph_grid.cuh"

namespace {

using namespace sfgrid;

constexpr int SPH_BS = 128;
constexpr double K_INV_SQRT_PI = 0.56418958354775628694807945156077258584405062932900;  // common.h:24
constexpr double K_PI_1_5 = 5.56832799683170784528481798211883570201362439028324;       // common.h:29
constexpr float GRID_SIDE = 0.25f;  // momentum radius 1 = 4 cells
constexpr float GRID_INV = 4.0f;
constexpr int SET_REACH = 4;
constexpr float EXP_CUT = 88.0f;    // exp(-88) < FLT_MIN = 2^-126
constexpr float MARGIN_LO = 1.0f - 1.0f / 1024.0f, MARGIN_HI = 1.0f + 1.0f / 1024.0f;

struct SphWork {
    uint32_t* nbr = nullptr;   // momentum-pass neighbour counts per body
    uint64_t* hash = nullptr;  // and their set hashes (SFGPU_FLAG_STATS)
    // cell grid (FAST)
    uint32_t tbits = 0, tsize = 0;
    uint64_t* keys = nullptr;
    uint32_t* vals = nullptr;
    SortWork sort;
    uint32_t* bstart = nullptr;
    uint32_t* bend = nullptr;
    uint32_t* bmix = nullptr;   // bucket holds more than one cell
    uint64_t* bhash = nullptr;  // per bucket: sum of the members' hashes
    uint64_t* cell = nullptr;   // sorted packed cell keys
    float4* px = nullptr;       // sorted x, y, z, m
    float2* pq = nullptr;       // sorted h, c = P / rho^2
    float* hw = nullptr;        // [0] h_max, [1] 88 h_max^2, [2] density on the grid (1) or all pairs (0)
    uint32_t* done = nullptr;   // [0] ticket, [1..] block partials
    sfchunk::ChunkQueue q;      // the warp passes' chunks, heaviest first
};

__global__ void __launch_bounds__(SPH_BS) k_sph_density(const float* __restrict__ pos, const float* __restrict__ mas,
                                                        const float* __restrict__ rad, uint32_t n, int exact,
                                                        const float* __restrict__ hw, float* __restrict__ rho) {
    if (hw && hw[2] != 0.0f) return;  // FAST: the grid pass has it
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

// EXACT momentum pass: all j in index order, Kahan sums (sph.c:172-277)
template <bool HASH>
__global__ void __launch_bounds__(SPH_BS) k_sph_momentum(const float* __restrict__ pos, const float* __restrict__ mas,
                                                         const float* __restrict__ rad, const float* __restrict__ rho,
                                                         const float* __restrict__ prs, uint32_t n, int exact,
                                                         float* __restrict__ acc, uint32_t* __restrict__ nbr,
                                                         uint64_t* __restrict__ hash) {
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
    uint64_t hs = 0;
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
            if (HASH) hs += sf_mix64(jt + jj);
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
    if (HASH) hash[i] = hs;
}

// ---- FAST: the cell grid ------------------------------------------------------
// h_max (block partials, the last block finishes), the exp cutoff and the
// density path.
__global__ void __launch_bounds__(256) k_ref_hmax(const float* __restrict__ rad, uint32_t n, uint32_t* done,
                                                  float* __restrict__ hw) {
    __shared__ float sh[256];
    __shared__ bool last;
    float m = 0.0f;
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) m = fmaxf(m, rad[i]);
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] = fmaxf(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        done[1 + blockIdx.x] = __float_as_uint(sh[0]);
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
        if (last) done[0] = 0u;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        float h = 0.0f;
        for (uint32_t b = 0; b < gridDim.x; b++) h = fmaxf(h, __uint_as_float(__ldcg(&done[1 + b])));
        const float rd2 = EXP_CUT * h * h;
        hw[0] = h;
        hw[1] = rd2;
        // the density's reach in cells (margin included) must fit the 4 of the grid walk
        hw[2] = (sqrtf(rd2 * MARGIN_HI) <= SET_REACH * GRID_SIDE) ? 1.0f : 0.0f;
    }
}

__global__ void k_ref_keys(const float* __restrict__ pos, uint32_t n, uint32_t mask, uint64_t* __restrict__ keys,
                           uint32_t* __restrict__ vals, uint32_t* d_status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int3 c = cell_of(pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u], GRID_INV);
    if (cell_clamped(c)) atomicOr(d_status, SFGPU_STATUS_SPH_CELLS);
    keys[i] = bucket_of(c, mask);
    vals[i] = i;
}

__global__ void k_ref_gather(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ V, uint32_t n,
                             const float* __restrict__ slab, uint32_t* __restrict__ bstart, uint32_t* __restrict__ bend,
                             float4* __restrict__ px, float2* __restrict__ pq, uint64_t* __restrict__ cell) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t b = (uint32_t)keys[k];
    if (k == 0 || (uint32_t)keys[k - 1] != b) bstart[b] = k;
    if (k == n - 1 || (uint32_t)keys[k + 1] != b) bend[b] = k + 1;
    const uint32_t p = V[k];
    const float x = slab[3u * p], y = slab[3u * p + 1u], z = slab[3u * p + 2u];
    px[k] = make_float4(x, y, z, slab[(size_t)9 * n + p]);
    pq[k] = make_float2(slab[(size_t)13 * n + p], 0.0f);
    cell[k] = pack_cell(cell_of(x, y, z, GRID_INV));
}

// with q.est set, also each 32-body chunk's cost estimate (the
// populations of its bodies' buckets)
__global__ void k_ref_mix(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ V, uint32_t n,
                          const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
                          const uint64_t* __restrict__ cell, uint32_t* __restrict__ bmix,
                          uint64_t* __restrict__ bhash, sfchunk::ChunkQueue q) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t pop = 0;
    if (k < n) {
        const uint32_t b = (uint32_t)keys[k];
        const uint32_t s = bstart[b];
        if (k != s && cell[k] != cell[s]) bmix[b] = 1u;
        if (bhash) atomicAdd((unsigned long long*)&bhash[b], (unsigned long long)sf_mix64(V[k]));
        pop = bend[b] - s;
    }
    if (q.est && (k & ~31u) < n) sfchunk::note_cost(q, k >> 5, pop);
}

// One body against the cells of its reach: a callback per candidate pair,
// and per cell a flag saying whether every body of the cell is inside
// `r2_whole` (then `whole(j0, j1, b)` is called first).
struct CellRange {
    uint32_t j0, j1, chk;
    uint64_t want;
};

__device__ __forceinline__ bool cell_lookup(int3 c, uint32_t mask, const uint32_t* __restrict__ bstart,
                                            const uint32_t* __restrict__ bend, const uint32_t* __restrict__ bmix,
                                            const uint64_t* __restrict__ cell, CellRange& r, uint32_t& b) {
    b = bucket_of(c, mask);
    r.j0 = bstart[b];
    r.j1 = bend[b];
    if (r.j1 <= r.j0) return false;
    r.want = pack_cell(c);
    r.chk = bmix[b];
    return r.chk || cell[r.j0] == r.want;
}

// FAST density on the grid: pairs with r^2 < 88 h_max^2 (the rest have
// exp(-r^2/h^2) below FLT_MIN for both kernels).  The per-pair term:
__device__ __forceinline__ float ref_density_term(float r2, float ai3, float ihi2, float hj, float mj,
                                                  float inv_sqrt_pi) {
    const float aj = __fdividef(inv_sqrt_pi, hj);
    const float wi = ai3 * expf(-r2 * ihi2);
    const float wj = aj * aj * aj * expf(-r2 / (hj * hj));
    return 0.5f * (wi + wj) * mj;
}
__device__ __forceinline__ int ref_density_reach(float rd2) {
    return min(SET_REACH, (int)ceilf(sqrtf(rd2 * MARGIN_HI) * GRID_INV));
}
// One body's scan: every cell within `reach` whose box comes within the
// radius, every pair tested.
__device__ __forceinline__ float ref_density_body(const float4& a, float hi, float rd2, int reach, uint32_t mask,
                                                  const uint32_t* __restrict__ bstart,
                                                  const uint32_t* __restrict__ bend,
                                                  const uint32_t* __restrict__ bmix,
                                                  const uint64_t* __restrict__ cell, const float4* __restrict__ px,
                                                  const float2* __restrict__ pq) {
    const float inv_sqrt_pi = (float)K_INV_SQRT_PI;
    const float ai = __fdividef(inv_sqrt_pi, hi);
    const float ai3 = ai * ai * ai;
    const float ihi2 = 1.0f / (hi * hi);
    const int3 c0 = cell_of(a.x, a.y, a.z, GRID_INV);
    float sum = 0.0f;
    for (int dz = -reach; dz <= reach; dz++)
        for (int dy = -reach; dy <= reach; dy++)
            for (int dx = -reach; dx <= reach; dx++) {
                const int3 c = make_int3(c0.x + dx, c0.y + dy, c0.z + dz);
                float dmin2, dmax2;
                box_dist2(a.x, a.y, a.z, c.x * GRID_SIDE, c.y * GRID_SIDE, c.z * GRID_SIDE, GRID_SIDE, dmin2, dmax2);
                if (dmin2 * MARGIN_LO > rd2) continue;
                CellRange r;
                uint32_t b;
                if (!cell_lookup(c, mask, bstart, bend, bmix, cell, r, b)) continue;
                for (uint32_t j = r.j0; j < r.j1; j++) {
                    if (r.chk && cell[j] != r.want) continue;
                    const float4 q = px[j];
                    const float ex = fsub(a.x, q.x), ey = fsub(a.y, q.y), ez = fsub(a.z, q.z);
                    const float r2 = fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez));
                    if (!(r2 < rd2)) continue;
                    sum += ref_density_term(r2, ai3, ihi2, pq[j].x, q.w, inv_sqrt_pi);
                }
            }
    return sum;
}

// One thread per sorted body (sph_path 2).
__global__ void __launch_bounds__(128) k_ref_density_grid(uint32_t n, uint32_t mask, const uint32_t* __restrict__ bstart,
                                                          const uint32_t* __restrict__ bend,
                                                          const uint32_t* __restrict__ bmix,
                                                          const uint64_t* __restrict__ cell,
                                                          const float4* __restrict__ px, const float2* __restrict__ pq,
                                                          const uint32_t* __restrict__ V, const float* __restrict__ hw,
                                                          float* __restrict__ rho) {
    if (hw[2] == 0.0f) return;  // the all-pairs tiles have it
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float rd2 = hw[1];
    rho[V[k]] = ref_density_body(px[k], pq[k].x, rd2, ref_density_reach(rd2), mask, bstart, bend, bmix, cell, px, pq);
}

// The grid passes by warps (the default): one warp per 32 consecutive
// sorted bodies, which nearly always share a cell of side 1/4.  The warp
// visits the union of its bodies' cells; each lane classifies every cell
// exactly as its per-body scan would (reach, box distance), the cell's
// bodies are staged in shared memory 32 at a time, each lane first takes
// its neighbour decisions over the staged bodies into a bit mask and then
// evaluates its own terms in candidate order.  So every body adds the same
// terms in the same order as the per-body scan, while the warp's loads are
// coalesced and its loops no longer diverge body by body.  A warp whose
// bodies span more than 3 cells on an axis, or reach beyond the packed
// key's range, runs the per-body scans.  The warps are persistent and take
// their chunks heaviest first (chunks.cuh).
constexpr int RW_WARPS = 4;
// The density warp pass takes a register-budget hint (one resident block
// asked for: 68 registers, no spills, instead of 56 with spills; measured
// 13.0-13.5 against 13.7-14.6 ms per pass on the 262,144-body gas); the
// momentum pass measured slower with it and keeps ptxas's own choice.

__device__ __forceinline__ void ref_density_chunk(uint32_t k0, uint32_t n, uint32_t mask,
                                                  const uint32_t* __restrict__ bstart,
                                                  const uint32_t* __restrict__ bend,
                                                  const uint32_t* __restrict__ bmix,
                                                  const uint64_t* __restrict__ cell, const float4* __restrict__ px,
                                                  const float2* __restrict__ pq, const uint32_t* __restrict__ V,
                                                  const float* __restrict__ hw, float* __restrict__ rho, float4* sq,
                                                  float* sh) {
    const int lane = threadIdx.x & 31;
    if (k0 >= n) return;
    const uint32_t k = k0 + (uint32_t)lane;
    const bool live = k < n;
    const uint32_t kk = live ? k : n - 1u;
    const float rd2 = hw[1];
    const int reach = ref_density_reach(rd2);
    const float4 a = px[kk];
    const float hi = pq[kk].x;
    const int3 c0 = cell_of(a.x, a.y, a.z, GRID_INV);
    const int zlo = __reduce_min_sync(0xffffffffu, c0.z), zhi = __reduce_max_sync(0xffffffffu, c0.z);
    const int ylo = __reduce_min_sync(0xffffffffu, c0.y), yhi = __reduce_max_sync(0xffffffffu, c0.y);
    const int xlo = __reduce_min_sync(0xffffffffu, c0.x), xhi = __reduce_max_sync(0xffffffffu, c0.x);
    const bool compact = (uint32_t)zhi - (uint32_t)zlo <= 2u && (uint32_t)yhi - (uint32_t)ylo <= 2u &&
                         (uint32_t)xhi - (uint32_t)xlo <= 2u && !__any_sync(0xffffffffu, cell_clamped(c0));
    if (!compact) {
        if (live) rho[V[k]] = ref_density_body(a, hi, rd2, reach, mask, bstart, bend, bmix, cell, px, pq);
        return;
    }
    const float inv_sqrt_pi = (float)K_INV_SQRT_PI;
    const float ai = __fdividef(inv_sqrt_pi, hi);
    const float ai3 = ai * ai * ai;
    const float ihi2 = 1.0f / (hi * hi);
    float sum = 0.0f;
    for (int cz = zlo - reach; cz <= zhi + reach; cz++)
        for (int cy = ylo - reach; cy <= yhi + reach; cy++)
            for (int cx = xlo - reach; cx <= xhi + reach; cx++) {
                const int3 c = make_int3(cx, cy, cz);
                bool need = false;
                if (live && abs(cx - c0.x) <= reach && abs(cy - c0.y) <= reach && abs(cz - c0.z) <= reach) {
                    float dmin2, dmax2;
                    box_dist2(a.x, a.y, a.z, c.x * GRID_SIDE, c.y * GRID_SIDE, c.z * GRID_SIDE, GRID_SIDE, dmin2,
                              dmax2);
                    need = !(dmin2 * MARGIN_LO > rd2);
                }
                if (!__any_sync(0xffffffffu, need)) continue;
                CellRange r;
                uint32_t b;
                if (!cell_lookup(c, mask, bstart, bend, bmix, cell, r, b)) continue;
                for (uint32_t jb = r.j0; jb < r.j1; jb += 32u) {
                    const uint32_t j = jb + (uint32_t)lane;
                    const bool ok = j < r.j1 && (!r.chk || cell[j] == r.want);
                    __syncwarp();
                    if (ok) {
                        sq[lane] = px[j];
                        sh[lane] = pq[j].x;
                    }
                    const uint32_t vm = __ballot_sync(0xffffffffu, ok);
                    __syncwarp();
                    uint32_t hits = 0u;
                    if (need) {
                        for (uint32_t mm = vm; mm; mm &= mm - 1u) {
                            const int t = __ffs(mm) - 1;
                            const float4 q = sq[t];
                            const float ex = fsub(a.x, q.x), ey = fsub(a.y, q.y), ez = fsub(a.z, q.z);
                            const float r2 = fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez));
                            if (r2 < rd2) hits |= 1u << t;
                        }
                    }
                    // two terms per round: the second's arithmetic overlaps the
                    // first's, the sum takes them in order
                    auto dterm = [&](int t) {
                        const float4 q = sq[t];
                        const float ex = fsub(a.x, q.x), ey = fsub(a.y, q.y), ez = fsub(a.z, q.z);
                        const float r2 = fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez));
                        sum += ref_density_term(r2, ai3, ihi2, sh[t], q.w, inv_sqrt_pi);
                    };
                    while (__any_sync(0xffffffffu, hits != 0u)) {
                        if (hits) {
                            const int t1 = __ffs(hits) - 1;
                            hits &= hits - 1u;
                            const int t2 = hits ? __ffs(hits) - 1 : -1;
                            if (t2 >= 0) hits &= hits - 1u;
                            dterm(t1);
                            if (t2 >= 0) dterm(t2);
                        }
                    }
                }
            }
    if (live) rho[V[k]] = sum;
}

__global__ void __launch_bounds__(RW_WARPS * 32, 1) k_ref_density_warp(
    uint32_t n, uint32_t mask, const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
    const uint32_t* __restrict__ bmix, const uint64_t* __restrict__ cell, const float4* __restrict__ px,
    const float2* __restrict__ pq, const uint32_t* __restrict__ V, const float* __restrict__ hw,
    float* __restrict__ rho, sfchunk::ChunkQueue q) {
    __shared__ float4 s_q[RW_WARPS][32];
    __shared__ float s_h[RW_WARPS][32];
    if (hw[2] == 0.0f) return;  // the all-pairs tiles have it (no warp takes a chunk)
    const int w = threadIdx.x >> 5;
    sfchunk::Taker t = sfchunk::taker(q);
    for (;;) {
        const uint32_t c = sfchunk::next(q, t);
        if (c == 0xFFFFFFFFu) break;
        const long long t0 = clock64();
        ref_density_chunk(c * 32u, n, mask, bstart, bend, bmix, cell, px, pq, V, hw, rho, s_q[w], s_h[w]);
        sfchunk::record(q, 0, c, clock64() - t0);
    }
    sfchunk::warp_exit(q, gridDim.x * RW_WARPS);
}

// pressure (sph.c:148-159) into the slab, c = P/rho^2 into the sorted records
__global__ void k_ref_eos(const uint32_t* __restrict__ V, uint32_t n, float* __restrict__ slab,
                          float2* __restrict__ pq) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t p = V[k];
    const float rho = slab[(size_t)14 * n + p];
    const float t = fmul(0.1f, rho);
    const float P = fmul(t, t);
    slab[(size_t)15 * n + p] = P;
    const float rho2 = fmul(rho, rho);
    pq[k].y = (0.0f < rho2) ? fdiv(P, rho2) : 0.0f;
}

// FAST momentum on the grid: the set {j : fl(r^2) <= 1} (cells inside the
// radius taken whole), force terms where r^2 < 88 h_max^2.  The per-pair
// term (sph.c:254-268, FAST arithmetic):
__device__ __forceinline__ void ref_momentum_term(float ex, float ey, float ez, float r2, float ihi2, float m2_den_i,
                                                  float ci, float hj, float cj, float pi15, float& sx, float& sy,
                                                  float& sz) {
    const float ni = m2_den_i * expf(-r2 * ihi2);
    const float nj = -2.0f * expf(-r2 / (hj * hj)) / (pi15 * hj * hj * hj * hj * hj);
    const float g = 0.5f * (ni + nj) * (ci + cj);
    sx += g * ex;
    sy += g * ey;
    sz += g * ez;
}

// One body's scan: every cell within 4 whose box comes within the radius.
template <bool HASH>
__device__ __forceinline__ void ref_momentum_body(const float4& a, float hi, float ci, float rf2, uint32_t mask,
                                                  const uint32_t* __restrict__ bstart,
                                                  const uint32_t* __restrict__ bend,
                                                  const uint32_t* __restrict__ bmix,
                                                  const uint64_t* __restrict__ bhash,
                                                  const uint64_t* __restrict__ cell, const float4* __restrict__ px,
                                                  const float2* __restrict__ pq, const uint32_t* __restrict__ V,
                                                  float& sx, float& sy, float& sz, uint32_t& count, uint64_t& hs) {
    const float pi15 = (float)K_PI_1_5;
    const float ihi2 = 1.0f / (hi * hi);
    const float m2_den_i = -2.0f / (pi15 * hi * hi * hi * hi * hi);
    const int3 c0 = cell_of(a.x, a.y, a.z, GRID_INV);
    for (int dz = -SET_REACH; dz <= SET_REACH; dz++)
        for (int dy = -SET_REACH; dy <= SET_REACH; dy++)
            for (int dx = -SET_REACH; dx <= SET_REACH; dx++) {
                const int3 c = make_int3(c0.x + dx, c0.y + dy, c0.z + dz);
                float dmin2, dmax2;
                box_dist2(a.x, a.y, a.z, c.x * GRID_SIDE, c.y * GRID_SIDE, c.z * GRID_SIDE, GRID_SIDE, dmin2, dmax2);
                if (dmin2 * MARGIN_LO > 1.0f) continue;
                CellRange r;
                uint32_t b;
                if (!cell_lookup(c, mask, bstart, bend, bmix, cell, r, b)) continue;
                const bool whole = !r.chk && !cell_clamped(c) && dmax2 * MARGIN_HI < 1.0f;
                if (whole) {
                    count += r.j1 - r.j0;
                    if (HASH) hs += bhash[b];
                    if (dmin2 * MARGIN_LO >= rf2) continue;  // no term of the cell is a normal number
                }
                for (uint32_t j = r.j0; j < r.j1; j++) {
                    if (r.chk && cell[j] != r.want) continue;
                    const float4 q = px[j];
                    const float ex = fsub(a.x, q.x), ey = fsub(a.y, q.y), ez = fsub(a.z, q.z);
                    const float r2 = fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez));
                    if (!whole) {
                        if (r2 > 1.0f) continue;  // sph.c:231
                        count++;
                        if (HASH) hs += sf_mix64(V[j]);
                    }
                    if (!(r2 < rf2)) continue;
                    const float2 qj = pq[j];
                    ref_momentum_term(ex, ey, ez, r2, ihi2, m2_den_i, ci, qj.x, qj.y, pi15, sx, sy, sz);
                }
            }
}

// sph.c:274-276: acc += -m_i * sum
__device__ __forceinline__ void ref_momentum_store(uint32_t p, float mi, float sx, float sy, float sz, uint32_t count,
                                                   uint64_t hs, bool with_hash, float* __restrict__ acc,
                                                   uint32_t* __restrict__ nbr, uint64_t* __restrict__ hash) {
    acc[3u * p + 0u] = fadd(acc[3u * p + 0u], fmul(-mi, sx));
    acc[3u * p + 1u] = fadd(acc[3u * p + 1u], fmul(-mi, sy));
    acc[3u * p + 2u] = fadd(acc[3u * p + 2u], fmul(-mi, sz));
    nbr[p] = count;
    if (with_hash) hash[p] = hs;
}

// One thread per sorted body (sph_path 2).
template <bool HASH>
__global__ void __launch_bounds__(128) k_ref_momentum_grid(
    uint32_t n, uint32_t mask, const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
    const uint32_t* __restrict__ bmix, const uint64_t* __restrict__ bhash, const uint64_t* __restrict__ cell,
    const float4* __restrict__ px, const float2* __restrict__ pq, const uint32_t* __restrict__ V,
    const float* __restrict__ hw, float* __restrict__ acc, uint32_t* __restrict__ nbr,
    uint64_t* __restrict__ hash) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 a = px[k];
    const float2 qi = pq[k];
    float sx = 0.f, sy = 0.f, sz = 0.f;
    uint32_t count = 0;
    uint64_t hs = 0;
    ref_momentum_body<HASH>(a, qi.x, qi.y, hw[1], mask, bstart, bend, bmix, bhash, cell, px, pq, V, sx, sy, sz, count,
                            hs);
    ref_momentum_store(V[k], a.w, sx, sy, sz, count, hs, HASH, acc, nbr, hash);
}

// The default momentum pass, by warps (see k_ref_density_warp).  A lane
// whose box test puts a cell wholly inside the radius counts it whole (as
// its per-body scan does) and tests its bodies only for force terms.
template <bool HASH>
__device__ __forceinline__ void ref_momentum_chunk(
    uint32_t k0, uint32_t n, uint32_t mask, const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
    const uint32_t* __restrict__ bmix, const uint64_t* __restrict__ bhash, const uint64_t* __restrict__ cell,
    const float4* __restrict__ px, const float2* __restrict__ pq, const uint32_t* __restrict__ V,
    const float* __restrict__ hw, float* __restrict__ acc, uint32_t* __restrict__ nbr, uint64_t* __restrict__ hash,
    float4* sq, float2* sp, uint64_t* sm) {
    const int lane = threadIdx.x & 31;
    if (k0 >= n) return;
    const uint32_t k = k0 + (uint32_t)lane;
    const bool live = k < n;
    const uint32_t kk = live ? k : n - 1u;
    const float rf2 = hw[1];
    const float4 a = px[kk];
    const float2 qi = pq[kk];
    const float hi = qi.x, ci = qi.y;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    uint32_t count = 0;
    uint64_t hs = 0;
    const int3 c0 = cell_of(a.x, a.y, a.z, GRID_INV);
    const int zlo = __reduce_min_sync(0xffffffffu, c0.z), zhi = __reduce_max_sync(0xffffffffu, c0.z);
    const int ylo = __reduce_min_sync(0xffffffffu, c0.y), yhi = __reduce_max_sync(0xffffffffu, c0.y);
    const int xlo = __reduce_min_sync(0xffffffffu, c0.x), xhi = __reduce_max_sync(0xffffffffu, c0.x);
    const bool compact = (uint32_t)zhi - (uint32_t)zlo <= 2u && (uint32_t)yhi - (uint32_t)ylo <= 2u &&
                         (uint32_t)xhi - (uint32_t)xlo <= 2u && !__any_sync(0xffffffffu, cell_clamped(c0));
    if (!compact) {
        if (live) {
            ref_momentum_body<HASH>(a, hi, ci, rf2, mask, bstart, bend, bmix, bhash, cell, px, pq, V, sx, sy, sz,
                                    count, hs);
            ref_momentum_store(V[k], a.w, sx, sy, sz, count, hs, HASH, acc, nbr, hash);
        }
        return;
    }
    const float pi15 = (float)K_PI_1_5;
    const float ihi2 = 1.0f / (hi * hi);
    const float m2_den_i = -2.0f / (pi15 * hi * hi * hi * hi * hi);
    for (int cz = zlo - SET_REACH; cz <= zhi + SET_REACH; cz++)
        for (int cy = ylo - SET_REACH; cy <= yhi + SET_REACH; cy++)
            for (int cx = xlo - SET_REACH; cx <= xhi + SET_REACH; cx++) {
                const int3 c = make_int3(cx, cy, cz);
                bool need = false;
                float dmin2 = 0.f, dmax2 = 0.f;
                if (live && abs(cx - c0.x) <= SET_REACH && abs(cy - c0.y) <= SET_REACH &&
                    abs(cz - c0.z) <= SET_REACH) {
                    box_dist2(a.x, a.y, a.z, c.x * GRID_SIDE, c.y * GRID_SIDE, c.z * GRID_SIDE, GRID_SIDE, dmin2,
                              dmax2);
                    need = !(dmin2 * MARGIN_LO > 1.0f);
                }
                if (!__any_sync(0xffffffffu, need)) continue;
                CellRange r;
                uint32_t b;
                if (!cell_lookup(c, mask, bstart, bend, bmix, cell, r, b)) continue;
                const bool whole = need && !r.chk && !cell_clamped(c) && dmax2 * MARGIN_HI < 1.0f;
                if (whole) {
                    count += r.j1 - r.j0;
                    if (HASH) hs += bhash[b];
                }
                const bool pairs = need && !(whole && dmin2 * MARGIN_LO >= rf2);
                if (!__any_sync(0xffffffffu, pairs)) continue;
                for (uint32_t jb = r.j0; jb < r.j1; jb += 32u) {
                    const uint32_t j = jb + (uint32_t)lane;
                    const bool ok = j < r.j1 && (!r.chk || cell[j] == r.want);
                    __syncwarp();
                    if (ok) {
                        sq[lane] = px[j];
                        sp[lane] = pq[j];
                        if (HASH) sm[lane] = sf_mix64(V[j]);
                    }
                    const uint32_t vm = __ballot_sync(0xffffffffu, ok);
                    __syncwarp();
                    uint32_t hits = 0u;
                    if (pairs) {
                        for (uint32_t mm = vm; mm; mm &= mm - 1u) {
                            const int t = __ffs(mm) - 1;
                            const float4 q = sq[t];
                            const float ex = fsub(a.x, q.x), ey = fsub(a.y, q.y), ez = fsub(a.z, q.z);
                            const float r2 = fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez));
                            if (!whole) {
                                if (r2 > 1.0f) continue;  // sph.c:231
                                count++;
                                if (HASH) hs += sm[t];
                            }
                            if (r2 < rf2) hits |= 1u << t;
                        }
                    }
                    // two terms per round (the sums take them in order)
                    auto mterm = [&](int t) {
                        const float4 q = sq[t];
                        const float ex = fsub(a.x, q.x), ey = fsub(a.y, q.y), ez = fsub(a.z, q.z);
                        const float r2 = fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez));
                        const float2 qj = sp[t];
                        ref_momentum_term(ex, ey, ez, r2, ihi2, m2_den_i, ci, qj.x, qj.y, pi15, sx, sy, sz);
                    };
                    while (__any_sync(0xffffffffu, hits != 0u)) {
                        if (hits) {
                            const int t1 = __ffs(hits) - 1;
                            hits &= hits - 1u;
                            const int t2 = hits ? __ffs(hits) - 1 : -1;
                            if (t2 >= 0) hits &= hits - 1u;
                            mterm(t1);
                            if (t2 >= 0) mterm(t2);
                        }
                    }
                }
            }
    if (live) ref_momentum_store(V[k], a.w, sx, sy, sz, count, hs, HASH, acc, nbr, hash);
}

template <bool HASH>
__global__ void __launch_bounds__(RW_WARPS * 32) k_ref_momentum_warp(
    uint32_t n, uint32_t mask, const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
    const uint32_t* __restrict__ bmix, const uint64_t* __restrict__ bhash, const uint64_t* __restrict__ cell,
    const float4* __restrict__ px, const float2* __restrict__ pq, const uint32_t* __restrict__ V,
    const float* __restrict__ hw, float* __restrict__ acc, uint32_t* __restrict__ nbr,
    uint64_t* __restrict__ hash, sfchunk::ChunkQueue q) {
    __shared__ float4 s_q[RW_WARPS][32];
    __shared__ float2 s_p[RW_WARPS][32];
    __shared__ uint64_t s_m[RW_WARPS][HASH ? 32 : 1];
    const int w = threadIdx.x >> 5;
    sfchunk::Taker t = sfchunk::taker(q);
    for (;;) {
        const uint32_t c = sfchunk::next(q, t);
        if (c == 0xFFFFFFFFu) break;
        const long long t0 = clock64();
        ref_momentum_chunk<HASH>(c * 32u, n, mask, bstart, bend, bmix, bhash, cell, px, pq, V, hw, acc, nbr, hash,
                                 s_q[w], s_p[w], s_m[w]);
        sfchunk::record(q, 1, c, clock64() - t0);
    }
    sfchunk::warp_exit(q, gridDim.x * RW_WARPS);
}

}  // namespace

int sf_sph_cubic_alloc(sfgpu_sim* s);
void sf_sph_cubic_free(sfgpu_sim* s);
int sf_sph_cubic(sfgpu_sim* s);

int sf_sph_alloc(sfgpu_sim* s) {
    SphWork* w = new SphWork();
    s->sph = w;
    const uint32_t n = std::max<uint32_t>(s->n, 1);
    SF_CUDA(cudaMalloc(&w->nbr, sizeof(uint32_t) * n));
    SF_CUDA(cudaMemset(w->nbr, 0, sizeof(uint32_t) * n));
    if (s->p.flags & SFGPU_FLAG_STATS) {
        SF_CUDA(cudaMalloc(&w->hash, sizeof(uint64_t) * n));
        SF_CUDA(cudaMemset(w->hash, 0, sizeof(uint64_t) * n));
    }
    if (s->p.sph == SFGPU_SPH_CUBIC) return sf_sph_cubic_alloc(s);
    if (s->p.math == SFGPU_MATH_EXACT) return SFGPU_OK;  // all pairs, no grid
    w->tbits = 1;
    while ((1u << w->tbits) < 2u * n) w->tbits++;
    w->tsize = 1u << w->tbits;
    SF_CUDA(cudaMalloc(&w->keys, sizeof(uint64_t) * n));
    SF_CUDA(cudaMalloc(&w->vals, sizeof(uint32_t) * n));
    if (sf_sort_alloc(w->sort, n) != SFGPU_OK) return SFGPU_FAILURE;
    if (s->p.spin_limit) w->sort.spin_limit = s->p.spin_limit;
    SF_CUDA(cudaMalloc(&w->bstart, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->bend, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->bmix, sizeof(uint32_t) * w->tsize));
    if (w->hash) SF_CUDA(cudaMalloc(&w->bhash, sizeof(uint64_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->cell, sizeof(uint64_t) * n));
    SF_CUDA(cudaMalloc(&w->px, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->pq, sizeof(float2) * n));
    SF_CUDA(cudaMalloc(&w->hw, sizeof(float) * 4));
    SF_CUDA(cudaMalloc(&w->done, sizeof(uint32_t) * (1 + 1024)));
    SF_CUDA(cudaMemset(w->done, 0, sizeof(uint32_t) * (1 + 1024)));
    if (sfchunk::alloc(w->q, n) != SFGPU_OK) return SFGPU_FAILURE;
    return SFGPU_OK;
}

void sf_sph_free(sfgpu_sim* s) {
    SphWork* w = (SphWork*)s->sph;
    if (!w) return;
    if (s->p.sph == SFGPU_SPH_CUBIC) sf_sph_cubic_free(s);
    cudaFree(w->nbr);
    cudaFree(w->hash);
    cudaFree(w->keys);
    cudaFree(w->vals);
    sf_sort_free(w->sort);
    cudaFree(w->bstart);
    cudaFree(w->bend);
    cudaFree(w->bmix);
    cudaFree(w->bhash);
    cudaFree(w->cell);
    cudaFree(w->px);
    cudaFree(w->pq);
    cudaFree(w->hw);
    cudaFree(w->done);
    sfchunk::release(w->q);
    delete w;
    s->sph = nullptr;
}

uint32_t* sf_sph_neighbour_counts(sfgpu_sim* s) { return s->sph ? ((SphWork*)s->sph)->nbr : nullptr; }
uint64_t* sf_sph_neighbour_hashes(sfgpu_sim* s) { return s->sph ? ((SphWork*)s->sph)->hash : nullptr; }

int sf_stage_sph(sfgpu_sim* s) {
    if (s->p.sph == SFGPU_SPH_CUBIC) return sf_sph_cubic(s);
    SphWork* w = (SphWork*)s->sph;
    const uint32_t n = s->n;
    cudaStream_t st = s->stream;
    float* slab = s->slab;
    const float* pos = slab;
    float* acc = slab + (size_t)6 * n;
    const float* mas = slab + (size_t)9 * n;
    const float* rad = slab + (size_t)13 * n;
    float* rho = slab + (size_t)14 * n;
    float* prs = slab + (size_t)15 * n;
    const uint32_t grid = sf_ceil_div(n, SPH_BS);
    if (s->p.math == SFGPU_MATH_EXACT) {
        int tk = s->timer.begin(st, "sph_density");
        k_sph_density<<<grid, SPH_BS, 0, st>>>(pos, mas, rad, n, 1, nullptr, rho);
        SF_CHECK_LAUNCH();
        k_sph_eos<<<sf_ceil_div(n, 256), 256, 0, st>>>(rho, n, prs);
        SF_CHECK_LAUNCH();
        s->timer.end(st, tk);
        tk = s->timer.begin(st, "sph_force");
        if (w->hash)
            k_sph_momentum<true><<<grid, SPH_BS, 0, st>>>(pos, mas, rad, rho, prs, n, 1, acc, w->nbr, w->hash);
        else
            k_sph_momentum<false><<<grid, SPH_BS, 0, st>>>(pos, mas, rad, rho, prs, n, 1, acc, w->nbr, nullptr);
        SF_CHECK_LAUNCH();
        s->timer.end(st, tk);
        return SFGPU_OK;
    }
    // FAST: the cell grid
    int tk = s->timer.begin(st, "sph_grid");
    const uint32_t hb = std::min<uint32_t>(sf_ceil_div(n, 256), 1024);
    k_ref_hmax<<<hb, 256, 0, st>>>(rad, n, w->done, w->hw);
    SF_CHECK_LAUNCH();
    const uint32_t mask = w->tsize - 1;
    const uint32_t nb = sf_ceil_div(n, 256);
    k_ref_keys<<<nb, 256, 0, st>>>(pos, n, mask, w->keys, w->vals, s->d_status);
    SF_CHECK_LAUNCH();
    if (sf_sort_pairs(w->keys, w->vals, n, (int)w->tbits, w->sort, st, s->d_status) != SFGPU_OK)
        return SFGPU_FAILURE;
    SF_CUDA(cudaMemsetAsync(w->bstart, 0, sizeof(uint32_t) * w->tsize, st));
    SF_CUDA(cudaMemsetAsync(w->bend, 0, sizeof(uint32_t) * w->tsize, st));
    SF_CUDA(cudaMemsetAsync(w->bmix, 0, sizeof(uint32_t) * w->tsize, st));
    if (w->bhash) SF_CUDA(cudaMemsetAsync(w->bhash, 0, sizeof(uint64_t) * w->tsize, st));
    k_ref_gather<<<nb, 256, 0, st>>>(w->keys, w->vals, n, slab, w->bstart, w->bend, w->px, w->pq, w->cell);
    SF_CHECK_LAUNCH();
    const bool by_warp = s->p.sph_path != 2;
    sfchunk::ChunkQueue q = w->q;
    if (!by_warp) q.est = nullptr;  // the per-body passes take no chunks
    k_ref_mix<<<nb, 256, 0, st>>>(w->keys, w->vals, n, w->bstart, w->bend, w->cell, w->bmix, w->bhash, q);
    SF_CHECK_LAUNCH();

    s->timer.end(st, tk);
    tk = s->timer.begin(st, "sph_density");
    static uint32_t wave[3] = {0, 0, 0};  // density, momentum with hashes, momentum
    if (!wave[0]) {
        wave[0] = sfchunk::wave_blocks(k_ref_density_warp, RW_WARPS * 32, 0xFFFFFFFFu);
        wave[1] = sfchunk::wave_blocks(k_ref_momentum_warp<true>, RW_WARPS * 32, 0xFFFFFFFFu);
        wave[2] = sfchunk::wave_blocks(k_ref_momentum_warp<false>, RW_WARPS * 32, 0xFFFFFFFFu);
    }
    const uint32_t most = sf_ceil_div(w->q.nchunks, RW_WARPS);
    if (by_warp) {
        sfchunk::k_chunk_order<<<1, 1024, 0, st>>>(w->q, 0);
        SF_CHECK_LAUNCH();
    }
    if (by_warp)
        k_ref_density_warp<<<std::min(wave[0], most), RW_WARPS * 32, 0, st>>>(
            n, mask, w->bstart, w->bend, w->bmix, w->cell, w->px, w->pq, w->vals, w->hw, rho, w->q);
    else
        k_ref_density_grid<<<sf_ceil_div(n, 128), 128, 0, st>>>(n, mask, w->bstart, w->bend, w->bmix, w->cell,
                                                               w->px, w->pq, w->vals, w->hw, rho);
    SF_CHECK_LAUNCH();
    k_sph_density<<<grid, SPH_BS, 0, st>>>(pos, mas, rad, n, 0, w->hw, rho);
    SF_CHECK_LAUNCH();
    k_ref_eos<<<nb, 256, 0, st>>>(w->vals, n, slab, w->pq);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    tk = s->timer.begin(st, "sph_force");
    if (by_warp) {
        sfchunk::k_chunk_order<<<1, 1024, 0, st>>>(w->q, 1);
        SF_CHECK_LAUNCH();
    }
    if (by_warp && w->hash)
        k_ref_momentum_warp<true><<<std::min(wave[1], most), RW_WARPS * 32, 0, st>>>(
            n, mask, w->bstart, w->bend, w->bmix, w->bhash, w->cell, w->px, w->pq, w->vals, w->hw, acc, w->nbr,
            w->hash, w->q);
    else if (by_warp)
        k_ref_momentum_warp<false><<<std::min(wave[2], most), RW_WARPS * 32, 0, st>>>(
            n, mask, w->bstart, w->bend, w->bmix, nullptr, w->cell, w->px, w->pq, w->vals, w->hw, acc, w->nbr,
            nullptr, w->q);
    else if (w->hash)
        k_ref_momentum_grid<true><<<sf_ceil_div(n, 128), 128, 0, st>>>(n, mask, w->bstart, w->bend, w->bmix,
                                                                       w->bhash, w->cell, w->px, w->pq, w->vals,
                                                                       w->hw, acc, w->nbr, w->hash);
    else
        k_ref_momentum_grid<false><<<sf_ceil_div(n, 128), 128, 0, st>>>(n, mask, w->bstart, w->bend, w->bmix,
                                                                        nullptr, w->cell, w->px, w->pq, w->vals,
                                                                        w->hw, acc, w->nbr, nullptr);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    return SFGPU_OK;
}
