// sph_cubic.cu -- cubic-spline SPH with an ideal-gas equation of state and
// Monaghan artificial viscosity (no counterpart in the reference, whose SPH
// is the Gaussian all-pairs form of src/sph.c).
//
//   W(r,h)  = 1/(pi h^3) (1 - 1.5 q^2 + 0.75 q^3), q < 1;  0.25 (2-q)^3 / (pi h^3), q < 2
//   rho_i   = sum_j m_j (W(r,h_i) + W(r,h_j))/2                 (j = i included)
//   P_i     = (gamma-1) rho_i u_i,  c_i = sqrt(gamma (gamma-1) u_i)
//   dv_i/dt = -sum_j m_j (P_i/rho_i^2 + P_j/rho_j^2 + Pi_ij) grad_i W_ij
//   du_i/dt =  sum_j m_j (P_i/rho_i^2 + Pi_ij/2) v_ij . grad_i W_ij
//   Pi_ij   = (-alpha cbar mu + beta mu^2)/rhobar if v_ij.r_ij < 0,
//             mu = h v_ij.r_ij/(r^2 + 0.01 h^2), h = (h_i+h_j)/2
// Neighbours: fl((dx^2 + dy^2) + dz^2) < fl((2 max(h_i,h_j))^2) in FP32.
//
// Neighbour search on the hashed cell grid of sph_grid.cuh.  The search
// radius is R = 2 h_max; cells have side R / REACH (slightly enlarged, so
// that FP32 rounding never puts a neighbour more than REACH cells away).
// A body's scan takes the rows of cells (dy, dz) in [-REACH, REACH]^2 whose
// distance from the body is below R, and in each row only the x-range of
// cells the sphere of radius R reaches: with REACH = 1 the 3 x 3 rows of
// side-2h cells with at most 2 cells per row, with REACH = 2 about 84 cells
// of side h holding 2.5x the candidates of the sphere, whose extra cell
// look-ups cost more than the candidates they save.  The default pass
// (sfgpu_params.sph_path 0, REACH = 1; 3 with REACH = 2) runs one warp per
// 32 sorted bodies over the union of their scans (cubic_chunk below),
// persistent warps taking the chunks heaviest first (chunks.cuh); paths 2
// (REACH = 1) and 1 (REACH = 2) run one thread per body.  Each candidate is
// tested with the FP32 expression above; bodies of another cell that
// shares the bucket are skipped by cell key, so none is counted twice.  With SFGPU_FLAG_STATS the
// density pass also sums an order-independent hash of every body's
// neighbour set (j = i included).
#include <climits>

#include "internal.cuh"
#include "chunks.cuh"
#include "sph_grid.cuh"

namespace {

using namespace sfgrid;

constexpr float PI_F = 3.14159265358979323846f;
constexpr float MARGIN_HI = 1.0f + 1.0f / 1024.0f;

struct CubicWork {
    uint32_t tbits = 0, tsize = 0;
    int reach = 1;
    uint32_t path = 0;  // sfgpu_params.sph_path
    uint64_t* keys = nullptr;
    uint32_t* vals = nullptr;
    SortWork sort;
    uint32_t* bstart = nullptr;
    uint32_t* bend = nullptr;
    float4* px = nullptr;      // sorted x, y, z, m
    float4* pv = nullptr;      // sorted vx, vy, vz, u
    float4* pd = nullptr;      // sorted rho, P/rho^2, c, h
    float4* ph = nullptr;      // sorted h, u, c, 1/h
    uint32_t* bmix = nullptr;  // per bucket: holds more than one cell
    uint64_t* cell = nullptr;  // sorted packed cell coordinates
    uint64_t* mixv = nullptr;  // sorted: hash of each body's index (SFGPU_FLAG_STATS)
    float* grid = nullptr;     // [0] cell side, [1] 1/side, [2] search radius R = 2 h_max
    uint32_t* done = nullptr;
    sfchunk::ChunkQueue q;     // the warp passes' chunks, heaviest first
};

// The kernel and its derivative from q = r / h and 1 / h (the passes keep
// 1 / h of every body, so no division runs per pair).  Both pieces are
// computed and one selected (no branch), so consecutive pairs' terms can
// be computed side by side.
__device__ __forceinline__ float w_cubic(float r, float ih) {
    const float q = r * ih;
    const float s = ih * ih * ih * (1.0f / PI_F);
    const float inner = s * (1.0f - 1.5f * q * q + 0.75f * q * q * q);
    const float t = 2.0f - q;
    const float outer = s * 0.25f * t * t * t;
    return q < 1.0f ? inner : (q < 2.0f ? outer : 0.0f);
}
__device__ __forceinline__ float dw_cubic(float r, float ih) {
    const float q = r * ih;
    const float ih2 = ih * ih;
    const float s = ih2 * ih2 * (1.0f / PI_F);
    const float inner = s * (-3.0f * q + 2.25f * q * q);
    const float t = 2.0f - q;
    const float outer = s * (-0.75f * t * t);
    return q < 1.0f ? inner : (q < 2.0f ? outer : 0.0f);
}
// the FP32 neighbour decision (same expression as the oracle)
__device__ __forceinline__ bool is_neighbour(float dx, float dy, float dz, float hi, float hj, float& r2) {
    r2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
    const float s = fmul(2.0f, fmaxf(hi, hj));
    return r2 < fmul(s, s);
}
// The same decision for two candidates (negated coordinates nx, ny, nz and
// S = (2 h_j)^2 each) against body (ax, ay, az) with Si = (2 h_i)^2, bit 0
// and bit 1: a - q as a + (-q), the squares on paired instructions, their
// sums scalar (ptxas fuses a paired product into a following paired add,
// which would round r^2 differently), and r^2 < (2 max(h_i, h_j))^2 as
// r^2 < max((2 h_i)^2, (2 h_j)^2) (squaring and rounding keep the order):
// the same bits as is_neighbour.
__device__ __forceinline__ uint32_t neighbours2(float2 ax, float2 ay, float2 az, float2 nx, float2 ny, float2 nz,
                                                float2 S, float Si) {
    const float2 dx = __fadd2_rn(ax, nx), dy = __fadd2_rn(ay, ny), dz = __fadd2_rn(az, nz);
    const float2 px = __fmul2_rn(dx, dx), py = __fmul2_rn(dy, dy), pz = __fmul2_rn(dz, dz);
    const float r0 = fadd(fadd(px.x, py.x), pz.x), r1 = fadd(fadd(px.y, py.y), pz.y);
    return (r0 < fmaxf(Si, S.x) ? 1u : 0u) | (r1 < fmaxf(Si, S.y) ? 2u : 0u);
}

__global__ void __launch_bounds__(256) k_hmax(const float* __restrict__ rad, uint32_t n, int reach, uint32_t* done,
                                              float* __restrict__ grid, uint32_t* part) {
    __shared__ float sh[256];
    float m = 0.0f;
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) m = fmaxf(m, rad[i]);
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] = fmaxf(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = __float_as_uint(sh[0]);
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
        if (last) *done = 0u;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        float h = 0.0f;
        for (uint32_t b = 0; b < gridDim.x; b++) h = fmaxf(h, __uint_as_float(__ldcg(&part[b])));
        const float side = 2.0f * h * (1.0f + 1.0f / 4096.0f) / (float)reach;
        grid[0] = side;
        grid[1] = side > 0.0f ? 1.0f / side : 0.0f;
        grid[2] = 2.0f * h;
    }
}

__global__ void k_cell_keys(const float* __restrict__ pos, uint32_t n, const float* __restrict__ grid, uint32_t mask,
                            uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t* d_status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int3 c = cell_of(pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u], grid[1]);
    if (cell_clamped(c)) atomicOr(d_status, SFGPU_STATUS_SPH_CELLS);
    keys[i] = bucket_of(c, mask);
    vals[i] = i;
}

__global__ void k_cell_gather(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ V, uint32_t n,
                              const float* __restrict__ slab, const float* __restrict__ u,
                              const float* __restrict__ grid, uint32_t* __restrict__ bstart,
                              uint32_t* __restrict__ bend, float4* __restrict__ px, float4* __restrict__ pv,
                              uint64_t* __restrict__ cell, float4* __restrict__ ph, float gamma,
                              uint64_t* __restrict__ mixv) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t b = (uint32_t)keys[k];
    if (k == 0 || (uint32_t)keys[k - 1] != b) bstart[b] = k;
    if (k == n - 1 || (uint32_t)keys[k + 1] != b) bend[b] = k + 1;
    const uint32_t p = V[k];
    const float* pos = slab;
    const float* vel = slab + (size_t)3 * n;
    const float x = pos[3u * p], y = pos[3u * p + 1u], z = pos[3u * p + 2u];
    px[k] = make_float4(x, y, z, slab[(size_t)9 * n + p]);
    pv[k] = make_float4(vel[3u * p], vel[3u * p + 1u], vel[3u * p + 2u], u[p]);
    cell[k] = pack_cell(cell_of(x, y, z, grid[1]));
    const float uu = u[p];
    const float hh = slab[(size_t)13 * n + p];
    ph[k] = make_float4(hh, uu, sqrtf(gamma * (gamma - 1.0f) * uu), 1.0f / hh);
    if (mixv) mixv[k] = sf_mix64(p);
}

// buckets that hold more than one cell; with q.est set, each 32-body
// chunk's cost estimate (the populations of its bodies' buckets)
__global__ void k_bucket_mix(const uint64_t* __restrict__ keys, uint32_t n, const uint32_t* __restrict__ bstart,
                             const uint32_t* __restrict__ bend, const uint64_t* __restrict__ cell,
                             uint32_t* __restrict__ bmix, sfchunk::ChunkQueue q) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t pop = 0;
    if (k < n) {
        const uint32_t b = (uint32_t)keys[k];
        const uint32_t s = bstart[b];
        if (k != s && cell[k] != cell[s]) bmix[b] = 1u;
        pop = bend[b] - s;
    }
    if (q.est && (k & ~31u) < n) sfchunk::note_cost(q, k >> 5, pop);
}

__device__ __forceinline__ bool density_pair(const float4& a, float hi, float ihi, const float4& q, float hj,
                                             float ihj, float& rho, uint32_t& count) {
    const float rx = fsub(a.x, q.x), ry = fsub(a.y, q.y), rz = fsub(a.z, q.z);
    float r2;
    if (!is_neighbour(rx, ry, rz, hi, hj, r2)) return false;
    const float r = r2 > 0.0f ? r2 * rsqrtf(r2) : 0.0f;
    count++;
    rho += q.w * 0.5f * (w_cubic(r, ihi) + w_cubic(r, ihj));
    return true;
}

// di: (rho, P/rho^2, c, 1/h) of body i; dj: (rho, P/rho^2, c, h) of body j
__device__ __forceinline__ void force_pair(const float4& a, float hi, const float4& di, const float4& vi,
                                           const float4& q, const float4& vj, const float4& dj, float alpha,
                                           float beta, float& ax, float& ay, float& az, float& du) {
    const float rx = fsub(a.x, q.x), ry = fsub(a.y, q.y), rz = fsub(a.z, q.z);
    const float hj = dj.w;
    float r2;
    if (!is_neighbour(rx, ry, rz, hi, hj, r2)) return;
    if (!(r2 > 0.0f)) return;
    const float rinv = rsqrtf(r2);
    const float r = r2 * rinv;
    const float g = 0.5f * (dw_cubic(r, di.w) + dw_cubic(r, __fdividef(1.0f, hj))) * rinv;
    const float vx = vi.x - vj.x, vy = vi.y - vj.y, vz = vi.z - vj.z;
    const float vr = vx * rx + vy * ry + vz * rz;
    const float h = 0.5f * (hi + hj);
    const float mu = __fdividef(h * vr, r2 + 0.01f * h * h);
    const float pi_ij = __fdividef(-alpha * 0.5f * (di.z + dj.z) * mu + beta * mu * mu, 0.5f * (di.x + dj.x));
    const float visc = vr < 0.0f ? pi_ij : 0.0f;  // approaching pairs only (computed for all, no branch)
    const float f = q.w * (di.y + dj.y + visc) * g;
    ax -= f * rx;
    ay -= f * ry;
    az -= f * rz;
    du += q.w * (di.y + 0.5f * visc) * g * vr;
}

// The per-body scan: the rows of cells within R of body k, each row's
// x-range of cells within R, every candidate tested; results in o0..o3,
// count, hs.
template <int REACH, bool FORCE, bool HASH>
__device__ __forceinline__ void body_scan(uint32_t k, const float4& a, float hi, float ihi, const float4& di,
                                          const float4& vi, float side, float inv, float R2, uint32_t mask,
                                          const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
                                          const uint32_t* __restrict__ bmix, const float4* __restrict__ px,
                                          const float4* __restrict__ ph, const float4* __restrict__ pv,
                                          const uint64_t* __restrict__ cell, const float4* __restrict__ pd,
                                          float alpha, float beta, const uint64_t* __restrict__ mixv, float& o0,
                                          float& o1, float& o2, float& o3, uint32_t& count, uint64_t& hs) {
    const int3 c0 = cell_of(a.x, a.y, a.z, inv);
    for (int dz = -REACH; dz <= REACH; dz++) {
        const float lz = (float)(c0.z + dz) * side;
        const float gz = fmaxf(0.f, fmaxf(lz - a.z, a.z - (lz + side)));
        for (int dy = -REACH; dy <= REACH; dy++) {
            const float ly = (float)(c0.y + dy) * side;
            const float gy = fmaxf(0.f, fmaxf(ly - a.y, a.y - (ly + side)));
            const float rem = R2 - (gy * gy + gz * gz);
            if (!(rem > 0.0f)) continue;
            // the cells of the row the sphere reaches (one cell of margin
            // each way is covered by the enlarged side)
            const float ext = sqrtf(rem) * MARGIN_HI;
            const int x0 = max(c0.x - REACH, (int)floorf((a.x - ext) * inv));
            const int x1 = min(c0.x + REACH, (int)floorf((a.x + ext) * inv));
            for (int cx = x0; cx <= x1; cx++) {
                const int3 c = make_int3(cx, c0.y + dy, c0.z + dz);
                const uint32_t b = bucket_of(c, mask);
                const uint32_t j0 = bstart[b], j1 = bend[b];
                if (j1 <= j0) continue;
                const uint64_t want = pack_cell(c);
                const uint32_t chk = bmix[b];
                if (!chk && cell[j0] != want) continue;
#pragma unroll 2
                for (uint32_t j = j0; j < j1; j++) {
                    if (chk && cell[j] != want) continue;
                    const float4 q = px[j];
                    if (!FORCE) {
                        const float4 hj = ph[j];
                        const bool hit = density_pair(a, hi, ihi, q, hj.x, hj.w, o0, count);
                        if (HASH && hit) hs += mixv[j];
                    } else if (j != k) {
                        force_pair(a, hi, di, vi, q, pv[j], pd[j], alpha, beta, o0, o1, o2, o3);
                    }
                }
            }
        }
    }
}

// Results of body k (sorted slot) to the slab: density pass rho, P, the
// (rho, P/rho^2, c, h) record, neighbour count and hash; force pass the
// added acceleration and du/dt.
template <bool FORCE, bool HASH>
__device__ __forceinline__ void body_store(uint32_t k, uint32_t n, const float4* __restrict__ ph,
                                           float4* __restrict__ pd, const uint32_t* __restrict__ V, float gamma,
                                           float* __restrict__ slab, float* __restrict__ dudt,
                                           uint32_t* __restrict__ nbr, uint64_t* __restrict__ hash, float o0,
                                           float o1, float o2, float o3, uint32_t count, uint64_t hs) {
    const uint32_t p = V[k];
    if (!FORCE) {
        const float4 hh = ph[k];
        const float rho = o0, u = hh.y;
        const float P = (gamma - 1.0f) * rho * u;
        pd[k] = make_float4(rho, rho > 0.0f ? P / (rho * rho) : 0.0f, hh.z, hh.x);
        slab[(size_t)14 * n + p] = rho;
        slab[(size_t)15 * n + p] = P;
        nbr[p] = count;
        if (HASH) hash[p] = hs;
    } else {
        float* acc = slab + (size_t)6 * n;
        acc[3u * p + 0u] += o0;
        acc[3u * p + 1u] += o1;
        acc[3u * p + 2u] += o2;
        dudt[p] = o3;
    }
}

// One thread per sorted body (sfgpu_params.sph_path 1 and 2).
template <int REACH, bool FORCE, bool HASH>
__global__ void __launch_bounds__(128) k_cubic_body(uint32_t n, const float* __restrict__ grid, uint32_t mask,
                                                    const uint32_t* __restrict__ bstart,
                                                    const uint32_t* __restrict__ bend,
                                                    const uint32_t* __restrict__ bmix, const float4* __restrict__ px,
                                                    const float4* __restrict__ ph, const float4* __restrict__ pv,
                                                    const uint64_t* __restrict__ cell, float4* __restrict__ pd,
                                                    const uint32_t* __restrict__ V, float gamma, float alpha,
                                                    float beta, float* __restrict__ slab, float* __restrict__ dudt,
                                                    uint32_t* __restrict__ nbr, const uint64_t* __restrict__ mixv,
                                                    uint64_t* __restrict__ hash) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float side = grid[0], inv = grid[1], R = grid[2];
    const float R2 = R * R * MARGIN_HI;
    const float4 a = px[k];
    const float hi = ph[k].x;
    const float ihi = 1.0f / hi;
    float4 di = make_float4(0.f, 0.f, 0.f, 0.f), vi = di;
    if (FORCE) {
        di = pd[k];
        di.w = ihi;  // the pair terms take body i's 1 / h
        vi = pv[k];
    }
    float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
    uint32_t count = 0;
    uint64_t hs = 0;
    body_scan<REACH, FORCE, HASH>(k, a, hi, ihi, di, vi, side, inv, R2, mask, bstart, bend, bmix, px, ph, pv, cell,
                                  pd, alpha, beta, mixv, o0, o1, o2, o3, count, hs);
    body_store<FORCE, HASH>(k, n, ph, pd, V, gamma, slab, dudt, nbr, hash, o0, o1, o2, o3, count, hs);
}

// The default pass (sph_path 0): one warp per 32 consecutive sorted bodies,
// which sit close together.  The warp visits the union of its bodies'
// rows and row x-ranges (the per-body scan above with REACH = 1); each cell's
// bodies are staged in shared memory 32 at a time with coalesced loads.  A
// lane first tests every staged candidate against its body (the FP32
// neighbour decision, on cells its own scan visits) into a bit mask, then
// evaluates its hits in ascending order: the warp iterates as many times as
// its busiest lane has hits, not once per candidate, and every body adds
// the same terms in the same order as the per-body scan, so both give the
// same bits.  A warp whose bodies span more than 3 cells on an axis (sparse
// regions) runs the per-body scan instead.
constexpr int CW_WARPS = 4;
// Register budgets by the resident blocks each pass asks for (without a
// hint ptxas settles at 56 registers with spills for the density passes,
// 64 with spills for the force pass).  Measured on the 262,144-body Plummer
// gas: the force pass at 96 registers (one block asked for, no spills)
// 0.58 ms against 0.67 at 64; the density passes at 80 registers (six
// blocks) 0.435 ms against 0.449 at 64.
constexpr int CW_MIN_BLOCKS = 6;
constexpr int CW_MIN_BLOCKS_FORCE = 1;
template <int REACH, bool FORCE, bool HASH>
__device__ __forceinline__ void cubic_chunk(uint32_t k0, uint32_t n, const float* __restrict__ grid, uint32_t mask,
                                            const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
                                            const uint32_t* __restrict__ bmix, const float4* __restrict__ px,
                                            const float4* __restrict__ ph, const float4* __restrict__ pv,
                                            const uint64_t* __restrict__ cell, float4* __restrict__ pd,
                                            const uint32_t* __restrict__ V, float gamma, float alpha, float beta,
                                            float* __restrict__ slab, float* __restrict__ dudt,
                                            uint32_t* __restrict__ nbr, const uint64_t* __restrict__ mixv,
                                            uint64_t* __restrict__ hash, float4* sq, float4* sh, float4* sv,
                                            uint64_t* sm, float* st4) {
    const int lane = threadIdx.x & 31;
    if (k0 >= n) return;
    const uint32_t k = k0 + (uint32_t)lane;
    const bool live = k < n;
    const uint32_t kk = live ? k : n - 1u;  // a lane past the end shadows the warp's last body
    const float side = grid[0], inv = grid[1], R = grid[2];
    const float R2 = R * R * MARGIN_HI;
    const float4 a = px[kk];
    const float hi = ph[kk].x;
    const float ihi = 1.0f / hi;
    const float Si = fmul(fmul(2.0f, hi), fmul(2.0f, hi));  // (2 h_i)^2
    float4 di = make_float4(0.f, 0.f, 0.f, 0.f), vi = di;
    if (FORCE) {
        di = pd[kk];
        di.w = ihi;
        vi = pv[kk];
    }
    float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
    uint32_t count = 0;
    uint64_t hs = 0;
    const int3 c0 = cell_of(a.x, a.y, a.z, inv);
    const int zlo = __reduce_min_sync(0xffffffffu, c0.z), zhi = __reduce_max_sync(0xffffffffu, c0.z);
    const int ylo = __reduce_min_sync(0xffffffffu, c0.y), yhi = __reduce_max_sync(0xffffffffu, c0.y);
    const int xlo = __reduce_min_sync(0xffffffffu, c0.x), xhi = __reduce_max_sync(0xffffffffu, c0.x);
    // cell spans as unsigned differences (no overflow for far-apart cells);
    // a body beyond the packed key's range takes the per-body scan
    const bool compact = (uint32_t)zhi - (uint32_t)zlo <= 2u && (uint32_t)yhi - (uint32_t)ylo <= 2u &&
                         (uint32_t)xhi - (uint32_t)xlo <= 2u && !__any_sync(0xffffffffu, cell_clamped(c0));
    if (!compact) {
        if (live) {
            body_scan<REACH, FORCE, HASH>(k, a, hi, ihi, di, vi, side, inv, R2, mask, bstart, bend, bmix, px, ph, pv,
                                      cell, pd, alpha, beta, mixv, o0, o1, o2, o3, count, hs);
            body_store<FORCE, HASH>(k, n, ph, pd, V, gamma, slab, dudt, nbr, hash, o0, o1, o2, o3, count, hs);
        }
        return;
    }
    for (int cz = zlo - REACH; cz <= zhi + REACH; cz++) {
        const float lz = (float)cz * side;
        const float gz = fmaxf(0.f, fmaxf(lz - a.z, a.z - (lz + side)));
        for (int cy = ylo - REACH; cy <= yhi + REACH; cy++) {
            // this lane's part of the row, exactly as its per-body scan
            // would take it (x0 > x1: none)
            const float ly = (float)cy * side;
            const float gy = fmaxf(0.f, fmaxf(ly - a.y, a.y - (ly + side)));
            const float rem = R2 - (gy * gy + gz * gz);
            int x0 = 1, x1 = 0;
            if (live && rem > 0.0f && cz >= c0.z - REACH && cz <= c0.z + REACH && cy >= c0.y - REACH &&
                cy <= c0.y + REACH) {
                const float ext = sqrtf(rem) * MARGIN_HI;
                x0 = max(c0.x - REACH, (int)floorf((a.x - ext) * inv));
                x1 = min(c0.x + REACH, (int)floorf((a.x + ext) * inv));
            }
            const bool any = x0 <= x1;
            if (!__any_sync(0xffffffffu, any)) continue;
            const int wx0 = __reduce_min_sync(0xffffffffu, any ? x0 : INT_MAX);
            const int wx1 = __reduce_max_sync(0xffffffffu, any ? x1 : INT_MIN);
            for (int cx = wx0; cx <= wx1; cx++) {
                const int3 c = make_int3(cx, cy, cz);
                const uint32_t b = bucket_of(c, mask);
                const uint32_t j0 = bstart[b], j1 = bend[b];
                if (j1 <= j0) continue;
                const uint64_t want = pack_cell(c);
                const uint32_t chk = bmix[b];
                if (!chk && cell[j0] != want) continue;
                const bool mine = cx >= x0 && cx <= x1;  // the cell is on this lane's own scan
                for (uint32_t jb = j0; jb < j1; jb += 32u) {
                    const uint32_t j = jb + (uint32_t)lane;
                    const bool ok = j < j1 && (!chk || cell[j] == want);
                    __syncwarp();
                    if (ok) {
                        const float4 qj = px[j];
                        float hj;
                        sq[lane] = qj;
                        if (FORCE) {
                            const float4 dj = pd[j];
                            sh[lane] = dj;
                            sv[lane] = pv[j];
                            hj = dj.w;
                        } else {
                            const float4 pj = ph[j];
                            sh[lane] = pj;
                            if (HASH) sm[lane] = mixv[j];
                            hj = pj.x;
                        }
                        if (!FORCE) {  // the paired test's operands: -x, -y, -z and (2 h)^2
                            const float sj = fmul(2.0f, hj);
                            st4[lane] = -qj.x;
                            st4[32 + lane] = -qj.y;
                            st4[64 + lane] = -qj.z;
                            st4[96 + lane] = fmul(sj, sj);
                        }
                    }
                    const uint32_t vm = __ballot_sync(0xffffffffu, ok);
                    __syncwarp();
                    // pass 1: the neighbour decisions of this lane's body
                    // (a full batch unrolled: its tests are independent)
                    uint32_t hits = 0u;
                    auto test = [&](int t) {
                        const float4 q = sq[t];
                        const float hj = FORCE ? sh[t].w : sh[t].x;
                        float r2;
                        const bool nb = is_neighbour(fsub(a.x, q.x), fsub(a.y, q.y), fsub(a.z, q.z), hi, hj, r2);
                        if (nb && (!FORCE || jb + (uint32_t)t != k)) hits |= 1u << t;
                    };
                    if (mine) {
                        if (!FORCE && vm == 0xffffffffu) {
                            // two candidates per paired FP32 instruction
                            // (neighbours2: the same decision bits as
                            // is_neighbour)
                            const float2* tx = reinterpret_cast<const float2*>(st4);
                            const float2* ty = reinterpret_cast<const float2*>(st4 + 32);
                            const float2* tz = reinterpret_cast<const float2*>(st4 + 64);
                            const float2* tS = reinterpret_cast<const float2*>(st4 + 96);
                            const float2 ax2 = make_float2(a.x, a.x), ay2 = make_float2(a.y, a.y);
                            const float2 az2 = make_float2(a.z, a.z);
#pragma unroll 8
                            for (int u = 0; u < 16; u++)
                                hits |= neighbours2(ax2, ay2, az2, tx[u], ty[u], tz[u], tS[u], Si) << (2 * u);
                        } else if (vm == 0xffffffffu) {
#pragma unroll 8
                            for (int t = 0; t < 32; t++) test(t);
                        } else {
                            for (uint32_t mm = vm; mm; mm &= mm - 1u) test(__ffs(mm) - 1);
                        }
                    }
                    // pass 2: the terms, in candidate order, two per round
                    // (the second's arithmetic overlaps the first's; the
                    // sums take them in order)
                    auto term = [&](int t) {
                        const float4 q = sq[t];
                        if (!FORCE) {
                            const float4 hj = sh[t];
                            density_pair(a, hi, ihi, q, hj.x, hj.w, o0, count);
                            if (HASH) hs += sm[t];
                        } else {
                            force_pair(a, hi, di, vi, q, sv[t], sh[t], alpha, beta, o0, o1, o2, o3);
                        }
                    };
                    while (__any_sync(0xffffffffu, hits != 0u)) {
                        if (hits) {
                            const int t1 = __ffs(hits) - 1;
                            hits &= hits - 1u;
                            const int t2 = hits ? __ffs(hits) - 1 : -1;
                            if (t2 >= 0) hits &= hits - 1u;
                            term(t1);
                            if (t2 >= 0) term(t2);
                        }
                    }
                }
            }
        }
    }
    if (live) body_store<FORCE, HASH>(k, n, ph, pd, V, gamma, slab, dudt, nbr, hash, o0, o1, o2, o3, count, hs);
}

// The pass: one resident wave of persistent warps taking chunks of 32
// sorted bodies heaviest first (chunks.cuh).
template <int REACH, bool FORCE, bool HASH>
__global__ void __launch_bounds__(CW_WARPS * 32, FORCE ? CW_MIN_BLOCKS_FORCE : CW_MIN_BLOCKS) k_cubic_warp(uint32_t n, const float* __restrict__ grid,
                                                             uint32_t mask, const uint32_t* __restrict__ bstart,
                                                             const uint32_t* __restrict__ bend,
                                                             const uint32_t* __restrict__ bmix,
                                                             const float4* __restrict__ px,
                                                             const float4* __restrict__ ph,
                                                             const float4* __restrict__ pv,
                                                             const uint64_t* __restrict__ cell,
                                                             float4* __restrict__ pd, const uint32_t* __restrict__ V,
                                                             float gamma, float alpha, float beta,
                                                             float* __restrict__ slab, float* __restrict__ dudt,
                                                             uint32_t* __restrict__ nbr,
                                                             const uint64_t* __restrict__ mixv,
                                                             uint64_t* __restrict__ hash, sfchunk::ChunkQueue q) {
    __shared__ float4 s_q[CW_WARPS][32];  // candidate x, y, z, m
    __shared__ float4 s_h[CW_WARPS][32];  // density: (h, u, c, 1/h); force: (rho, P/rho^2, c, h)
    __shared__ float4 s_v[CW_WARPS][32];  // force: vx, vy, vz, u
    __shared__ uint64_t s_m[CW_WARPS][HASH ? 32 : 1];
    __shared__ __align__(16) float s_t[CW_WARPS][4 * 32];  // -x, -y, -z, (2 h)^2 of each candidate
    const int w = threadIdx.x >> 5;
    sfchunk::Taker t = sfchunk::taker(q);
    for (;;) {
        const uint32_t c = sfchunk::next(q, t);
        if (c == 0xFFFFFFFFu) break;
        const long long t0 = clock64();
        cubic_chunk<REACH, FORCE, HASH>(c * 32u, n, grid, mask, bstart, bend, bmix, px, ph, pv, cell, pd, V, gamma, alpha,
                                 beta, slab, dudt, nbr, mixv, hash, s_q[w], s_h[w], s_v[w], s_m[w], s_t[w]);
        sfchunk::record(q, FORCE ? 1 : 0, c, clock64() - t0);
    }
    sfchunk::warp_exit(q, gridDim.x * CW_WARPS);
}

template <int REACH>
int launch_passes(sfgpu_sim* s, CubicWork* w, uint32_t mask, uint32_t* nbr, uint64_t* hash) {
    cudaStream_t st = s->stream;
    const uint32_t n = s->n;
    const float gamma = (float)s->p.sph_gamma, alpha = (float)s->p.sph_alpha, beta = (float)s->p.sph_beta;
    const bool warp = w->path == 0 || w->path == 3;
    const uint32_t bb = sf_ceil_div(n, 128);
    // one resident wave of each warp pass (chunks.cuh)
    static uint32_t wave[3] = {0, 0, 0};  // density, density with hashes, force
    const uint32_t most = sf_ceil_div(w->q.nchunks, CW_WARPS);
    if (!wave[0]) {
        wave[0] = sfchunk::wave_blocks(k_cubic_warp<REACH, false, false>, CW_WARPS * 32, 0xFFFFFFFFu);
        wave[1] = sfchunk::wave_blocks(k_cubic_warp<REACH, false, true>, CW_WARPS * 32, 0xFFFFFFFFu);
        wave[2] = sfchunk::wave_blocks(k_cubic_warp<REACH, true, false>, CW_WARPS * 32, 0xFFFFFFFFu);
    }
    int tk = s->timer.begin(st, "sph_density");
    if (warp) {
        sfchunk::k_chunk_order<<<1, 1024, 0, st>>>(w->q, 0);
        SF_CHECK_LAUNCH();
    }
    if (warp && hash)
        k_cubic_warp<REACH, false, true><<<std::min(wave[1], most), CW_WARPS * 32, 0, st>>>(
            n, w->grid, mask, w->bstart, w->bend, w->bmix, w->px, w->ph, w->pv, w->cell, w->pd, w->vals, gamma, alpha,
            beta, s->slab, s->dudt, nbr, w->mixv, hash, w->q);
    else if (warp)
        k_cubic_warp<REACH, false, false><<<std::min(wave[0], most), CW_WARPS * 32, 0, st>>>(
            n, w->grid, mask, w->bstart, w->bend, w->bmix, w->px, w->ph, w->pv, w->cell, w->pd, w->vals, gamma, alpha,
            beta, s->slab, s->dudt, nbr, nullptr, nullptr, w->q);
    else if (hash)
        k_cubic_body<REACH, false, true><<<bb, 128, 0, st>>>(n, w->grid, mask, w->bstart, w->bend, w->bmix, w->px,
                                                             w->ph, w->pv, w->cell, w->pd, w->vals, gamma, alpha,
                                                             beta, s->slab, s->dudt, nbr, w->mixv, hash);
    else
        k_cubic_body<REACH, false, false><<<bb, 128, 0, st>>>(n, w->grid, mask, w->bstart, w->bend, w->bmix, w->px,
                                                              w->ph, w->pv, w->cell, w->pd, w->vals, gamma, alpha,
                                                              beta, s->slab, s->dudt, nbr, nullptr, nullptr);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    tk = s->timer.begin(st, "sph_force");
    if (warp) {
        sfchunk::k_chunk_order<<<1, 1024, 0, st>>>(w->q, 1);
        SF_CHECK_LAUNCH();
    }
    if (warp)
        k_cubic_warp<REACH, true, false><<<std::min(wave[2], most), CW_WARPS * 32, 0, st>>>(
            n, w->grid, mask, w->bstart, w->bend, w->bmix, w->px, w->ph, w->pv, w->cell, w->pd, w->vals, gamma, alpha,
            beta, s->slab, s->dudt, nbr, nullptr, nullptr, w->q);
    else
        k_cubic_body<REACH, true, false><<<bb, 128, 0, st>>>(n, w->grid, mask, w->bstart, w->bend, w->bmix, w->px,
                                                             w->ph, w->pv, w->cell, w->pd, w->vals, gamma, alpha,
                                                             beta, s->slab, s->dudt, nbr, nullptr, nullptr);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    return SFGPU_OK;
}

}  // namespace

uint32_t* sf_sph_neighbour_counts(sfgpu_sim* s);
uint64_t* sf_sph_neighbour_hashes(sfgpu_sim* s);

int sf_sph_cubic_alloc(sfgpu_sim* s) {
    CubicWork* w = new CubicWork();
    s->sph_cubic = w;
    const uint32_t n = std::max<uint32_t>(s->n, 1);
    w->path = s->p.sph_path;
    w->reach = (s->p.sph_path == 1 || s->p.sph_path == 3) ? 2 : 1;
    w->tbits = 1;
    while ((1u << w->tbits) < 2u * n) w->tbits++;
    w->tsize = 1u << w->tbits;
    SF_CUDA(cudaMalloc(&w->keys, sizeof(uint64_t) * n));
    SF_CUDA(cudaMalloc(&w->vals, sizeof(uint32_t) * n));
    if (sf_sort_alloc(w->sort, n) != SFGPU_OK) return SFGPU_FAILURE;
    if (s->p.spin_limit) w->sort.spin_limit = s->p.spin_limit;
    SF_CUDA(cudaMalloc(&w->bstart, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->bend, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->px, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->pv, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->pd, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->ph, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->bmix, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->cell, sizeof(uint64_t) * n));
    if (s->p.flags & SFGPU_FLAG_STATS) SF_CUDA(cudaMalloc(&w->mixv, sizeof(uint64_t) * n));
    SF_CUDA(cudaMalloc(&w->grid, sizeof(float) * 4));
    SF_CUDA(cudaMalloc(&w->done, sizeof(uint32_t) * (1024 + 1)));
    SF_CUDA(cudaMemset(w->done, 0, sizeof(uint32_t) * (1024 + 1)));
    if (sfchunk::alloc(w->q, n) != SFGPU_OK) return SFGPU_FAILURE;
    SF_CUDA(cudaMalloc(&s->u, sizeof(float) * n));
    SF_CUDA(cudaMalloc(&s->dudt, sizeof(float) * n));
    SF_CUDA(cudaMemset(s->u, 0, sizeof(float) * n));
    SF_CUDA(cudaMemset(s->dudt, 0, sizeof(float) * n));
    return SFGPU_OK;
}

void sf_sph_cubic_free(sfgpu_sim* s) {
    CubicWork* w = (CubicWork*)s->sph_cubic;
    if (!w) return;
    cudaFree(w->keys);
    cudaFree(w->vals);
    sf_sort_free(w->sort);
    cudaFree(w->bstart);
    cudaFree(w->bend);
    cudaFree(w->px);
    cudaFree(w->pv);
    cudaFree(w->pd);
    cudaFree(w->ph);
    cudaFree(w->bmix);
    cudaFree(w->cell);
    cudaFree(w->mixv);
    cudaFree(w->grid);
    cudaFree(w->done);
    sfchunk::release(w->q);
    delete w;
    s->sph_cubic = nullptr;
}

int sf_sph_cubic(sfgpu_sim* s) {
    CubicWork* w = (CubicWork*)s->sph_cubic;
    const uint32_t n = s->n;
    cudaStream_t st = s->stream;
    const uint32_t hb = std::min<uint32_t>(sf_ceil_div(n, 256), 1024);
    int tk = s->timer.begin(st, "sph_grid");
    k_hmax<<<hb, 256, 0, st>>>(s->slab + (size_t)13 * n, n, w->reach, w->done, w->grid, w->done + 1);
    SF_CHECK_LAUNCH();
    const uint32_t mask = w->tsize - 1;
    const uint32_t nb = sf_ceil_div(n, 256);
    k_cell_keys<<<nb, 256, 0, st>>>(s->slab, n, w->grid, mask, w->keys, w->vals, s->d_status);
    SF_CHECK_LAUNCH();
    if (sf_sort_pairs(w->keys, w->vals, n, (int)w->tbits, w->sort, st, s->d_status) != SFGPU_OK)
        return SFGPU_FAILURE;
    SF_CUDA(cudaMemsetAsync(w->bstart, 0, sizeof(uint32_t) * w->tsize, st));
    SF_CUDA(cudaMemsetAsync(w->bend, 0, sizeof(uint32_t) * w->tsize, st));
    SF_CUDA(cudaMemsetAsync(w->bmix, 0, sizeof(uint32_t) * w->tsize, st));
    const float gamma = (float)s->p.sph_gamma;
    k_cell_gather<<<nb, 256, 0, st>>>(w->keys, w->vals, n, s->slab, s->u, w->grid, w->bstart, w->bend, w->px, w->pv,
                                      w->cell, w->ph, gamma, w->mixv);
    SF_CHECK_LAUNCH();
    sfchunk::ChunkQueue q = w->q;
    if (w->path != 0 && w->path != 3) q.est = nullptr;  // the per-body passes take no chunks
    k_bucket_mix<<<nb, 256, 0, st>>>(w->keys, n, w->bstart, w->bend, w->cell, w->bmix, q);
    SF_CHECK_LAUNCH();

    s->timer.end(st, tk);
    uint32_t* nbr = sf_sph_neighbour_counts(s);
    uint64_t* hash = w->mixv ? sf_sph_neighbour_hashes(s) : nullptr;
    if (w->reach == 1) return launch_passes<1>(s, w, mask, nbr, hash);
    return launch_passes<2>(s, w, mask, nbr, hash);
}

// ---- check of the paired neighbour test ---------------------------------------
namespace {
__device__ __forceinline__ uint32_t chk_mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
// n random cases of a body and two candidates placed about 2 max(h_i, h_j)
// away (r^2 within a few ulps of the bound in many of them): neighbours2
// against is_neighbour, mismatches counted in *bad.
__global__ void k_neighbours2_check(uint32_t n, uint32_t seed, unsigned long long* bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto u = [&](uint32_t k) {
        return (float)(chk_mix(seed * 0x9E3779B9u ^ chk_mix(16u * i + k)) >> 8) * (1.0f / 16777216.0f);
    };
    const float ax = fsub(fmul(2.0f, u(0)), 1.0f), ay = fsub(fmul(2.0f, u(1)), 1.0f), az = fsub(fmul(2.0f, u(2)), 1.0f);
    const float hi = fadd(0.01f, fmul(0.09f, u(3)));
    float qx[2], qy[2], qz[2], hj[2];
    uint32_t want = 0;
#pragma unroll
    for (int c = 0; c < 2; c++) {
        hj[c] = fadd(0.01f, fmul(0.09f, u(4 + 5 * c)));
        const float R = fmul(2.0f, fmaxf(hi, hj[c]));
        const float dx = fsub(fmul(2.0f, u(5 + 5 * c)), 1.0f), dy = fsub(fmul(2.0f, u(6 + 5 * c)), 1.0f);
        const float dz = fsub(fmul(2.0f, u(7 + 5 * c)), 1.0f);
        const float len = fadd(__fsqrt_rn(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz))), 1e-6f);
        const float sc = fdiv(R, len);
        qx[c] = fadd(ax, fmul(dx, sc));
        qy[c] = fadd(ay, fmul(dy, sc));
        qz[c] = fadd(az, fmul(dz, sc));
        float r2;
        if (is_neighbour(fsub(ax, qx[c]), fsub(ay, qy[c]), fsub(az, qz[c]), hi, hj[c], r2)) want |= 1u << c;
    }
    const float si = fmul(2.0f, hi), s0 = fmul(2.0f, hj[0]), s1 = fmul(2.0f, hj[1]);
    const uint32_t got = neighbours2(make_float2(ax, ax), make_float2(ay, ay), make_float2(az, az),
                                     make_float2(-qx[0], -qx[1]), make_float2(-qy[0], -qy[1]),
                                     make_float2(-qz[0], -qz[1]), make_float2(fmul(s0, s0), fmul(s1, s1)),
                                     fmul(si, si));
    if (got != want) atomicAdd(bad, 1ull);
}
}  // namespace

int sf_sph_neighbours2_check(uint32_t n, uint32_t seed, unsigned long long* d_bad, cudaStream_t st) {
    k_neighbours2_check<<<sf_ceil_div(n, 256), 256, 0, st>>>(n, seed, d_bad);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}
