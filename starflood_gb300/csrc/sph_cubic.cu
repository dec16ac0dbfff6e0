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
// Neighbour search: cells of side 2 h_max (slightly enlarged, so that FP32
// rounding can never put two neighbours two cells apart), hashed into a
// table of 2^k >= 2N buckets; bodies are radix sorted by bucket, so a cell's
// bodies are one contiguous run of records.  Each pass then works a warp per
// 32-body slice of a cell (k_cubic_cells): the slice's bodies share their 27
// neighbour cells, whose records the warp reads together (one broadcast load
// per record); bodies whose cell coordinates differ from the scanned cell's
// (hash collisions) are skipped, so none is counted twice.
#include "internal.cuh"

namespace {

constexpr int CELL_BITS = 21;  // per axis in the packed cell key
constexpr int32_t CELL_OFF = 1 << (CELL_BITS - 1);
constexpr float PI_F = 3.14159265358979323846f;

struct CubicWork {
    uint32_t tbits = 0, tsize = 0;
    uint64_t* keys = nullptr;
    uint32_t* vals = nullptr;
    SortWork sort;
    uint32_t* bstart = nullptr;
    uint32_t* bend = nullptr;
    float4* px = nullptr;      // sorted x, y, z, m
    float4* pv = nullptr;      // sorted vx, vy, vz, u
    float4* pd = nullptr;      // sorted rho, P/rho^2, c, h
    float4* ph = nullptr;      // sorted h, u, c
    uint32_t* bmix = nullptr;  // per bucket: holds more than one cell
    uint2* items = nullptr;    // (bucket, first body) of every 32-body slice
    uint32_t* counters = nullptr;  // [0] items [1] density ticket [2] force ticket
    uint64_t* cell = nullptr;  // sorted packed cell coordinates
    float* grid = nullptr;     // [0] cell side, [1] 1/side
    uint32_t* done = nullptr;
};

__device__ __forceinline__ int3 cell_of(float x, float y, float z, float inv) {
    return make_int3((int)floorf(x * inv), (int)floorf(y * inv), (int)floorf(z * inv));
}
__device__ __forceinline__ uint64_t pack_cell(int3 c) {
    auto f = [](int v) {
        v = max(-CELL_OFF, min(CELL_OFF - 1, v));
        return (uint64_t)(uint32_t)(v + CELL_OFF);
    };
    return (f(c.x) << (2 * CELL_BITS)) | (f(c.y) << CELL_BITS) | f(c.z);
}
// Bucket = the low bits of the cell's Morton code (3-way bit interleave of
// the offset coordinates): neighbouring cells land in nearby buckets, so
// bodies sorted by bucket are also sorted in space and consecutive threads
// scan overlapping neighbourhoods.  Cells further apart than the table's
// period share buckets; those buckets are filtered by cell key.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // low 10 bits to every third bit
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ uint32_t bucket_of(int3 c, uint32_t mask) {
    const uint32_t x = (uint32_t)(c.x + CELL_OFF), y = (uint32_t)(c.y + CELL_OFF), z = (uint32_t)(c.z + CELL_OFF);
    return ((spread3(x) << 2) | (spread3(y) << 1) | spread3(z)) & mask;
}

__device__ __forceinline__ float w_cubic(float r, float h) {
    const float q = r / h;
    const float s = 1.0f / (PI_F * h * h * h);
    if (q < 1.0f) return s * (1.0f - 1.5f * q * q + 0.75f * q * q * q);
    if (q < 2.0f) {
        const float t = 2.0f - q;
        return s * 0.25f * t * t * t;
    }
    return 0.0f;
}
__device__ __forceinline__ float dw_cubic(float r, float h) {
    const float q = r / h;
    const float s = 1.0f / (PI_F * h * h * h * h);
    if (q < 1.0f) return s * (-3.0f * q + 2.25f * q * q);
    if (q < 2.0f) {
        const float t = 2.0f - q;
        return s * (-0.75f * t * t);
    }
    return 0.0f;
}
// the FP32 neighbour decision (same expression as the oracle)
__device__ __forceinline__ bool is_neighbour(float dx, float dy, float dz, float hi, float hj, float& r2) {
    r2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
    const float s = fmul(2.0f, fmaxf(hi, hj));
    return r2 < fmul(s, s);
}

__global__ void __launch_bounds__(256) k_hmax(const float* __restrict__ rad, uint32_t n, uint32_t* done,
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
        const float side = 2.0f * h * (1.0f + 1.0f / 4096.0f);
        grid[0] = side;
        grid[1] = side > 0.0f ? 1.0f / side : 0.0f;
    }
}

__global__ void k_cell_keys(const float* __restrict__ pos, uint32_t n, const float* __restrict__ grid, uint32_t mask,
                            uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int3 c = cell_of(pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u], grid[1]);
    keys[i] = bucket_of(c, mask);
    vals[i] = i;
}

__global__ void k_cell_gather(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ V, uint32_t n,
                              const float* __restrict__ slab, const float* __restrict__ u,
                              const float* __restrict__ grid, uint32_t* __restrict__ bstart,
                              uint32_t* __restrict__ bend, float4* __restrict__ px, float4* __restrict__ pv,
                              uint64_t* __restrict__ cell, float4* __restrict__ ph, float gamma) {
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
    ph[k] = make_float4(slab[(size_t)13 * n + p], uu, sqrtf(gamma * (gamma - 1.0f) * uu), 0.0f);
}

// ---- warp per cell ------------------------------------------------------------
// One work item per 32-body slice of an occupied bucket.  For a bucket that
// holds one cell (the usual case with a table of >= 2N buckets) the slice's
// 32 bodies share their 27 neighbour cells, so the warp walks those cells'
// records together: every record is one broadcast load for the whole warp
// and each lane tests it against its own body.  Lanes 0..26 first look up the
// 27 neighbour buckets side by side; a neighbour bucket that holds another
// cell is skipped whole, one that holds several cells is filtered record by
// record.  A centre bucket that holds several cells (hash collision) runs
// each lane's own 27-cell scan (body_direct).  Records: density 32 B
// (x,y,z,m | h,u,c), force 48 B (x,y,z,m | v,u | rho,P/rho^2,c,h).
constexpr int WARP_BLOCK = 128;

__device__ __forceinline__ void density_pair(const float4& a, float hi, const float4& q, float hj, float& rho,
                                             uint32_t& count) {
    const float rx = fsub(a.x, q.x), ry = fsub(a.y, q.y), rz = fsub(a.z, q.z);
    float r2;
    if (!is_neighbour(rx, ry, rz, hi, hj, r2)) return;
    const float r = sqrtf(r2);
    count++;
    rho += q.w * 0.5f * (w_cubic(r, hi) + w_cubic(r, hj));
}

__device__ __forceinline__ void force_pair(const float4& a, float hi, const float4& di, const float4& vi,
                                           const float4& q, const float4& vj, const float4& dj, float alpha,
                                           float beta, float& ax, float& ay, float& az, float& du) {
    const float rx = fsub(a.x, q.x), ry = fsub(a.y, q.y), rz = fsub(a.z, q.z);
    const float hj = dj.w;
    float r2;
    if (!is_neighbour(rx, ry, rz, hi, hj, r2)) return;
    const float r = sqrtf(r2);
    if (!(r > 0.0f)) return;
    const float g = 0.5f * (dw_cubic(r, hi) + dw_cubic(r, hj)) / r;
    const float vx = vi.x - vj.x, vy = vi.y - vj.y, vz = vi.z - vj.z;
    const float vr = vx * rx + vy * ry + vz * rz;
    float visc = 0.0f;
    if (vr < 0.0f) {
        const float h = 0.5f * (hi + hj);
        const float mu = h * vr / (r2 + 0.01f * h * h);
        visc = (-alpha * 0.5f * (di.z + dj.z) * mu + beta * mu * mu) / (0.5f * (di.x + dj.x));
    }
    const float f = q.w * (di.y + dj.y + visc) * g;
    ax -= f * rx;
    ay -= f * ry;
    az -= f * rz;
    du += q.w * (di.y + 0.5f * visc) * g * vr;
}

// one body against its 27 neighbour cells, its own scan
template <bool FORCE>
__device__ __forceinline__ void body_direct(uint32_t k, uint32_t mask, const float* __restrict__ grid,
                            const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
                            const float4* __restrict__ px, const float4* __restrict__ ph,
                            const float4* __restrict__ pv, const uint64_t* __restrict__ cell,
                            const float4* __restrict__ pd, float alpha, float beta, float& o0, float& o1,
                            float& o2, float& o3, uint32_t& count) {
    const float4 a = px[k];
    const float hi = ph[k].x;
    const int3 c0 = cell_of(a.x, a.y, a.z, grid[1]);
    float4 di = make_float4(0.f, 0.f, 0.f, 0.f), vi = di;
    if (FORCE) {
        di = pd[k];
        vi = pv[k];
    }
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int3 c = make_int3(c0.x + dx, c0.y + dy, c0.z + dz);
                const uint64_t want = pack_cell(c);
                const uint32_t b = bucket_of(c, mask);
                const uint32_t j0 = bstart[b], j1 = bend[b];
                for (uint32_t j = j0; j < j1; j++) {
                    if (cell[j] != want) continue;
                    if (!FORCE) {
                        density_pair(a, hi, px[j], ph[j].x, o0, count);
                    } else if (j != k) {
                        force_pair(a, hi, di, vi, px[j], pv[j], pd[j], alpha, beta, o0, o1, o2, o3);
                    }
                }
            }
}

template <bool FORCE>
__device__ __forceinline__ void finish_body(uint32_t k, uint32_t n, float gamma, const float4* __restrict__ ph,
                                            const uint32_t* __restrict__ V, float4* __restrict__ pd,
                                            float* __restrict__ slab, float* __restrict__ dudt,
                                            uint32_t* __restrict__ nbr, float o0, float o1, float o2, float o3,
                                            uint32_t count) {
    const uint32_t p = V[k];
    if (!FORCE) {
        const float4 hh = ph[k];
        const float rho = o0, u = hh.y;
        const float P = (gamma - 1.0f) * rho * u;
        pd[k] = make_float4(rho, rho > 0.0f ? P / (rho * rho) : 0.0f, hh.z, hh.x);
        slab[(size_t)14 * n + p] = rho;
        slab[(size_t)15 * n + p] = P;
        nbr[p] = count;
    } else {
        float* acc = slab + (size_t)6 * n;
        acc[3u * p + 0u] += o0;
        acc[3u * p + 1u] += o1;
        acc[3u * p + 2u] += o2;
        dudt[p] = o3;
    }
}

// one thread per body, each scanning its own 27 cells (sf_params.sph_path 0)
template <bool FORCE>
__global__ void __launch_bounds__(128) k_cubic_body(uint32_t n, const float* __restrict__ grid, uint32_t mask,
                                                    const uint32_t* __restrict__ bstart,
                                                    const uint32_t* __restrict__ bend, const float4* __restrict__ px,
                                                    const float4* __restrict__ ph, const float4* __restrict__ pv,
                                                    const uint64_t* __restrict__ cell, float4* __restrict__ pd,
                                                    const uint32_t* __restrict__ V, float gamma, float alpha,
                                                    float beta, float* __restrict__ slab, float* __restrict__ dudt,
                                                    uint32_t* __restrict__ nbr) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
    uint32_t count = 0;
    body_direct<FORCE>(k, mask, grid, bstart, bend, px, ph, pv, cell, pd, alpha, beta, o0, o1, o2, o3, count);
    finish_body<FORCE>(k, n, gamma, ph, V, pd, slab, dudt, nbr, o0, o1, o2, o3, count);
}

template <bool FORCE>
__global__ void __launch_bounds__(WARP_BLOCK, 4) k_cubic_cells(
    uint32_t n, const float* __restrict__ grid, uint32_t mask, const uint32_t* __restrict__ bstart,
    const uint32_t* __restrict__ bend, const uint32_t* __restrict__ bmix, const uint2* __restrict__ items,
    const uint32_t* __restrict__ nitems_p, uint32_t* __restrict__ ticket, const float4* __restrict__ px,
    const float4* __restrict__ ph, const float4* __restrict__ pv, const uint64_t* __restrict__ cell,
    float4* __restrict__ pd, const uint32_t* __restrict__ V, float gamma, float alpha, float beta,
    float* __restrict__ slab, float* __restrict__ dudt, uint32_t* __restrict__ nbr) {
    const int lane = threadIdx.x & 31;
    const uint32_t nitems = *nitems_p;
    while (true) {
        uint32_t it = 0;
        if (lane == 0) it = atomicAdd(ticket, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= nitems) break;
        const uint2 item = items[it];  // (bucket, first body of the slice)
        const uint32_t b = item.x;
        const uint32_t c1 = min(bend[b], item.y + 32u);
        const uint32_t k = item.y + lane;
        const bool live = k < c1;
        float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
        uint32_t count = 0;
        if (bmix[b]) {
            if (live)
                body_direct<FORCE>(k, mask, grid, bstart, bend, px, ph, pv, cell, pd, alpha, beta, o0, o1, o2, o3,
                                   count);
        } else {
            const float4 a = px[live ? k : item.y];
            const float hi = ph[live ? k : item.y].x;
            float4 di = make_float4(0.f, 0.f, 0.f, 0.f), vi = di;
            if (FORCE) {
                di = pd[live ? k : item.y];
                vi = pv[live ? k : item.y];
            }
            // lanes 0..26: neighbour bucket t's range (empty when it holds
            // another cell) and whether its records need the cell filter
            uint32_t j0 = 0, j1 = 0, check = 0;
            uint64_t want = 0;
            if (lane < 27) {
                const float4 a0 = px[item.y];
                const int3 cc = cell_of(a0.x, a0.y, a0.z, grid[1]);
                const int3 c = make_int3(cc.x + (lane % 3) - 1, cc.y + (lane / 3) % 3 - 1, cc.z + lane / 9 - 1);
                want = pack_cell(c);
                const uint32_t nbk = bucket_of(c, mask);
                j0 = bstart[nbk];
                j1 = bend[nbk];
                if (j1 > j0) {
                    if (bmix[nbk]) check = 1;
                    else if (cell[j0] != want) j1 = j0;
                }
            }
            for (int t = 0; t < 27; t++) {
                const uint32_t s0 = __shfl_sync(0xffffffffu, j0, t);
                const uint32_t s1 = __shfl_sync(0xffffffffu, j1, t);
                if (s0 == s1) continue;
                const uint32_t chk = __shfl_sync(0xffffffffu, check, t);
                const uint64_t wt = __shfl_sync(0xffffffffu, want, t);
#pragma unroll 2
                for (uint32_t j = s0; j < s1; j++) {
                    if (chk && cell[j] != wt) continue;
                    const float4 q = px[j];
                    if (!FORCE) {
                        density_pair(a, hi, q, ph[j].x, o0, count);
                    } else {
                        const float4 vj = pv[j], dj = pd[j];
                        if (j != k) force_pair(a, hi, di, vi, q, vj, dj, alpha, beta, o0, o1, o2, o3);
                    }
                }
            }
        }
        if (live) finish_body<FORCE>(k, n, gamma, ph, V, pd, slab, dudt, nbr, o0, o1, o2, o3, count);
    }
}

// Work items (bucket, first body) for every 32-body slice of every occupied
// bucket, and the buckets that hold more than one cell.
__global__ void k_bucket_items(const uint64_t* __restrict__ keys, uint32_t n, const uint32_t* __restrict__ bstart,
                               const uint32_t* __restrict__ bend, const uint64_t* __restrict__ cell,
                               uint32_t* __restrict__ bmix, uint2* __restrict__ items, uint32_t* __restrict__ nitems) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t b = (uint32_t)keys[k];
    const uint32_t s = bstart[b];
    if (((k - s) & 31u) == 0) items[atomicAdd(nitems, 1u)] = make_uint2(b, k);
    if (k != s && cell[k] != cell[s]) bmix[b] = 1u;
    (void)bend;
}

}  // namespace

uint32_t* sf_sph_neighbour_counts(sfgpu_sim* s);

int sf_sph_cubic_alloc(sfgpu_sim* s) {
    CubicWork* w = new CubicWork();
    s->sph_cubic = w;
    const uint32_t n = std::max<uint32_t>(s->n, 1);
    w->tbits = 1;
    while ((1u << w->tbits) < 2u * n) w->tbits++;
    w->tsize = 1u << w->tbits;
    SF_CUDA(cudaMalloc(&w->keys, sizeof(uint64_t) * n));
    SF_CUDA(cudaMalloc(&w->vals, sizeof(uint32_t) * n));
    if (sf_sort_alloc(w->sort, n) != SFGPU_OK) return SFGPU_FAILURE;
    SF_CUDA(cudaMalloc(&w->bstart, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->bend, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->px, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->pv, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->pd, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->ph, sizeof(float4) * n));
    SF_CUDA(cudaMalloc(&w->bmix, sizeof(uint32_t) * w->tsize));
    SF_CUDA(cudaMalloc(&w->items, sizeof(uint2) * n));
    SF_CUDA(cudaMalloc(&w->counters, sizeof(uint32_t) * 4));
    SF_CUDA(cudaMalloc(&w->cell, sizeof(uint64_t) * n));
    SF_CUDA(cudaMalloc(&w->grid, sizeof(float) * 4 + sizeof(float) * n));
    SF_CUDA(cudaMalloc(&w->done, sizeof(uint32_t) * (1024 + 1)));
    SF_CUDA(cudaMemset(w->done, 0, sizeof(uint32_t) * (1024 + 1)));
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
    cudaFree(w->items);
    cudaFree(w->counters);
    cudaFree(w->cell);
    cudaFree(w->grid);
    cudaFree(w->done);
    delete w;
    s->sph_cubic = nullptr;
}

int sf_sph_cubic(sfgpu_sim* s) {
    CubicWork* w = (CubicWork*)s->sph_cubic;
    const uint32_t n = s->n;
    cudaStream_t st = s->stream;
    const uint32_t hb = std::min<uint32_t>(sf_ceil_div(n, 256), 1024);
    int tk = s->timer.begin(st, "sph_grid");
    k_hmax<<<hb, 256, 0, st>>>(s->slab + (size_t)13 * n, n, w->done, w->grid, w->done + 1);
    SF_CHECK_LAUNCH();
    const uint32_t mask = w->tsize - 1;
    const uint32_t nb = sf_ceil_div(n, 256);
    k_cell_keys<<<nb, 256, 0, st>>>(s->slab, n, w->grid, mask, w->keys, w->vals);
    SF_CHECK_LAUNCH();
    if (sf_sort_pairs(w->keys, w->vals, n, (int)w->tbits, w->sort, st, s->d_status) != SFGPU_OK)
        return SFGPU_FAILURE;
    SF_CUDA(cudaMemsetAsync(w->bstart, 0, sizeof(uint32_t) * w->tsize, st));
    SF_CUDA(cudaMemsetAsync(w->bend, 0, sizeof(uint32_t) * w->tsize, st));
    SF_CUDA(cudaMemsetAsync(w->bmix, 0, sizeof(uint32_t) * w->tsize, st));
    SF_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(uint32_t) * 4, st));
    const float gamma = (float)s->p.sph_gamma, alpha = (float)s->p.sph_alpha, beta = (float)s->p.sph_beta;
    k_cell_gather<<<nb, 256, 0, st>>>(w->keys, w->vals, n, s->slab, s->u, w->grid, w->bstart, w->bend, w->px, w->pv,
                                      w->cell, w->ph, gamma);
    SF_CHECK_LAUNCH();
    k_bucket_items<<<nb, 256, 0, st>>>(w->keys, n, w->bstart, w->bend, w->cell, w->bmix, w->items, w->counters);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    uint32_t* nbr = sf_sph_neighbour_counts(s);
    const uint32_t tb = (uint32_t)sf_num_sms() * 8u;  // persistent warps, up to 8 blocks of 4 per SM
    const bool warp_path = s->p.sph_path == 1;
    const uint32_t bb = sf_ceil_div(n, 128);
    tk = s->timer.begin(st, "sph_density");
    if (warp_path)
        k_cubic_cells<false><<<tb, WARP_BLOCK, 0, st>>>(n, w->grid, mask, w->bstart, w->bend, w->bmix, w->items,
                                                        w->counters, w->counters + 1, w->px, w->ph, w->pv, w->cell,
                                                        w->pd, w->vals, gamma, alpha, beta, s->slab, s->dudt, nbr);
    else
        k_cubic_body<false><<<bb, 128, 0, st>>>(n, w->grid, mask, w->bstart, w->bend, w->px, w->ph, w->pv, w->cell,
                                                w->pd, w->vals, gamma, alpha, beta, s->slab, s->dudt, nbr);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    tk = s->timer.begin(st, "sph_force");
    if (warp_path)
        k_cubic_cells<true><<<tb, WARP_BLOCK, 0, st>>>(n, w->grid, mask, w->bstart, w->bend, w->bmix, w->items,
                                                       w->counters, w->counters + 2, w->px, w->ph, w->pv, w->cell,
                                                       w->pd, w->vals, gamma, alpha, beta, s->slab, s->dudt, nbr);
    else
        k_cubic_body<true><<<bb, 128, 0, st>>>(n, w->grid, mask, w->bstart, w->bend, w->px, w->ph, w->pv, w->cell,
                                               w->pd, w->vals, gamma, alpha, beta, s->slab, s->dudt, nbr);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    return SFGPU_OK;
}
