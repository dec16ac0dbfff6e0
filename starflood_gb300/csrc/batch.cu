// batch.cu -- the batched and adjoint forms (no counterpart in the reference,
// which runs one system per process).
//
// Batched: many independent systems of uneven N share one slab (the
// reference layout over the concatenated bodies) and one persistent PP launch
// per force evaluation: CTAs take (system, i-tile, j-chunk) work items from an
// atomic ticket, write per-chunk partial sums, and a second kernel adds each
// body's partials in chunk order (deterministic).  The leapfrog reuses the
// slab kernels of kdk.cu over all bodies.  sfgpu_batch_run captures K whole
// steps into one CUDA graph.  The tile shape (bodies per thread, j-chunk)
// is picked by sfgpu_batch_autotune, which times the candidates on the batch.
//
// Adjoint: for the KDK map with a = a(x),
//   v' = v + h a(x),  x1 = x + dt v',  v1 = v' + h a(x1)      (h = dt/2)
// the reverse sweep is, step k = K-1 .. 0:
//   vbar += dt xbar;   xbar += J(x_k)^T (c_k vbar),  c_k = 2h (k > 0), h (k = 0)
// (the kick at the end of step k-1 and the kick at the start of step k see
// the same force and the same cotangent, so their two VJPs merge; the final
// kick's VJP vanishes because the loss does not depend on v_K).  The force
// VJP, with a_i = c_i sum_j m_j d_ij phi_ij, d_ij = x_j - x_i,
// phi = (r^2+eps^2)^-1.5, psi = (r^2+eps^2)^-2.5, K_ij = phi I - 3 psi d d^T,
// b_j = c_j abar_j, is
//   xbar_k += sum_j K_kj (m_k b_j - m_j b_k),
// one O(N^2) pass per step.  Positions are checkpointed every `checkpoint`
// steps on the forward sweep and each segment is recomputed before its
// reverse sweep.
#include <algorithm>
#include <vector>

#include "internal.cuh"

struct BatchItem {
    uint32_t sys, i0, j0, chunk;
};

struct sfgpu_batch {
    sfgpu_sim* sim = nullptr;   // PP simulation over all bodies (slab, stream, kdk)
    uint32_t nsys = 0, total = 0;
    std::vector<uint32_t> h_off;
    uint32_t* off = nullptr;       // device offsets (nsys+1)
    uint32_t* sys_of = nullptr;    // system of each body
    uint32_t* part_off = nullptr;  // partial-sum base per system (float4 units)
    uint32_t* nchunk = nullptr;    // j-chunks per system
    BatchItem* items = nullptr;
    uint32_t nitems = 0;
    float4* part = nullptr;
    size_t part_cap = 0;
    uint32_t* ticket = nullptr;
    int config = -1;               // tile shape index
    uint32_t jchunk = 0;
    cudaGraphExec_t graph = nullptr;
    uint32_t graph_steps = 0;
    // adjoint
    float* abar = nullptr;    // 3 * total
    float* xbar = nullptr;    // 3 * total
    float* vbar = nullptr;    // 3 * total
    float* ckpt = nullptr;    // checkpoints of pos, vel
    size_t ckpt_cap = 0;
    float* seg = nullptr;     // positions of one segment
    size_t seg_cap = 0;
    double* d_loss = nullptr;
    uint2* vjp_blk = nullptr;      // (system, first body) per VJP block
    uint32_t vjp_nblk = 0;
    float* fin = nullptr;          // final state kept across the reverse sweep
    double* loss_part = nullptr;
    uint32_t* loss_done = nullptr;
};

namespace {

struct TileConfig {
    int bs, ipt;
    uint32_t jchunk;
};
// candidate shapes for the autotuner (threads per CTA, bodies per thread, j-chunk); the last two are held
// to 64 registers so that 8 CTAs of 128 threads fit on an SM (the persistent grid's CTAs per SM)
const TileConfig kConfigs[] = {{128, 4, 2048}, {128, 8, 2048}, {128, 8, 4096}, {256, 4, 4096}, {128, 8, 8192},
                               {128, 4, 2048}, {128, 4, 4096}};
constexpr int kNumConfigs = sizeof(kConfigs) / sizeof(kConfigs[0]);

template <int BS, int IPT, int MINB = 1>
__global__ void __launch_bounds__(BS, MINB) k_batch_pp(const BatchItem* __restrict__ items, uint32_t nitems,
                                                 uint32_t* ticket, const uint32_t* __restrict__ off,
                                                 const uint32_t* __restrict__ part_off, uint32_t jchunk,
                                                 const float* __restrict__ pos, const float* __restrict__ mas,
                                                 float eps2, float4* __restrict__ part) {
    __shared__ float4 sj[2][BS];
    __shared__ uint32_t s_item;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        __syncthreads();
        if (it >= nitems) break;
        const BatchItem w = items[it];
        const uint32_t base = off[w.sys], nb = off[w.sys + 1] - base;
        // bodies i0 + k*BS + tid, k < IPT, as IPT/2 pairs on the paired FP32
        // instructions (pp_pair_step)
        constexpr int PAIRS = IPT / 2;
        float2 nx[PAIRS], ny[PAIRS], nz[PAIRS], ax[PAIRS], ay[PAIRS], az[PAIRS], ph[PAIRS];
#pragma unroll
        for (int q = 0; q < PAIRS; q++) {
            const uint32_t i0 = w.i0 + (2 * q) * BS + threadIdx.x, i1 = i0 + BS;
            nx[q] = make_float2(i0 < nb ? -pos[3u * (base + i0)] : 0.f, i1 < nb ? -pos[3u * (base + i1)] : 0.f);
            ny[q] = make_float2(i0 < nb ? -pos[3u * (base + i0) + 1u] : 0.f,
                                i1 < nb ? -pos[3u * (base + i1) + 1u] : 0.f);
            nz[q] = make_float2(i0 < nb ? -pos[3u * (base + i0) + 2u] : 0.f,
                                i1 < nb ? -pos[3u * (base + i1) + 2u] : 0.f);
            ax[q] = ay[q] = az[q] = ph[q] = make_float2(0.f, 0.f);
        }
        const float2 e2 = make_float2(eps2, eps2);
        const uint32_t j1 = min(nb, w.j0 + jchunk);
        for (uint32_t jt = w.j0; jt < j1; jt += BS) {
            const uint32_t j = jt + threadIdx.x;
            float x = 0.f, y = 0.f, z = 0.f, m = 0.f;  // padding: zero mass
            if (j < j1) {
                x = pos[3u * (base + j)];
                y = pos[3u * (base + j) + 1u];
                z = pos[3u * (base + j) + 2u];
                m = mas[base + j];
            }
            __syncthreads();
            sj[0][threadIdx.x] = make_float4(x, x, y, y);
            sj[1][threadIdx.x] = make_float4(z, z, m, m);
            __syncthreads();
            // each tile's BS terms in their own sums, added to the running
            // ones once per tile: two-level summation keeps the FP32
            // rounding of a j-chunk near that of one tile
            float2 tx[PAIRS], ty[PAIRS], tz[PAIRS], tp[PAIRS];
#pragma unroll
            for (int q = 0; q < PAIRS; q++) tx[q] = ty[q] = tz[q] = tp[q] = make_float2(0.f, 0.f);
#pragma unroll 4
            for (int jj = 0; jj < BS; jj++) {
                const float4 A = sj[0][jj], B = sj[1][jj];
                const float2 sx = make_float2(A.x, A.y), sy = make_float2(A.z, A.w);
                const float2 sz = make_float2(B.x, B.y), sw = make_float2(B.z, B.w);
#pragma unroll
                for (int q = 0; q < PAIRS; q++)
                    pp_pair_step<2>(sx, sy, sz, sw, nx[q], ny[q], nz[q], e2, tx[q], ty[q], tz[q], tp[q]);
            }
#pragma unroll
            for (int q = 0; q < PAIRS; q++) {
                ax[q] = __fadd2_rn(ax[q], tx[q]);
                ay[q] = __fadd2_rn(ay[q], ty[q]);
                az[q] = __fadd2_rn(az[q], tz[q]);
                ph[q] = __fadd2_rn(ph[q], tp[q]);
            }
        }
        float4* out = part + part_off[w.sys] + (size_t)w.chunk * nb;
#pragma unroll
        for (int q = 0; q < PAIRS; q++) {
            const uint32_t i0 = w.i0 + (2 * q) * BS + threadIdx.x, i1 = i0 + BS;
            if (i0 < nb) out[i0] = make_float4(ax[q].x, ay[q].x, az[q].x, ph[q].x);
            if (i1 < nb) out[i1] = make_float4(ax[q].y, ay[q].y, az[q].y, ph[q].y);
        }
        __syncthreads();
    }
}

__global__ void k_batch_reduce(const float4* __restrict__ part, const uint32_t* __restrict__ off,
                               const uint32_t* __restrict__ sys_of, const uint32_t* __restrict__ part_off,
                               const uint32_t* __restrict__ nchunk, uint32_t total, const float* __restrict__ mas,
                               ForceConsts fc, float* __restrict__ acc, float* __restrict__ pot) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const uint32_t b = sys_of[g];
    const uint32_t base = off[b], nb = off[b + 1] - base, i = g - base;
    const float4* p = part + part_off[b] + i;
    float4 s = p[0];
    for (uint32_t c = 1; c < nchunk[b]; c++) {
        const float4 t = p[(size_t)c * nb];
        s.x += t.x;
        s.y += t.y;
        s.z += t.z;
        s.w += t.w;
    }
    const float gg = -fc.neg_g;
    const float scale = fc.physical ? gg : gg * mas[g];
    acc[3u * g + 0u] = scale * s.x;
    acc[3u * g + 1u] = scale * s.y;
    acc[3u * g + 2u] = scale * s.z;
    pot[g] = fc.neg_g * s.w;
}

// xbar_k += sum_j K_kj (m_k b_j - m_j b_k), b = coef c abar (see file
// comment), with j-tiles of the same system in shared memory, on the paired
// FP32 instructions: each thread owns VJP_IPT
// bodies k (as VJP_IPT/2 pairs, one body per half of a float2), every j of
// a tile is staged duplicated ((x,x,y,y), (z,z,m,m), (bx,bx,by,by),
// (bz,bz,-,-)) so one 128-bit shared load feeds both halves, and every
// arithmetic step of a (k, j) term is one instruction for two bodies.
// Block r covers bodies [i0, i0 + VJP_BS * VJP_IPT) of system blk[r].x.
constexpr int VJP_BS = 128;
constexpr int VJP_IPT = 4;
__global__ void __launch_bounds__(VJP_BS) k_batch_vjp2(const uint2* __restrict__ blk, const uint32_t* __restrict__ off,
                                                       const float* __restrict__ pos, const float* __restrict__ mas,
                                                       const float* __restrict__ abar, float coef, ForceConsts fc,
                                                       float* __restrict__ xbar) {
    __shared__ float4 sj[4][VJP_BS];
    constexpr int PAIRS = VJP_IPT / 2;
    const uint2 w = blk[blockIdx.x];
    const uint32_t base = off[w.x], nb = off[w.x + 1] - base;
    const float cg = -fc.neg_g;
    float2 nx[PAIRS], ny[PAIRS], nz[PAIRS], mk[PAIRS], bkx[PAIRS], bky[PAIRS], bkz[PAIRS], gx[PAIRS], gy[PAIRS],
        gz[PAIRS];
#pragma unroll
    for (int q = 0; q < PAIRS; q++) {
        float v[2][7];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const uint32_t i = w.y + (uint32_t)(2 * q + h) * VJP_BS + threadIdx.x;
            const bool live = i < nb;
            const uint32_t g = base + (live ? i : 0u);
            const float m = live ? mas[g] : 0.f;
            const float ck = coef * (fc.physical ? cg : cg * m);
            v[h][0] = live ? -pos[3u * g] : 0.f;
            v[h][1] = live ? -pos[3u * g + 1u] : 0.f;
            v[h][2] = live ? -pos[3u * g + 2u] : 0.f;
            v[h][3] = m;
            v[h][4] = live ? ck * abar[3u * g] : 0.f;
            v[h][5] = live ? ck * abar[3u * g + 1u] : 0.f;
            v[h][6] = live ? ck * abar[3u * g + 2u] : 0.f;
        }
        nx[q] = make_float2(v[0][0], v[1][0]);
        ny[q] = make_float2(v[0][1], v[1][1]);
        nz[q] = make_float2(v[0][2], v[1][2]);
        mk[q] = make_float2(v[0][3], v[1][3]);
        bkx[q] = make_float2(v[0][4], v[1][4]);
        bky[q] = make_float2(v[0][5], v[1][5]);
        bkz[q] = make_float2(v[0][6], v[1][6]);
        gx[q] = gy[q] = gz[q] = make_float2(0.f, 0.f);
    }
    const float2 e2 = make_float2(fc.eps2, fc.eps2);
    const float2 m3 = make_float2(-3.0f, -3.0f);
    for (uint32_t jt = 0; jt < nb; jt += VJP_BS) {
        const uint32_t j = jt + threadIdx.x;
        float x = 0.f, y = 0.f, z = 0.f, m = 0.f, bx = 0.f, by = 0.f, bz = 0.f;  // padding: zero mass, zero cotangent
        if (j < nb) {
            const uint32_t g = base + j;
            m = mas[g];
            const float cj = coef * (fc.physical ? cg : cg * m);
            x = pos[3u * g];
            y = pos[3u * g + 1u];
            z = pos[3u * g + 2u];
            bx = cj * abar[3u * g];
            by = cj * abar[3u * g + 1u];
            bz = cj * abar[3u * g + 2u];
        }
        __syncthreads();
        sj[0][threadIdx.x] = make_float4(x, x, y, y);
        sj[1][threadIdx.x] = make_float4(z, z, m, m);
        sj[2][threadIdx.x] = make_float4(bx, bx, by, by);
        sj[3][threadIdx.x] = make_float4(bz, bz, 0.f, 0.f);
        __syncthreads();
        const uint32_t cnt = min((uint32_t)VJP_BS, nb - jt);
#pragma unroll 2
        for (uint32_t jj = 0; jj < cnt; jj++) {
            const float4 A = sj[0][jj], B = sj[1][jj], Cb = sj[2][jj], D = sj[3][jj];
            const float2 xj = make_float2(A.x, A.y), yj = make_float2(A.z, A.w);
            const float2 zj = make_float2(B.x, B.y), mj = make_float2(B.z, B.w);
            const float2 bjx = make_float2(Cb.x, Cb.y), bjy = make_float2(Cb.z, Cb.w), bjz = make_float2(D.x, D.y);
#pragma unroll
            for (int q = 0; q < PAIRS; q++) {
                const float2 dx = __fadd2_rn(xj, nx[q]), dy = __fadd2_rn(yj, ny[q]), dz = __fadd2_rn(zj, nz[q]);
                float2 r2 = __ffma2_rn(dz, dz, e2);
                r2 = __ffma2_rn(dy, dy, r2);
                r2 = __ffma2_rn(dx, dx, r2);
                const float2 inv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                const float2 inv2 = __fmul2_rn(inv, inv);
                const float2 phi = __fmul2_rn(inv, inv2);
                // w = m_k b_j - m_j b_k; the gradient term phi w - 3 phi inv^2 d (d . w)
                const float2 wx = __ffma2_rn(mk[q], bjx, __fmul2_rn(mj, make_float2(-bkx[q].x, -bkx[q].y)));
                const float2 wy = __ffma2_rn(mk[q], bjy, __fmul2_rn(mj, make_float2(-bky[q].x, -bky[q].y)));
                const float2 wz = __ffma2_rn(mk[q], bjz, __fmul2_rn(mj, make_float2(-bkz[q].x, -bkz[q].y)));
                float2 dw = __fmul2_rn(dz, wz);
                dw = __ffma2_rn(dy, wy, dw);
                dw = __ffma2_rn(dx, wx, dw);
                const float2 t = __fmul2_rn(__fmul2_rn(m3, __fmul2_rn(phi, inv2)), dw);  // -3 phi inv^2 (d . w)
                gx[q] = __ffma2_rn(t, dx, __ffma2_rn(phi, wx, gx[q]));
                gy[q] = __ffma2_rn(t, dy, __ffma2_rn(phi, wy, gy[q]));
                gz[q] = __ffma2_rn(t, dz, __ffma2_rn(phi, wz, gz[q]));
            }
        }
    }
#pragma unroll
    for (int q = 0; q < PAIRS; q++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const uint32_t i = w.y + (uint32_t)(2 * q + h) * VJP_BS + threadIdx.x;
            if (i < nb) {
                const uint32_t g = base + i;
                xbar[3u * g] += h ? gx[q].y : gx[q].x;
                xbar[3u * g + 1u] += h ? gy[q].y : gy[q].x;
                xbar[3u * g + 2u] += h ? gz[q].y : gz[q].x;
            }
        }
}

__global__ void k_axpy(float* __restrict__ y, const float* __restrict__ x, float a, size_t m) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x)
        y[i] += a * x[i];
}

// dL/dx_K for L = sum_b mean_{i in b} |x_i|^2, and L itself (per-block
// partials, last block adds them in order)
__global__ void k_loss_grad(const uint32_t* __restrict__ off, const uint32_t* __restrict__ sys_of, uint32_t total,
                            const float* __restrict__ pos, float* __restrict__ xbar, float* __restrict__ vbar,
                            double* __restrict__ part, uint32_t* done, double* loss) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (g < total) {
        const uint32_t b = sys_of[g];
        const float inv_n = 1.0f / (float)(off[b + 1] - off[b]);
        const float x = pos[3u * g], y = pos[3u * g + 1u], z = pos[3u * g + 2u];
        xbar[3u * g] = 2.0f * inv_n * x;
        xbar[3u * g + 1u] = 2.0f * inv_n * y;
        xbar[3u * g + 2u] = 2.0f * inv_n * z;
        vbar[3u * g] = vbar[3u * g + 1u] = vbar[3u * g + 2u] = 0.0f;
        l = ((double)x * x + (double)y * y + (double)z * z) * (double)inv_n;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = l;
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
    if (last && threadIdx.x == 0) {
        __threadfence();
        double t = 0.0;
        for (uint32_t b = 0; b < gridDim.x; b++) t += __ldcg(&part[b]);
        *loss = t;
    }
}

size_t batch_part_need(const std::vector<uint32_t>& off, uint32_t jchunk, std::vector<uint32_t>& part_off,
                       std::vector<uint32_t>& nchunk) {
    size_t acc = 0;
    const uint32_t nsys = (uint32_t)off.size() - 1;
    part_off.resize(nsys);
    nchunk.resize(nsys);
    for (uint32_t b = 0; b < nsys; b++) {
        const uint32_t nb = off[b + 1] - off[b];
        nchunk[b] = std::max<uint32_t>(1u, sf_ceil_div(nb, jchunk));
        part_off[b] = (uint32_t)acc;
        acc += (size_t)nchunk[b] * nb;
    }
    return acc;
}

int batch_configure(sfgpu_batch* b, int cfg) {
    const TileConfig& c = kConfigs[cfg];
    std::vector<uint32_t> part_off, nchunk;
    const size_t need = batch_part_need(b->h_off, c.jchunk, part_off, nchunk);
    if (need > b->part_cap) {
        cudaFree(b->part);
        b->part = nullptr;
        SF_CUDA(cudaMalloc(&b->part, sizeof(float4) * std::max<size_t>(need, 1)));
        b->part_cap = need;
    }
    std::vector<BatchItem> items;
    const uint32_t per = (uint32_t)(c.bs * c.ipt);
    // largest systems first, so that the long items start early
    std::vector<uint32_t> order(b->nsys);
    for (uint32_t s = 0; s < b->nsys; s++) order[s] = s;
    std::sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        return (b->h_off[x + 1] - b->h_off[x]) > (b->h_off[y + 1] - b->h_off[y]);
    });
    for (uint32_t s : order) {
        const uint32_t nb = b->h_off[s + 1] - b->h_off[s];
        for (uint32_t ch = 0; ch < nchunk[s]; ch++)
            for (uint32_t i0 = 0; i0 < nb; i0 += per) items.push_back({s, i0, ch * c.jchunk, ch});
    }
    cudaFree(b->items);
    b->items = nullptr;
    SF_CUDA(cudaMalloc(&b->items, sizeof(BatchItem) * std::max<size_t>(items.size(), 1)));
    SF_CUDA(cudaMemcpy(b->items, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice));
    SF_CUDA(cudaMemcpy(b->part_off, part_off.data(), sizeof(uint32_t) * b->nsys, cudaMemcpyHostToDevice));
    SF_CUDA(cudaMemcpy(b->nchunk, nchunk.data(), sizeof(uint32_t) * b->nsys, cudaMemcpyHostToDevice));
    b->nitems = (uint32_t)items.size();
    b->jchunk = c.jchunk;
    b->config = cfg;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return SFGPU_OK;
}

template <int BS, int IPT, int MINB = 1>
void launch_pp(sfgpu_batch* b, cudaStream_t st, const float* pos, const float* mas, float eps2, int grid) {
    k_batch_pp<BS, IPT, MINB><<<grid, BS, 0, st>>>(b->items, b->nitems, b->ticket, b->off, b->part_off, b->jchunk, pos,
                                              mas, eps2, b->part);
}

int batch_forces(sfgpu_batch* b, const float* pos) {
    sfgpu_sim* s = b->sim;
    const ForceConsts fc = sf_force_consts(s->p);
    const float* mas = s->slab + (size_t)9 * b->total;
    SF_CUDA(cudaMemsetAsync(b->ticket, 0, sizeof(uint32_t), s->stream));
    const int grid = sf_num_sms() * 8;  // persistent: a few CTAs per SM
    switch (b->config) {
        case 0: launch_pp<128, 4>(b, s->stream, pos, mas, fc.eps2, grid); break;
        case 1: launch_pp<128, 8>(b, s->stream, pos, mas, fc.eps2, grid); break;
        case 2: launch_pp<128, 8>(b, s->stream, pos, mas, fc.eps2, grid); break;
        case 3: launch_pp<256, 4>(b, s->stream, pos, mas, fc.eps2, grid); break;
        case 5:
        case 6: launch_pp<128, 4, 8>(b, s->stream, pos, mas, fc.eps2, grid); break;
        default: launch_pp<128, 8>(b, s->stream, pos, mas, fc.eps2, grid); break;
    }
    SF_CHECK_LAUNCH();
    k_batch_reduce<<<sf_ceil_div(b->total, 256), 256, 0, s->stream>>>(
        b->part, b->off, b->sys_of, b->part_off, b->nchunk, b->total, mas, fc, s->slab + (size_t)6 * b->total,
        s->slab + (size_t)10 * b->total);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

int batch_step(sfgpu_batch* b) {
    if (sf_stage_kick_drift(b->sim, false) != SFGPU_OK) return SFGPU_FAILURE;
    if (batch_forces(b, b->sim->slab) != SFGPU_OK) return SFGPU_FAILURE;
    return sf_stage_kick_energy(b->sim);
}

}  // namespace

extern "C" int sfgpu_batch_destroy(sfgpu_batch* b) {
    if (!b) return SFGPU_OK;
    if (b->sim) cudaStreamSynchronize(b->sim->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->off);
    cudaFree(b->sys_of);
    cudaFree(b->part_off);
    cudaFree(b->nchunk);
    cudaFree(b->items);
    cudaFree(b->part);
    cudaFree(b->ticket);
    cudaFree(b->abar);
    cudaFree(b->xbar);
    cudaFree(b->vbar);
    cudaFree(b->ckpt);
    cudaFree(b->seg);
    cudaFree(b->d_loss);
    cudaFree(b->vjp_blk);
    cudaFree(b->fin);
    cudaFree(b->loss_part);
    cudaFree(b->loss_done);
    sfgpu_destroy(b->sim);
    delete b;
    return SFGPU_OK;
}

extern "C" int sfgpu_batch_create(sfgpu_batch** out, uint32_t nsys, const uint32_t* offsets, const sfgpu_params* p) {
    sf_clear_error();
    if (!out || !offsets || !p || nsys == 0) {
        sf_set_error("sfgpu_batch_create: bad arguments");
        return SFGPU_FAILURE;
    }
    *out = nullptr;
    if (offsets[0] != 0) {
        sf_set_error("sfgpu_batch_create: offsets[0] must be 0");
        return SFGPU_FAILURE;
    }
    for (uint32_t b = 0; b < nsys; b++)
        if (offsets[b + 1] <= offsets[b]) {
            sf_set_error("sfgpu_batch_create: system %u is empty", b);
            return SFGPU_FAILURE;
        }
    sfgpu_params q = *p;
    q.solver = SFGPU_SOLVER_PP;
    q.sph = SFGPU_SPH_OFF;
    q.form = SFGPU_FORM_PLAIN;
    q.math = SFGPU_MATH_FAST;
    sfgpu_batch* b = new sfgpu_batch();
    b->nsys = nsys;
    b->total = offsets[nsys];
    b->h_off.assign(offsets, offsets + nsys + 1);
    if (sfgpu_create(&b->sim, b->total, &q) != SFGPU_OK) {
        delete b;
        return SFGPU_FAILURE;
    }
    std::vector<uint32_t> sys_of(b->total);
    for (uint32_t s = 0; s < nsys; s++)
        for (uint32_t i = offsets[s]; i < offsets[s + 1]; i++) sys_of[i] = s;
    auto fail = [&]() {
        sfgpu_batch_destroy(b);
        return SFGPU_FAILURE;
    };
#define BTRY(call)                                                              \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) {                                                \
            sf_set_error("sfgpu_batch_create: %s", cudaGetErrorString(e_));     \
            return fail();                                                      \
        }                                                                       \
    } while (0)
    BTRY(cudaMalloc(&b->off, sizeof(uint32_t) * (nsys + 1)));
    BTRY(cudaMalloc(&b->sys_of, sizeof(uint32_t) * b->total));
    BTRY(cudaMalloc(&b->part_off, sizeof(uint32_t) * nsys));
    BTRY(cudaMalloc(&b->nchunk, sizeof(uint32_t) * nsys));
    BTRY(cudaMalloc(&b->ticket, sizeof(uint32_t)));
    BTRY(cudaMalloc(&b->d_loss, sizeof(double) * 2));
    BTRY(cudaMemcpy(b->off, offsets, sizeof(uint32_t) * (nsys + 1), cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(b->sys_of, sys_of.data(), sizeof(uint32_t) * b->total, cudaMemcpyHostToDevice));
    {
        std::vector<uint2> blk;
        for (uint32_t sy = 0; sy < nsys; sy++)
            for (uint32_t i0 = 0; i0 < offsets[sy + 1] - offsets[sy]; i0 += VJP_BS * VJP_IPT)
                blk.push_back(make_uint2(sy, i0));
        b->vjp_nblk = (uint32_t)blk.size();
        BTRY(cudaMalloc(&b->vjp_blk, sizeof(uint2) * blk.size()));
        BTRY(cudaMemcpy(b->vjp_blk, blk.data(), sizeof(uint2) * blk.size(), cudaMemcpyHostToDevice));
    }
#undef BTRY
    if (batch_configure(b, 1) != SFGPU_OK) return fail();
    *out = b;
    return SFGPU_OK;
}

static int copy_vec(sfgpu_batch* b, float* dst_dev, const float* src_host, size_t count) {
    SF_CUDA(cudaMemcpyAsync(dst_dev, src_host, sizeof(float) * count, cudaMemcpyHostToDevice, b->sim->stream));
    return SFGPU_OK;
}

extern "C" int sfgpu_batch_upload(sfgpu_batch* b, const float* pos, const float* vel, const float* mas) {
    sf_clear_error();
    if (!b) return SFGPU_FAILURE;
    const size_t n = b->total;
    float* slab = b->sim->slab;
    if (pos && copy_vec(b, slab, pos, 3 * n) != SFGPU_OK) return SFGPU_FAILURE;
    if (vel && copy_vec(b, slab + 3 * n, vel, 3 * n) != SFGPU_OK) return SFGPU_FAILURE;
    if (mas && copy_vec(b, slab + 9 * n, mas, n) != SFGPU_OK) return SFGPU_FAILURE;
    SF_CUDA(cudaStreamSynchronize(b->sim->stream));
    return SFGPU_OK;
}

extern "C" int sfgpu_batch_download(sfgpu_batch* b, float* pos, float* vel, float* acc, float* pot) {
    sf_clear_error();
    if (!b) return SFGPU_FAILURE;
    const size_t n = b->total;
    const float* slab = b->sim->slab;
    cudaStream_t st = b->sim->stream;
    if (pos) SF_CUDA(cudaMemcpyAsync(pos, slab, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (vel) SF_CUDA(cudaMemcpyAsync(vel, slab + 3 * n, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (acc) SF_CUDA(cudaMemcpyAsync(acc, slab + 6 * n, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (pot) SF_CUDA(cudaMemcpyAsync(pot, slab + 10 * n, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    SF_CUDA(cudaStreamSynchronize(st));
    return SFGPU_OK;
}

extern "C" int sfgpu_batch_solve(sfgpu_batch* b) {
    sf_clear_error();
    if (!b) return SFGPU_FAILURE;
    return batch_forces(b, b->sim->slab);
}

extern "C" int sfgpu_batch_run(sfgpu_batch* b, uint32_t nsteps) {
    sf_clear_error();
    if (!b) return SFGPU_FAILURE;
    if (nsteps == 0) return SFGPU_OK;
    cudaStream_t st = b->sim->stream;
    if (!b->graph || b->graph_steps != nsteps) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g = nullptr;
        SF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int rc = SFGPU_OK;
        for (uint32_t k = 0; k < nsteps && rc == SFGPU_OK; k++) rc = batch_step(b);
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc != SFGPU_OK || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (ce != cudaSuccess) sf_set_error("sfgpu_batch_run: capture: %s", cudaGetErrorString(ce));
            return SFGPU_FAILURE;
        }
        const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            b->graph = nullptr;
            sf_set_error("sfgpu_batch_run: instantiate: %s", cudaGetErrorString(ie));
            return SFGPU_FAILURE;
        }
        b->graph_steps = nsteps;
    }
    SF_CUDA(cudaGraphLaunch(b->graph, st));
    return SFGPU_OK;
}

extern "C" int sfgpu_batch_autotune(sfgpu_batch* b, int* chosen) {
    sf_clear_error();
    if (!b) return SFGPU_FAILURE;
    cudaStream_t st = b->sim->stream;
    cudaEvent_t e0, e1;
    SF_CUDA(cudaEventCreate(&e0));
    SF_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_cfg = b->config;
    for (int c = 0; c < kNumConfigs; c++) {
        if (batch_configure(b, c) != SFGPU_OK) return SFGPU_FAILURE;
        if (batch_forces(b, b->sim->slab) != SFGPU_OK) return SFGPU_FAILURE;  // warm-up
        SF_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < 3; r++)
            if (batch_forces(b, b->sim->slab) != SFGPU_OK) return SFGPU_FAILURE;
        SF_CUDA(cudaEventRecord(e1, st));
        SF_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        SF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            best_cfg = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (batch_configure(b, best_cfg) != SFGPU_OK) return SFGPU_FAILURE;
    if (chosen) *chosen = best_cfg;
    return SFGPU_OK;
}

extern "C" int sfgpu_batch_synchronize(sfgpu_batch* b) {
    sf_clear_error();
    if (!b) return SFGPU_FAILURE;
    SF_CUDA(cudaStreamSynchronize(b->sim->stream));
    return SFGPU_OK;
}

extern "C" void* sfgpu_batch_stream(sfgpu_batch* b) { return b ? (void*)b->sim->stream : nullptr; }

static int ensure(float** p, size_t* cap, size_t need) {
    if (*cap >= need) return SFGPU_OK;
    cudaFree(*p);
    *p = nullptr;
    SF_CUDA(cudaMalloc(p, sizeof(float) * need));
    *cap = need;
    return SFGPU_OK;
}

static int vjp(sfgpu_batch* b, const float* pos, const float* abar, float coef, float* xbar) {
    const ForceConsts fc = sf_force_consts(b->sim->p);
    k_batch_vjp2<<<b->vjp_nblk, VJP_BS, 0, b->sim->stream>>>(b->vjp_blk, b->off, pos,
                                                              b->sim->slab + (size_t)9 * b->total, abar, coef, fc, xbar);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

extern "C" int sfgpu_batch_force_vjp(sfgpu_batch* b, const float* d_abar, float* d_xbar) {
    sf_clear_error();
    if (!b) return SFGPU_FAILURE;
    return vjp(b, b->sim->slab, d_abar, 1.0f, d_xbar);
}

extern "C" int sfgpu_batch_grad(sfgpu_batch* b, uint32_t nsteps, uint32_t checkpoint, float* grad_pos,
                                float* grad_vel, double* loss) {
    sf_clear_error();
    if (!b || checkpoint == 0) {
        sf_set_error("sfgpu_batch_grad: bad arguments");
        return SFGPU_FAILURE;
    }
    sfgpu_sim* s = b->sim;
    cudaStream_t st = s->stream;
    const size_t n3 = 3 * (size_t)b->total;
    const uint32_t nseg = sf_ceil_div(std::max<uint32_t>(nsteps, 1), checkpoint);
    if (ensure(&b->ckpt, &b->ckpt_cap, (size_t)nseg * 2 * n3) != SFGPU_OK) return SFGPU_FAILURE;
    if (ensure(&b->seg, &b->seg_cap, (size_t)checkpoint * n3) != SFGPU_OK) return SFGPU_FAILURE;
    if (!b->abar) {
        SF_CUDA(cudaMalloc(&b->abar, sizeof(float) * n3));
        SF_CUDA(cudaMalloc(&b->xbar, sizeof(float) * n3));
        SF_CUDA(cudaMalloc(&b->vbar, sizeof(float) * n3));
        SF_CUDA(cudaMalloc(&b->fin, sizeof(float) * 2 * n3));
        SF_CUDA(cudaMalloc(&b->loss_part, sizeof(double) * (sf_ceil_div(b->total, 256) + 1)));
        SF_CUDA(cudaMalloc(&b->loss_done, sizeof(uint32_t)));
        SF_CUDA(cudaMemset(b->loss_done, 0, sizeof(uint32_t)));
    }
    float* pos = s->slab;
    const float dt = (float)s->p.dt;
    // forward sweep with checkpoints of (pos, vel) every `checkpoint` steps
    if (batch_forces(b, pos) != SFGPU_OK) return SFGPU_FAILURE;
    for (uint32_t k = 0; k < nsteps; k++) {
        if (k % checkpoint == 0)
            SF_CUDA(cudaMemcpyAsync(b->ckpt + (size_t)(k / checkpoint) * 2 * n3, pos, sizeof(float) * 2 * n3,
                                    cudaMemcpyDeviceToDevice, st));
        if (batch_step(b) != SFGPU_OK) return SFGPU_FAILURE;
    }
    SF_CUDA(cudaMemcpyAsync(b->fin, pos, sizeof(float) * 2 * n3, cudaMemcpyDeviceToDevice, st));
    // loss and its gradient at the final positions
    k_loss_grad<<<sf_ceil_div(b->total, 256), 256, 0, st>>>(b->off, b->sys_of, b->total, pos, b->xbar, b->vbar,
                                                            b->loss_part, b->loss_done, b->d_loss);
    SF_CHECK_LAUNCH();
    // reverse sweep, one checkpointed segment at a time
    for (int sg = (int)nseg - 1; sg >= 0; sg--) {
        const uint32_t k0 = (uint32_t)sg * checkpoint;
        const uint32_t k1 = std::min(nsteps, k0 + checkpoint);
        SF_CUDA(cudaMemcpyAsync(pos, b->ckpt + (size_t)sg * 2 * n3, sizeof(float) * 2 * n3, cudaMemcpyDeviceToDevice,
                                st));
        if (batch_forces(b, pos) != SFGPU_OK) return SFGPU_FAILURE;
        for (uint32_t k = k0; k < k1; k++) {  // recompute, keeping x_k
            SF_CUDA(cudaMemcpyAsync(b->seg + (size_t)(k - k0) * n3, pos, sizeof(float) * n3, cudaMemcpyDeviceToDevice,
                                    st));
            if (k + 1 < k1 && batch_step(b) != SFGPU_OK) return SFGPU_FAILURE;
        }
        for (int k = (int)k1 - 1; k >= (int)k0; k--) {
            k_axpy<<<std::min<uint32_t>(sf_ceil_div(n3, 256), 2048), 256, 0, st>>>(b->vbar, b->xbar, dt, n3);
            SF_CHECK_LAUNCH();
            const float coef = k > 0 ? dt : 0.5f * dt;
            if (vjp(b, b->seg + (size_t)(k - (int)k0) * n3, b->vbar, coef, b->xbar) != SFGPU_OK)
                return SFGPU_FAILURE;
        }
    }
    // leave the batch at the final state
    SF_CUDA(cudaMemcpyAsync(pos, b->fin, sizeof(float) * 2 * n3, cudaMemcpyDeviceToDevice, st));
    if (batch_forces(b, pos) != SFGPU_OK) return SFGPU_FAILURE;
    if (grad_pos) SF_CUDA(cudaMemcpyAsync(grad_pos, b->xbar, sizeof(float) * n3, cudaMemcpyDeviceToHost, st));
    if (grad_vel) SF_CUDA(cudaMemcpyAsync(grad_vel, b->vbar, sizeof(float) * n3, cudaMemcpyDeviceToHost, st));
    if (loss) SF_CUDA(cudaMemcpyAsync(loss, b->d_loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    SF_CUDA(cudaStreamSynchronize(st));
    return SFGPU_OK;
}
