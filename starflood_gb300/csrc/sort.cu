// sort.cu -- stable LSD radix sort of (u64 key, u32 value) pairs.
//
// One global histogram pass computes the digit counts of every pass at once;
// each 7-bit digit pass is then a single kernel: tiles take tickets in launch
// order, rank their keys with warp match/ballot, and chain their per-digit
// offsets through a decoupled look-back over the preceding tiles.  All waits
// are bounded and report SFGPU_STATUS_SPIN instead of hanging.
#include "internal.cuh"

namespace {

constexpr int RADIX_BITS = 7;
constexpr int RADIX = 1 << RADIX_BITS;       // 128 buckets
constexpr int SORT_WARPS = 8;
constexpr int SORT_THREADS = SORT_WARPS * 32;
constexpr int SORT_TILE_MIN = SORT_THREADS * 2;              // 512 keys per tile
constexpr int MAX_PASSES = 10;
constexpr uint32_t FLAG_AGG = 1u << 30;
constexpr uint32_t FLAG_INC = 2u << 30;
constexpr uint32_t VALUE_MASK = (1u << 30) - 1u;
constexpr uint32_t SPIN_LIMIT = 1u << 24;

__global__ void __launch_bounds__(256) k_hist(const uint64_t* __restrict__ keys, uint32_t n, int passes,
                                              uint32_t* __restrict__ hist, const uint32_t* enable) {
    if (enable && *enable == 0u) return;
    __shared__ uint32_t sh[MAX_PASSES * RADIX];
    for (int i = threadIdx.x; i < passes * RADIX; i += blockDim.x) sh[i] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        for (int p = 0; p < passes; p++) {
            const uint32_t d = (uint32_t)(k >> (p * RADIX_BITS)) & (RADIX - 1);
            atomicAdd(&sh[p * RADIX + d], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * RADIX; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

template <int SORT_ITEMS>
__global__ void __launch_bounds__(SORT_THREADS) k_onesweep(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint32_t n, int shift, const uint32_t* __restrict__ hist,
    uint32_t* status, uint32_t* counter, uint32_t* d_status, const uint32_t* enable) {
    if (enable && *enable == 0u) return;
    __shared__ uint32_t s_tile;
    __shared__ uint32_t wcnt[SORT_WARPS][RADIX];
    __shared__ uint32_t base[RADIX];
    __shared__ uint32_t toff[RADIX];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
    for (int i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&wcnt[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;

    // exclusive scan of the global digit histogram (warps 0..3, 32 digits each)
    if (threadIdx.x < RADIX) {
        uint32_t v = hist[threadIdx.x];
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        base[threadIdx.x] = x - v;  // exclusive within the warp
    }
    __syncthreads();
    if (threadIdx.x < RADIX) {
        uint32_t add = 0;
        for (int w = 0; w < (threadIdx.x >> 5); w++) {
            const int last = w * 32 + 31;
            add += base[last] + hist[last];
        }
        toff[threadIdx.x] = base[threadIdx.x] + add;
    }
    __syncthreads();
    if (threadIdx.x < RADIX) base[threadIdx.x] = toff[threadIdx.x];
    __syncthreads();

    // load and rank
    uint64_t key[SORT_ITEMS];
    uint32_t val[SORT_ITEMS];
    uint32_t rank[SORT_ITEMS];
    uint32_t dig[SORT_ITEMS];
    const uint32_t lt = (1u << lane) - 1u;
    const size_t wbase = (size_t)tile * (SORT_THREADS * SORT_ITEMS) + (size_t)warp * (32 * SORT_ITEMS);
#pragma unroll
    for (int it = 0; it < SORT_ITEMS; it++) {
        const size_t e = wbase + (size_t)it * 32 + lane;
        const bool ok = e < n;
        key[it] = ok ? kin[e] : 0ull;
        val[it] = ok ? vin[e] : 0u;
        const uint32_t d = (uint32_t)(key[it] >> shift) & (RADIX - 1);
        dig[it] = ok ? d : 0xFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, ok ? d : (0x10000u + lane));
        uint32_t pre = 0;
        if (ok) pre = wcnt[warp][d];
        __syncwarp();
        if (ok && (peers & lt) == 0u) wcnt[warp][d] = pre + __popc(peers);
        __syncwarp();
        rank[it] = pre + __popc(peers & lt);
    }
    __syncthreads();

    // per-digit offsets of each warp inside the tile; tile totals
    __shared__ uint32_t tcount[RADIX];
    if (threadIdx.x < RADIX) {
        uint32_t run = 0;
        for (int w = 0; w < SORT_WARPS; w++) {
            const uint32_t c = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = run;
            run += c;
        }
        tcount[threadIdx.x] = run;
    }
    __syncthreads();

    // decoupled look-back across tiles, one digit per thread
    if (threadIdx.x < RADIX) {
        const int d = threadIdx.x;
        volatile uint32_t* st = status;
        uint32_t prefix = 0;
        if (tile == 0) {
            st[d] = FLAG_INC | tcount[d];
        } else {
            st[(size_t)tile * RADIX + d] = FLAG_AGG | tcount[d];
            int64_t look = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (look >= 0) {
                const uint32_t w = st[(size_t)look * RADIX + d];
                const uint32_t flag = w & ~VALUE_MASK;
                if (flag == 0u) {
                    if (++spins > SPIN_LIMIT) {
                        atomicOr(d_status, SFGPU_STATUS_SPIN);
                        break;
                    }
                    continue;
                }
                prefix += w & VALUE_MASK;
                if (flag == FLAG_INC) break;
                look--;
            }
            __threadfence();
            st[(size_t)tile * RADIX + d] = FLAG_INC | ((prefix + tcount[d]) & VALUE_MASK);
        }
        toff[d] = base[d] + prefix;
    }
    __syncthreads();

#pragma unroll
    for (int it = 0; it < SORT_ITEMS; it++) {
        if (dig[it] == 0xFFFFu) continue;
        const uint32_t d = dig[it];
        const uint32_t pos = toff[d] + wcnt[warp][d] + rank[it];
        kout[pos] = key[it];
        vout[pos] = val[it];
    }
}

__global__ void k_copy_pairs(const uint64_t* __restrict__ ks, const uint32_t* __restrict__ vs,
                             uint64_t* __restrict__ kd, uint32_t* __restrict__ vd, uint32_t n,
                             const uint32_t* enable) {
    if (enable && *enable == 0u) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        kd[i] = ks[i];
        vd[i] = vs[i];
    }
}

}  // namespace

int sf_sort_alloc(SortWork& w, size_t n) {
    sf_sort_free(w);
    const size_t tiles = (n + SORT_TILE_MIN - 1) / SORT_TILE_MIN + 1;
    SF_CUDA(cudaMalloc(&w.keys_b, sizeof(uint64_t) * (n ? n : 1)));
    SF_CUDA(cudaMalloc(&w.vals_b, sizeof(uint32_t) * (n ? n : 1)));
    SF_CUDA(cudaMalloc(&w.hist, sizeof(uint32_t) * MAX_PASSES * RADIX));
    SF_CUDA(cudaMalloc(&w.status, sizeof(uint32_t) * MAX_PASSES * tiles * RADIX));
    SF_CUDA(cudaMalloc(&w.counters, sizeof(uint32_t) * MAX_PASSES));
    w.cap = n;
    w.tiles_cap = tiles;
    return SFGPU_OK;
}

void sf_sort_free(SortWork& w) {
    cudaFree(w.keys_b);
    cudaFree(w.vals_b);
    cudaFree(w.hist);
    cudaFree(w.status);
    cudaFree(w.counters);
    w = SortWork{};
}

int sf_sort_pairs_keep(uint64_t* keys, uint32_t* vals, uint32_t n, int bits, SortWork& w, cudaStream_t st,
                       uint32_t* d_status, uint64_t** out_keys, uint32_t** out_vals, const uint32_t* enable) {
    *out_keys = keys;
    *out_vals = vals;
    if (n > w.cap) {
        sf_set_error("sort: %u keys exceed the work space of %zu", n, w.cap);
        return SFGPU_FAILURE;
    }
    if (n <= 1) return SFGPU_OK;
    const int passes = (bits + RADIX_BITS - 1) / RADIX_BITS;
    if (passes > MAX_PASSES) {
        sf_set_error("sort: %d key bits is too many", bits);
        return SFGPU_FAILURE;
    }
    // keys per thread, measured on GB300 (7 passes of 49-bit keys): 4 up to
    // 2^17 keys (0.087 ms at 65,536, against 0.101 with 2 or 8), 8 above
    // (0.128 ms at 262,144 and 0.253 ms at 1,048,576, against 0.142 / 0.291
    // with 4): fewer, fuller tiles shorten the look-back chains
    const int items = n <= (1u << 17) ? 4 : 8;
    const uint32_t tiles = sf_ceil_div(n, SORT_THREADS * items);
    SF_CUDA(cudaMemsetAsync(w.hist, 0, sizeof(uint32_t) * passes * RADIX, st));
    SF_CUDA(cudaMemsetAsync(w.counters, 0, sizeof(uint32_t) * passes, st));
    SF_CUDA(cudaMemsetAsync(w.status, 0, sizeof(uint32_t) * (size_t)passes * tiles * RADIX, st));
    const uint32_t hb = std::min<uint32_t>(sf_ceil_div(n, 256 * 8), (uint32_t)sf_num_sms() * 4);
    k_hist<<<hb, 256, 0, st>>>(keys, n, passes, w.hist, enable);
    SF_CHECK_LAUNCH();
    uint64_t* ka = keys;
    uint32_t* va = vals;
    uint64_t* kb = w.keys_b;
    uint32_t* vb = w.vals_b;
    for (int p = 0; p < passes; p++) {
        uint32_t* stp = w.status + (size_t)p * tiles * RADIX;
        if (items == 2)
            k_onesweep<2><<<tiles, SORT_THREADS, 0, st>>>(ka, va, kb, vb, n, p * RADIX_BITS, w.hist + p * RADIX, stp,
                                                          w.counters + p, d_status, enable);
        else if (items == 4)
            k_onesweep<4><<<tiles, SORT_THREADS, 0, st>>>(ka, va, kb, vb, n, p * RADIX_BITS, w.hist + p * RADIX, stp,
                                                          w.counters + p, d_status, enable);
        else
            k_onesweep<8><<<tiles, SORT_THREADS, 0, st>>>(ka, va, kb, vb, n, p * RADIX_BITS, w.hist + p * RADIX, stp,
                                                          w.counters + p, d_status, enable);
        SF_CHECK_LAUNCH();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    *out_keys = ka;
    *out_vals = va;
    return SFGPU_OK;
}

int sf_sort_pairs(uint64_t* keys, uint32_t* vals, uint32_t n, int bits, SortWork& w, cudaStream_t st,
                  uint32_t* d_status, const uint32_t*, const uint32_t* enable) {
    uint64_t* ka = keys;
    uint32_t* va = vals;
    if (sf_sort_pairs_keep(keys, vals, n, bits, w, st, d_status, &ka, &va, enable) != SFGPU_OK) return SFGPU_FAILURE;
    if (ka != keys) {
        const uint32_t cb = std::min<uint32_t>(sf_ceil_div(n, 256), (uint32_t)sf_num_sms() * 8);
        k_copy_pairs<<<cb, 256, 0, st>>>(ka, va, keys, vals, n, enable);
        SF_CHECK_LAUNCH();
    }
    return SFGPU_OK;
}
