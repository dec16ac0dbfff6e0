// sort.cu -- stable LSD radix sort of (u64 key, u32 value) pairs.
//
// One global histogram pass computes the digit counts of every pass at once;
// each 7-bit digit pass is then a single kernel: tiles take tickets in launch
// order, rank their keys with per-bit warp ballots, and chain their
// per-digit offsets through a decoupled look-back over the preceding tiles.
// Up to 2^17 pairs only the top digit takes a tile pass; each bucket of it
// is then sorted by one CTA in shared memory (below).  All waits are bounded
// and report SFGPU_STATUS_SPIN instead of hanging.
#include <cooperative_groups.h>

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
constexpr int LOOKBACK = 16;  // predecessor words read per look-back round

// The lanes of the warp holding the same 7-bit digit as this one (only this
// lane when !ok): the intersection of one ballot per digit bit, a fixed
// count of single-cycle votes.
__device__ __forceinline__ uint32_t digit_peers(uint32_t d, bool ok, int lane) {
#ifdef SORT_PEERS_MATCH
    return __match_any_sync(0xffffffffu, ok ? d : (0x10000u + (uint32_t)lane));
#else
    uint32_t m = __ballot_sync(0xffffffffu, ok);
#pragma unroll
    for (int b = 0; b < RADIX_BITS; b++) {
        const uint32_t bit = (d >> b) & 1u;
        const uint32_t bb = __ballot_sync(0xffffffffu, bit != 0u);
        m &= bit ? bb : ~bb;
    }
    return ok ? m : (1u << lane);
#endif
}

// Digit histograms of passes [p0, passes) of the n keys, added into hist
// (cleared by the caller).
__device__ __forceinline__ void hist_digits(const uint64_t* __restrict__ keys, uint32_t n, int p0, int passes,
                                            uint32_t* __restrict__ hist, uint32_t* sh, uint32_t first,
                                            uint32_t stride) {
    for (int i = threadIdx.x; i < passes * RADIX; i += blockDim.x) sh[i] = 0u;
    __syncthreads();
    for (uint32_t i = first; i < n; i += stride) {
        const uint64_t k = keys[i];
        for (int p = p0; p < passes; p++) {
            const uint32_t d = (uint32_t)(k >> (p * RADIX_BITS)) & (RADIX - 1);
            atomicAdd(&sh[p * RADIX + d], 1u);
        }
    }
    __syncthreads();
    for (int i = p0 * RADIX + threadIdx.x; i < passes * RADIX; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

__global__ void __launch_bounds__(256) k_hist(const uint64_t* __restrict__ keys, uint32_t n, int p0, int passes,
                                              uint32_t* __restrict__ hist, const uint32_t* enable) {
    if (enable && *enable == 0u) return;
    __shared__ uint32_t sh[MAX_PASSES * RADIX];
    hist_digits(keys, n, p0, passes, hist, sh, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// One tile of one pass: tile `tile` of (kin, vin) ranked and scattered into
// (kout, vout); `tile` is a ticket taken in launch order, or the block index
// when every tile is resident (cooperative launch).
template <int SORT_ITEMS>
__device__ __forceinline__ void onesweep_tile(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                              uint64_t* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                                              int shift, const uint32_t* __restrict__ hist, uint32_t* status,
                                              uint32_t tile, uint32_t* d_status, uint32_t spin_limit,
                                              uint32_t withheld) {
    __shared__ uint32_t wcnt[SORT_WARPS][RADIX];
    __shared__ uint32_t base[RADIX];
    __shared__ uint32_t toff[RADIX];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;

    for (int i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&wcnt[0][0])[i] = 0u;
    __syncthreads();

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
        const uint32_t peers = digit_peers(d, ok, lane);
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

    // decoupled look-back across tiles, one digit per thread; each round
    // reads the next LOOKBACK predecessors' words at once (independent loads,
    // one memory latency per round instead of one per tile) and sums them
    // nearest first up to the first inclusive prefix or unpublished tile
    if (threadIdx.x < RADIX) {
        const int d = threadIdx.x;
        volatile uint32_t* st = status;
        uint32_t prefix = 0;
        const bool publish = tile != withheld;
        if (tile == 0) {
            if (publish) st[d] = FLAG_INC | tcount[d];
        } else {
            if (publish) st[(size_t)tile * RADIX + d] = FLAG_AGG | tcount[d];
            int64_t look = (int64_t)tile - 1;
            uint32_t spins = 0;
            bool done = false;
            while (!done) {
                uint32_t w[LOOKBACK];
#pragma unroll
                for (int b = 0; b < LOOKBACK; b++)
                    w[b] = (look - b >= 0) ? st[(size_t)(look - b) * RADIX + d] : 0u;
                bool stalled = false;
#pragma unroll
                for (int b = 0; b < LOOKBACK; b++) {
                    if (done || stalled) continue;
                    const uint32_t flag = w[b] & ~VALUE_MASK;
                    if (flag == 0u) {
                        stalled = true;
                        continue;
                    }
                    prefix += w[b] & VALUE_MASK;
                    look--;
                    if (flag == FLAG_INC) done = true;
                }
                if (stalled && ++spins > spin_limit) {
                    // a predecessor never published: give up (the offsets
                    // stay within [0, n) but the order is wrong) and say so
                    atomicOr(d_status, SFGPU_STATUS_SPIN);
                    break;
                }
            }
            __threadfence();
            if (publish) st[(size_t)tile * RADIX + d] = FLAG_INC | ((prefix + tcount[d]) & VALUE_MASK);
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

template <int SORT_ITEMS>
__global__ void __launch_bounds__(SORT_THREADS) k_onesweep(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint32_t n, int shift, const uint32_t* __restrict__ hist,
    uint32_t* status, uint32_t* counter, uint32_t* d_status, const uint32_t* enable, uint32_t spin_limit,
    uint32_t withheld) {
    if (enable && *enable == 0u) return;
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    onesweep_tile<SORT_ITEMS>(kin, vin, kout, vout, n, shift, hist, status, s_tile, d_status, spin_limit, withheld);
}

// Every pass of the tile sort in one cooperative launch (all tiles resident,
// a grid barrier between passes), from (k0, v0) ping-ponging with (k1, v1);
// the result ends in (k1, v1) (copied there when the pass count is even).
// Returns at once (the whole grid, before any barrier) unless *enable.
template <int SORT_ITEMS>
__global__ void __launch_bounds__(SORT_THREADS) k_onesweep_all(uint64_t* k0, uint32_t* v0, uint64_t* k1,
                                                               uint32_t* v1, uint32_t n, int passes,
                                                               uint32_t* hist, uint32_t* status,
                                                               uint32_t* d_status, const uint32_t* enable,
                                                               uint32_t spin_limit) {
    if (*enable == 0u) return;
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    const uint32_t tiles = gridDim.x;
    // the look-back words of every pass start clear (only this launch uses them)
    for (size_t i = (size_t)blockIdx.x * SORT_THREADS + threadIdx.x; i < (size_t)passes * tiles * RADIX;
         i += (size_t)tiles * SORT_THREADS)
        status[i] = 0u;
    // the digit histograms below the top one (the bucket path counted only
    // the top digit; its caller cleared them all)
    {
        __shared__ uint32_t sh[MAX_PASSES * RADIX];
        hist_digits(k0, n, 0, passes - 1, hist, sh, blockIdx.x * SORT_THREADS + threadIdx.x, tiles * SORT_THREADS);
    }
    grid.sync();
    uint64_t *ka = k0, *kb = k1;
    uint32_t *va = v0, *vb = v1;
    for (int p = 0; p < passes; p++) {
        onesweep_tile<SORT_ITEMS>(ka, va, kb, vb, n, p * RADIX_BITS, hist + p * RADIX,
                                  status + (size_t)p * tiles * RADIX, blockIdx.x, d_status, spin_limit,
                                  0xFFFFFFFFu);
        grid.sync();
        uint64_t* tk = ka;
        ka = kb;
        kb = tk;
        uint32_t* tv = va;
        va = vb;
        vb = tv;
    }
    if (ka != k1)
        for (uint32_t i = blockIdx.x * SORT_THREADS + threadIdx.x; i < n; i += tiles * SORT_THREADS) {
            k1[i] = ka[i];
            v1[i] = va[i];
        }
}

// ---- small sorts: one pass on the top digit, then every bucket in one CTA ----
// After a tile pass on the most significant digit, the pairs of bucket b
// (keys whose top digit is b) are contiguous.  One CTA per bucket finishes
// the low digits with stable LSD passes in its own shared memory: per pass,
// warps rank consecutive 32-key rounds (per-bit ballots), counts are
// prefixed over warps and digits, and every pair moves to its place in the
// other buffer; __syncthreads separate the steps, so no pass needs a
// grid-wide wait.  A bucket larger than BK_CAP (strongly clustered keys)
// raises a flag on which every tile pass runs in one cooperative launch.
#ifndef SF_BK_THREADS
// measured: 512 threads sort 2,000-key buckets slightly faster than 256 or
// 1024; whole 65,536-body Barnes-Hut step 0.227 ms at 512, 0.230 at 1024,
// 0.235 at 256
#define SF_BK_THREADS 512
#endif
constexpr int BK_THREADS = SF_BK_THREADS;
constexpr int BK_WARPS = BK_THREADS / 32;
constexpr uint32_t BK_CAP = 8192;        // pairs per bucket, 12 B each, two buffers
constexpr int BK_ITEMS = BK_CAP / BK_THREADS;
static_assert(BK_THREADS >= RADIX && BK_WARPS % 4 == 0 && BK_CAP % BK_THREADS == 0, "bucket sort shape");

struct BucketScratch {
    uint32_t* wcnt;   // [BK_WARPS][RADIX] per-warp counts, then their exclusive prefix
    uint32_t* gsum;   // [BK_THREADS / RADIX][RADIX] warp-group totals
    uint32_t* run;    // [RADIX] start of each digit in the destination
    uint32_t* wtot;   // [4] digit-scan warp totals
};

// One stable pass over [0, size <= BK_CAP) of src into dst (shared memory);
// digit = (key >> shift) & 127.  Warp w ranks positions [w 32 R, (w+1) 32 R)
// in R = ceil(size / 1024) rounds of 32 consecutive keys.
__device__ __forceinline__ void bucket_pass(const uint64_t* src_k, const uint32_t* src_v, uint64_t* dst_k,
                                            uint32_t* dst_v, uint32_t size, int shift, const BucketScratch& sc) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t rounds = (size + BK_THREADS - 1) / BK_THREADS;
    for (int i = threadIdx.x; i < BK_WARPS * RADIX; i += BK_THREADS) sc.wcnt[i] = 0u;
    __syncthreads();
    uint32_t dig[BK_ITEMS], rank[BK_ITEMS];
    uint32_t* wc = sc.wcnt + warp * RADIX;
#pragma unroll
    for (int it = 0; it < BK_ITEMS; it++) {
        dig[it] = 0xFFFFu;
        rank[it] = 0u;
        if ((uint32_t)it < rounds) {
            const uint32_t e = (uint32_t)warp * 32u * rounds + (uint32_t)it * 32u + (uint32_t)lane;
            const bool ok = e < size;
            const uint32_t d = ok ? (uint32_t)(src_k[e] >> shift) & (RADIX - 1) : 0u;
            const uint32_t peers = digit_peers(d, ok, lane);
            uint32_t pre = 0;
            if (ok) pre = wc[d];
            __syncwarp();
            if (ok && (peers & lt) == 0u) wc[d] = pre + __popc(peers);
            __syncwarp();
            if (ok) {
                dig[it] = d;
                rank[it] = pre + __popc(peers & lt);
            }
        }
    }
    __syncthreads();
    // per digit: exclusive prefix over the warps (BK_THREADS / RADIX groups;
    // thread (d, q) owns digit d of group q)
    const int d = threadIdx.x & (RADIX - 1), q = threadIdx.x >> 7;
    constexpr int WPQ = BK_WARPS / (BK_THREADS / RADIX);  // warps per (d, q) thread
    {
        uint32_t r = 0;
#pragma unroll
        for (int j = 0; j < WPQ; j++) {
            const uint32_t c = sc.wcnt[(WPQ * q + j) * RADIX + d];
            sc.wcnt[(WPQ * q + j) * RADIX + d] = r;
            r += c;
        }
        sc.gsum[q * RADIX + d] = r;
    }
    __syncthreads();
    {
        uint32_t add = 0, tot = 0;
#pragma unroll
        for (int j = 0; j < BK_THREADS / RADIX; j++) {
            const uint32_t g = sc.gsum[j * RADIX + d];
            add += j < q ? g : 0u;
            tot += g;
        }
#pragma unroll
        for (int j = 0; j < WPQ; j++) sc.wcnt[(WPQ * q + j) * RADIX + d] += add;
        if (q == 0) {  // digit totals -> exclusive digit starts (warps 0-3, one digit per thread)
            uint32_t x = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            sc.run[d] = x - tot;
            if (lane == 31) sc.wtot[warp] = x;
        }
    }
    __syncthreads();
    if (q == 0 && warp > 0) {
        uint32_t add = 0;
        for (int w = 0; w < warp; w++) add += sc.wtot[w];
        sc.run[d] += add;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < BK_ITEMS; it++) {
        if (dig[it] == 0xFFFFu) continue;
        const uint32_t e = (uint32_t)warp * 32u * rounds + (uint32_t)it * 32u + (uint32_t)lane;
        const uint32_t P = sc.run[dig[it]] + sc.wcnt[warp * RADIX + dig[it]] + rank[it];
        dst_k[P] = src_k[e];
        dst_v[P] = src_v[e];
    }
    __syncthreads();
}

// Sort of m <= RANK_MAX pairs by one warp: a bitonic network over 32 E
// slots (E = 1, 2 or 4 per lane, the unused ones +inf) on composite keys
// (the key bits below the digits the pairs share, shifted left 7, plus the
// pair's position): the composites are unique, so equal keys keep their
// order and the network's instability does not matter.  The pair at rank r
// lands at gk[r], gv[r].  O(m log^2 m) work in registers and shuffles.
constexpr uint32_t RANK_MAX = 128;
template <int E>
__device__ __forceinline__ void warp_bitonic_sort(const uint64_t* sk, const uint32_t* sv, uint32_t m,
                                                  uint64_t lowmask, uint64_t* gk, uint32_t* gv) {
    const uint32_t lane = threadIdx.x & 31;
    uint64_t v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
        const uint32_t e = (uint32_t)q * 32u + lane;
        v[q] = e < m ? (((sk[e] & lowmask) << 7) | e) : ~0ull;
    }
#pragma unroll
    for (int k = 2; k <= 32 * E; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {  // partner in another slot of the same lane
                const int qj = j >> 5;
#pragma unroll
                for (int q = 0; q < E; q++) {
                    if (q & qj) continue;
                    const uint32_t e = (uint32_t)q * 32u + lane;
                    const bool asc = (e & (uint32_t)k) == 0u;
                    const uint64_t x = v[q], y = v[q | qj];
                    const uint64_t lo = x < y ? x : y, hi = x < y ? y : x;
                    v[q] = asc ? lo : hi;
                    v[q | qj] = asc ? hi : lo;
                }
            } else {  // partner in lane ^ j, same slot
#pragma unroll
                for (int q = 0; q < E; q++) {
                    const uint64_t o = __shfl_xor_sync(0xffffffffu, v[q], j);
                    const uint32_t e = (uint32_t)q * 32u + lane;
                    const bool asc = (e & (uint32_t)k) == 0u;
                    const bool lower = (lane & (uint32_t)j) == 0u;
                    const uint64_t lo = v[q] < o ? v[q] : o, hi = v[q] < o ? o : v[q];
                    v[q] = (lower == asc) ? lo : hi;
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < E; q++) {
        const uint32_t e = (uint32_t)q * 32u + lane;
        if (e < m) {
            const uint32_t i = (uint32_t)(v[q] & 127u);
            gk[e] = sk[i];
            gv[e] = sv[i];
        }
    }
}
// The same network on composites the caller built (unique, the position in
// their low 13 bits): the pair at rank r is (ok[i], ov[i]), i the low 13
// bits of the r-th composite, written to gk[r], gv[r].
template <int E>
__device__ __forceinline__ void warp_bitonic_comp(const uint64_t* comp, uint32_t m, const uint64_t* ok,
                                                  const uint32_t* ov, uint64_t* gk, uint32_t* gv) {
    const uint32_t lane = threadIdx.x & 31;
    uint64_t v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
        const uint32_t e = (uint32_t)q * 32u + lane;
        v[q] = e < m ? comp[e] : ~0ull;
    }
#pragma unroll
    for (int k = 2; k <= 32 * E; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int qj = j >> 5;
#pragma unroll
                for (int q = 0; q < E; q++) {
                    if (q & qj) continue;
                    const uint32_t e = (uint32_t)q * 32u + lane;
                    const bool asc = (e & (uint32_t)k) == 0u;
                    const uint64_t x = v[q], y = v[q | qj];
                    const uint64_t lo = x < y ? x : y, hi = x < y ? y : x;
                    v[q] = asc ? lo : hi;
                    v[q | qj] = asc ? hi : lo;
                }
            } else {
#pragma unroll
                for (int q = 0; q < E; q++) {
                    const uint64_t o = __shfl_xor_sync(0xffffffffu, v[q], j);
                    const uint32_t e = (uint32_t)q * 32u + lane;
                    const bool asc = (e & (uint32_t)k) == 0u;
                    const bool lower = (lane & (uint32_t)j) == 0u;
                    const uint64_t lo = v[q] < o ? v[q] : o, hi = v[q] < o ? o : v[q];
                    v[q] = (lower == asc) ? lo : hi;
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < E; q++) {
        const uint32_t e = (uint32_t)q * 32u + lane;
        if (e < m) {
            const uint32_t i = (uint32_t)(v[q] & 8191u);
            gk[e] = ok[i];
            gv[e] = ov[i];
        }
    }
}

__device__ __forceinline__ void warp_small_sort(const uint64_t* sk, const uint32_t* sv, uint32_t m, uint64_t lowmask,
                                                uint64_t* gk, uint32_t* gv) {
    if (m <= 1u) {
        if (m == 1u && (threadIdx.x & 31) == 0) {
            gk[0] = sk[0];
            gv[0] = sv[0];
        }
    } else if (m <= 32u) {
        warp_bitonic_sort<1>(sk, sv, m, lowmask, gk, gv);
    } else if (m <= 64u) {
        warp_bitonic_sort<2>(sk, sv, m, lowmask, gk, gv);
    } else {
        warp_bitonic_sort<4>(sk, sv, m, lowmask, gk, gv);
    }
}

// CTAs per bucket: a bucket of m pairs is shared by min(BK_SPLIT,
// ceil(m / BK_SHARE)) CTAs, each sorting a range of its sub-buckets (the
// biggest bucket of a uniform sphere, 6,606 of 65,536 keys, set the whole
// launch when one CTA sorted it).
constexpr uint32_t BK_SPLIT = 4;
constexpr uint32_t BK_SHARE = 1024;

// Bucket blockIdx.x % RADIX of (Kb, Vb), sorted on its low digits, into (K,
// V), by share blockIdx.x / RADIX of its CTAs.  Up to RANK_MAX pairs, warp 0
// of the first CTA sorts the bucket with one network.  A larger bucket is
// split wide on its next bits (below), so that the biggest bucket costs a
// count, a scatter and many tiny sorts side by side instead of six passes.
// A bucket larger than BK_CAP is left alone and raises *big, which enables
// the full tile passes queued after this kernel.
__global__ void __launch_bounds__(BK_THREADS, 1) k_bucket_sort(const uint64_t* __restrict__ Kb,
                                                               const uint32_t* __restrict__ Vb,
                                                               uint64_t* __restrict__ K, uint32_t* __restrict__ V,
                                                               const uint32_t* __restrict__ hist_top,
                                                               int low_passes, uint32_t* big, const uint32_t* enable) {
    if (enable && *enable == 0u) return;
    extern __shared__ __align__(16) unsigned char bk_smem[];
    __shared__ uint32_t s_wcnt[BK_WARPS * RADIX], s_gsum[(BK_THREADS / RADIX) * RADIX], s_run[RADIX], s_wtot[4];
    uint64_t* k0 = reinterpret_cast<uint64_t*>(bk_smem);
    uint64_t* k1 = k0 + BK_CAP;
    uint32_t* v0 = reinterpret_cast<uint32_t*>(k1 + BK_CAP);
    uint32_t* v1 = v0 + BK_CAP;
    BucketScratch sc;
    sc.wcnt = s_wcnt;
    sc.gsum = s_gsum;
    sc.run = s_run;
    sc.wtot = s_wtot;
    __shared__ uint32_t s_range[2];
    const uint32_t b = blockIdx.x % RADIX, share = blockIdx.x / RADIX;
    if (threadIdx.x < 32) {
        uint32_t start = 0;
        for (uint32_t j = threadIdx.x; j < b; j += 32) start += hist_top[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) start += __shfl_xor_sync(0xffffffffu, start, o);
        if (threadIdx.x == 0) {
            s_range[0] = start;
            s_range[1] = hist_top[b];
        }
    }
    __syncthreads();
    const uint32_t start = s_range[0], size = s_range[1];
    if (size == 0u) return;
    if (size > BK_CAP) {
        if (share == 0u && threadIdx.x == 0) atomicOr(big, 1u);
        return;
    }
    const uint32_t shares = min(BK_SPLIT, (size + BK_SHARE - 1u) / BK_SHARE);
    if (share >= shares) return;
    // the bucket's pairs into shared memory (by the only CTA of a bucket
    // sorted whole), four loads in flight per thread before their stores
    // (they come from L2; one at a time the biggest bucket waits ~13 round
    // trips)
    auto load_bucket = [&]() {
        for (uint32_t e0 = threadIdx.x; e0 < size; e0 += 4u * BK_THREADS) {
            uint64_t kk[4];
            uint32_t vv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t e = e0 + (uint32_t)u * BK_THREADS;
                if (e < size) {
                    kk[u] = Kb[start + e];
                    vv[u] = Vb[start + e];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t e = e0 + (uint32_t)u * BK_THREADS;
                if (e < size) {
                    k0[e] = kk[u];
                    v0[e] = vv[u];
                }
            }
        }
        __syncthreads();
    };
    const int warp = threadIdx.x >> 5;
    if (size <= RANK_MAX) {  // the pairs share the top digit only
        load_bucket();
        if (warp == 0) warp_small_sort(k0, v0, size, (1ull << (low_passes * RADIX_BITS)) - 1ull, K + start, V + start);
        return;
    }
    // A wide split on the D bits below the top digit (D <= 10, sized for
    // ~4 pairs per sub-bucket): counts by shared atomics, offsets by a block
    // scan, and an unstable scatter of composites (the key bits below the
    // top digit, shifted left 13, plus the pair's position in the bucket),
    // which keep the pairs' order recoverable.  Sub-buckets of up to 16
    // pairs are then sorted by one thread each (a rank count over the
    // composites), up to RANK_MAX by one warp's network; a sub-bucket
    // above RANK_MAX (dense clusters), or keys too wide for the composite,
    // send the whole bucket through stable LSD passes instead.
    const int lowbits = low_passes * RADIX_BITS;
    int D = 1;
    while (D < 10 && (4u << D) < size) D++;
    D = min(D, lowbits);
    const uint32_t nsub = 1u << D;
    uint32_t* s_cnt = sc.wcnt;          // [1024]
    uint32_t* s_off = sc.wcnt + 1024;   // [1024]
    for (uint32_t d = threadIdx.x; d < nsub; d += BK_THREADS) s_cnt[d] = 0u;
    // every CTA of the bucket holds all of its pairs (read once from L2)
    load_bucket();
    const int dshift = lowbits - D;
    for (uint32_t e = threadIdx.x; e < size; e += BK_THREADS)
        atomicAdd(&s_cnt[(uint32_t)(k0[e] >> dshift) & (nsub - 1u)], 1u);
    __syncthreads();
    // exclusive scan of the counts (two per thread) and their maximum
    __shared__ uint32_t s_wsum[BK_WARPS], s_wmax[BK_WARPS];
    {
        const int lane = threadIdx.x & 31;
        const uint32_t i0 = 2u * threadIdx.x;
        const uint32_t c0 = i0 < nsub ? s_cnt[i0] : 0u, c1 = i0 + 1u < nsub ? s_cnt[i0 + 1u] : 0u;
        uint32_t x = c0 + c1, mx = max(c0, c1);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        mx = __reduce_max_sync(0xffffffffu, mx);
        if (lane == 31) s_wsum[warp] = x;
        if (lane == 0) s_wmax[warp] = mx;
        __syncthreads();
        uint32_t add = 0, m_all = 0;
        for (int u = 0; u < BK_WARPS; u++) {
            if (u < warp) add += s_wsum[u];
            m_all = max(m_all, s_wmax[u]);
        }
        const uint32_t ex = add + x - (c0 + c1);
        if (i0 < nsub) s_off[i0] = ex;
        if (i0 + 1u < nsub) s_off[i0 + 1u] = ex + c0;
        if (threadIdx.x == 0) s_range[0] = m_all;  // the start is in a register already
    }
    __syncthreads();
    const uint32_t m_max = s_range[0];
    if (m_max <= RANK_MAX && lowbits + 13 <= 64) {
        // this CTA's sub-buckets [d0, d1), which start at `base` in the bucket
        const uint32_t d0 = share * nsub / shares, d1 = (share + 1u) * nsub / shares;
        const uint32_t base = s_off[d0];
        __syncthreads();
        const uint64_t lowmask = (lowbits >= 64) ? ~0ull : ((1ull << lowbits) - 1ull);
        for (uint32_t e = threadIdx.x; e < size; e += BK_THREADS) {  // this CTA's composites
            const uint64_t key = k0[e];
            const uint32_t d = (uint32_t)(key >> dshift) & (nsub - 1u);
            if (d < d0 || d >= d1) continue;
            const uint32_t pos = atomicAdd(&s_off[d], 1u);
            k1[pos - base] = ((key & lowmask) << 13) | e;
        }
        __syncthreads();
        // s_off[d] is now the end of sub-bucket d; the pairs are at their
        // bucket positions in (k0, v0)
        const uint64_t* kb = k0;
        const uint32_t* vb = v0;
        for (uint32_t d = d0 + threadIdx.x; d < d1; d += BK_THREADS) {
            const uint32_t m = s_cnt[d];
            if (m == 0u || m > 16u) continue;
            const uint32_t lo = s_off[d] - m;
            const uint64_t* c = k1 + (lo - base);
            for (uint32_t i = 0; i < m; i++) {
                const uint64_t ci = c[i];
                uint32_t r = 0;
                for (uint32_t j = 0; j < m; j++) r += c[j] < ci ? 1u : 0u;
                const uint32_t src = (uint32_t)(ci & 8191u);
                K[start + lo + r] = kb[src];
                V[start + lo + r] = vb[src];
            }
        }
        for (uint32_t d = d0 + (uint32_t)warp; d < d1; d += BK_WARPS) {
            const uint32_t m = s_cnt[d];
            if (m <= 16u) continue;
            const uint32_t lo = s_off[d] - m;
            const uint64_t* c = k1 + (lo - base);
            if (m <= 32u) warp_bitonic_comp<1>(c, m, kb, vb, K + start + lo, V + start + lo);
            else if (m <= 64u) warp_bitonic_comp<2>(c, m, kb, vb, K + start + lo, V + start + lo);
            else warp_bitonic_comp<4>(c, m, kb, vb, K + start + lo, V + start + lo);
        }
        return;
    }
    // stable LSD passes over every digit below the top one, by the first CTA
    if (share != 0u) return;
    uint64_t *ka = k0, *kb = k1;
    uint32_t *va = v0, *vb = v1;
    for (int p = 0; p < low_passes; p++) {
        bucket_pass(ka, va, kb, vb, size, p * RADIX_BITS, sc);
        uint64_t* tk = ka;
        ka = kb;
        kb = tk;
        uint32_t* tv = va;
        va = vb;
        vb = tv;
    }
    for (uint32_t e = threadIdx.x; e < size; e += BK_THREADS) {
        K[start + e] = ka[e];
        V[start + e] = va[e];
    }
}

size_t bucket_sort_smem() { return (size_t)BK_CAP * 24; }  // + 21 KB of static scratch

// The bucket path's work words cleared in one launch: the histograms of
// every pass, the tile tickets and overflow flag, the top pass's look-back
// words.
__global__ void k_sort_clear(uint32_t* __restrict__ hist, uint32_t nhist, uint32_t* __restrict__ counters,
                             uint32_t ncounters, uint32_t* __restrict__ status, uint32_t nstatus) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nhist + ncounters + nstatus;
         i += gridDim.x * blockDim.x) {
        if (i < nhist) hist[i] = 0u;
        else if (i < nhist + ncounters) counters[i - nhist] = 0u;
        else status[i - nhist - ncounters] = 0u;
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
    SF_CUDA(cudaMalloc(&w.counters, sizeof(uint32_t) * (MAX_PASSES + 1)));  // + the bucket overflow flag
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

SortClear sf_sort_clear_words(SortWork& w, uint32_t n, int bits) {
    SortClear c;
    const int passes = (bits + RADIX_BITS - 1) / RADIX_BITS;
    if (n <= 1 || n > BUCKET_SORT_MAX || n > w.cap || passes < 2 || passes >= MAX_PASSES ||
        (w.flags & SORT_NO_BUCKETS))
        return c;
    c.hist = w.hist;
    c.nhist = (uint32_t)passes * RADIX;
    c.counters = w.counters;
    c.ncounters = MAX_PASSES + 1;
    c.status = w.status;
    c.nstatus = sf_ceil_div(n, SORT_THREADS * 4) * RADIX;
    w.flags |= SORT_PRECLEARED;
    return c;
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
    // small arrays (where the per-pass tile look-back chains cost more than
    // the data movement): one tile pass on the top digit, then one CTA per
    // bucket for the rest; the result is left in (keys, vals)
    if (n <= BUCKET_SORT_MAX && passes >= 2 && passes < MAX_PASSES && !(w.flags & SORT_NO_BUCKETS)) {
        static bool smem_set = false;
        if (!smem_set) {
            SF_CUDA(cudaFuncSetAttribute(k_bucket_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bucket_sort_smem()));
            smem_set = true;
        }
        const int items = 4;
        const uint32_t tiles = sf_ceil_div(n, SORT_THREADS * items);
        uint32_t* big = w.counters + MAX_PASSES;
        // pass slot 0: the top digit; slots 1..passes: the gated fallback,
        // which clears its own
        if (!(w.flags & SORT_PRECLEARED)) {
            const uint32_t words = passes * RADIX + MAX_PASSES + 1 + tiles * RADIX;
            k_sort_clear<<<std::min<uint32_t>(sf_ceil_div(words, 256), 64u), 256, 0, st>>>(
                w.hist, passes * RADIX, w.counters, MAX_PASSES + 1, w.status, tiles * RADIX);
            SF_CHECK_LAUNCH();
        }
        w.flags &= ~SORT_PRECLEARED;
        const uint32_t hb = std::min<uint32_t>(sf_ceil_div(n, 256 * 8), (uint32_t)sf_num_sms() * 4);
        // the top digit's histogram (the fallback counts the others itself)
        k_hist<<<hb, 256, 0, st>>>(keys, n, passes - 1, passes, w.hist, enable);
        SF_CHECK_LAUNCH();
        const int top = passes - 1;
        k_onesweep<4><<<tiles, SORT_THREADS, 0, st>>>(keys, vals, w.keys_b, w.vals_b, n, top * RADIX_BITS,
                                                      w.hist + top * RADIX, w.status, w.counters, d_status, enable,
                                                      w.spin_limit, w.withheld);
        SF_CHECK_LAUNCH();
        k_bucket_sort<<<RADIX * BK_SPLIT, BK_THREADS, bucket_sort_smem(), st>>>(w.keys_b, w.vals_b, keys, vals,
                                                                     w.hist + top * RADIX, top, big, enable);
        SF_CHECK_LAUNCH();
        // fallback (only if a bucket overflowed): every pass from the top
        // pass's output, which holds all pairs, in one cooperative launch
        // (tiles <= 128 blocks, all resident), (keys, vals) as scratch
        {
            uint64_t* k0 = w.keys_b;
            uint32_t* v0 = w.vals_b;
            uint64_t* k1 = keys;
            uint32_t* v1 = vals;
            uint32_t nn = n;
            int np = passes;
            uint32_t* hh = w.hist;
            uint32_t* ss = w.status + (size_t)tiles * RADIX;
            uint32_t* ds = d_status;
            const uint32_t* en = big;
            uint32_t sl = w.spin_limit;
            void* args[] = {&k0, &v0, &k1, &v1, &nn, &np, &hh, &ss, &ds, &en, &sl};
            SF_CUDA(cudaLaunchCooperativeKernel((const void*)k_onesweep_all<4>, dim3(tiles), dim3(SORT_THREADS), args, 0,
                                                st));
            SF_CHECK_LAUNCH();
        }
        return SFGPU_OK;  // the result is back in (keys, vals)
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
    k_hist<<<hb, 256, 0, st>>>(keys, n, 0, passes, w.hist, enable);
    SF_CHECK_LAUNCH();
    uint64_t* ka = keys;
    uint32_t* va = vals;
    uint64_t* kb = w.keys_b;
    uint32_t* vb = w.vals_b;
    for (int p = 0; p < passes; p++) {
        uint32_t* stp = w.status + (size_t)p * tiles * RADIX;
        if (items == 2)
            k_onesweep<2><<<tiles, SORT_THREADS, 0, st>>>(ka, va, kb, vb, n, p * RADIX_BITS, w.hist + p * RADIX, stp,
                                                          w.counters + p, d_status, enable, w.spin_limit,
                                                          p == 0 ? w.withheld : 0xFFFFFFFFu);
        else if (items == 4)
            k_onesweep<4><<<tiles, SORT_THREADS, 0, st>>>(ka, va, kb, vb, n, p * RADIX_BITS, w.hist + p * RADIX, stp,
                                                          w.counters + p, d_status, enable, w.spin_limit,
                                                          p == 0 ? w.withheld : 0xFFFFFFFFu);
        else
            k_onesweep<8><<<tiles, SORT_THREADS, 0, st>>>(ka, va, kb, vb, n, p * RADIX_BITS, w.hist + p * RADIX, stp,
                                                          w.counters + p, d_status, enable, w.spin_limit,
                                                          p == 0 ? w.withheld : 0xFFFFFFFFu);
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

// ---------------------------------------------------------------------------
// Failure detection of the bounded look-back wait, without a GPU fault: one
// 7-bit tile pass over the given keys in which tile `withheld_tile` (0xFFFFFFFF:
// none) never publishes its look-back words, so the tiles after it wait on a
// word that nothing sets until `spin_limit` rounds have passed, then set
// SFGPU_STATUS_SPIN and finish.  With a single pass every scatter offset
// stays inside [0, n) whatever the wait gave (each tile's prefix can only
// fall short), so the call completes and the context stays usable; the
// order is then wrong for the keys after the withheld tile.
// ---------------------------------------------------------------------------
namespace {
int sort_host_keys(const char* who, const uint64_t* keys, uint32_t n, int bits, bool no_buckets,
                   uint32_t withheld_tile, uint32_t spin_limit, uint64_t* sorted, uint32_t* index,
                   uint32_t* status) {
    sf_clear_error();
    if (!keys || !sorted || !index || !status || n == 0) {
        sf_set_error("%s: NULL argument or n = 0", who);
        return SFGPU_FAILURE;
    }
    if (bits < 1 || bits > 64) {
        sf_set_error("%s: %d key bits (1..64)", who, bits);
        return SFGPU_FAILURE;
    }
    uint64_t* dk = nullptr;
    uint32_t* dv = nullptr;
    uint32_t* ds = nullptr;
    cudaStream_t st = nullptr;
    SortWork w;
    int rc = SFGPU_FAILURE;
    std::vector<uint32_t> iota(n);
    for (uint32_t i = 0; i < n; i++) iota[i] = i;
    do {
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) break;
        if (cudaMalloc(&dk, sizeof(uint64_t) * n) != cudaSuccess) break;
        if (cudaMalloc(&dv, sizeof(uint32_t) * n) != cudaSuccess) break;
        if (cudaMalloc(&ds, sizeof(uint32_t)) != cudaSuccess) break;
        if (cudaMemcpy(dk, keys, sizeof(uint64_t) * n, cudaMemcpyHostToDevice) != cudaSuccess) break;
        if (cudaMemcpy(dv, iota.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice) != cudaSuccess) break;
        if (cudaMemset(ds, 0, sizeof(uint32_t)) != cudaSuccess) break;
        if (sf_sort_alloc(w, n) != SFGPU_OK) break;
        if (no_buckets) w.flags |= SORT_NO_BUCKETS;
        if (spin_limit) w.spin_limit = spin_limit;
        w.withheld = withheld_tile;
        if (sf_sort_pairs(dk, dv, n, bits, w, st, ds) != SFGPU_OK) break;
        if (cudaStreamSynchronize(st) != cudaSuccess) break;
        if (cudaMemcpy(sorted, dk, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess) break;
        if (cudaMemcpy(index, dv, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess) break;
        if (cudaMemcpy(status, ds, sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess) break;
        rc = SFGPU_OK;
    } while (0);
    if (rc != SFGPU_OK && !*sfgpu_last_error()) sf_set_error("%s: %s", who, cudaGetErrorString(cudaGetLastError()));
    sf_sort_free(w);
    cudaFree(dk);
    cudaFree(dv);
    cudaFree(ds);
    if (st) cudaStreamDestroy(st);
    return rc;
}
}  // namespace

extern "C" int sfgpu_sort_withheld_check(const uint64_t* keys, uint32_t n, uint32_t withheld_tile,
                                         uint32_t spin_limit, uint64_t* sorted, uint32_t* index,
                                         uint32_t* status) {
    return sort_host_keys("sfgpu_sort_withheld_check", keys, n, RADIX_BITS, true, withheld_tile, spin_limit, sorted,
                          index, status);
}

// The library's stable sort of (key, index) pairs on host keys, through the
// same dispatch the tree build and the SPH cell grids use: up to 2^17 pairs
// one tile pass on the top digit and the per-bucket CTAs (with the
// cooperative tile passes behind them for a bucket over 8192 pairs), above
// that one tile pass per 7-bit digit.
extern "C" int sfgpu_sort_keys(const uint64_t* keys, uint32_t n, int bits, uint64_t* sorted, uint32_t* index,
                               uint32_t* status) {
    return sort_host_keys("sfgpu_sort_keys", keys, n, bits, false, 0xFFFFFFFFu, 0u, sorted, index, status);
}
