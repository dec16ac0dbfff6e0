// tree.cu -- the octree of tree_build (src/tree.c:74-318), built in parallel
// with the reference's exact topology.
//
// The reference inserts bodies one at a time; a node splits when its
// (leaf_cap+1)-th body arrives, the resident bodies move down by "mid < x"
// (tree.c:244-247) and every later arrival by "mid <= x" (tree.c:282-285),
// with mid = 0.5f*(min+max) recomputed per level in FP32.  Hence:
//
//  * the node set is {root} plus the 8 children of every cell holding more
//    than leaf_cap bodies at depth < depth_max;
//  * a body's path is the sequence of octants of its FP32 midpoint
//    comparisons, which differs between the two rules only when a coordinate
//    equals a midpoint exactly, and then only for the first leaf_cap bodies
//    (in index order) of a node that splits.
//
// So: (1) every body gets a provisional 48-bit key (3 bits per level, level 0
// most significant) with the "<=" rule, plus a mask of the levels where it sat
// exactly on a midplane; (2) keys are radix sorted (stable, so ties keep index
// order); (3) one block re-derives the digits of the few midplane bodies with
// the rank rule, and the bodies whose digits changed are merged back into
// the sorted order at their new keys; (4) split nodes
// are read off the sorted keys: position k starts a split node at level L iff
// k begins a level-L run (key[k-1] differs in the first L digits) and
// key[k+leaf_cap] shares those L digits; an exclusive scan of the per-position
// counts numbers the split nodes in depth-first (pre)order, and a split node s
// owns nodes 1+8s .. 8+8s for its octants; (5) monopoles come from exact
// fixed-point prefix sums of (m x, m y, m z, m) over the sorted bodies.
//
// Work per body: key pass reads 12 B and writes 12 B; each sort pass moves
// 12 B each way (one tile pass plus a shared-memory bucket sort up to 2^17
// bodies, seven tile passes above); the gather reads 16 B (random) and
// writes 16 B + 32 B of fixed-point sums.
#include <algorithm>

#include "internal.cuh"
#include "tree.cuh"

namespace {

constexpr uint64_t KEY_OUT = 1ull << 48;  // bodies outside the root cube sort last
constexpr int KEY_BITS = 49;
constexpr uint32_t TIE_CAP = 1024;

__device__ __forceinline__ int cpl_levels(uint64_t a, uint64_t b) {
    const uint64_t x = a ^ b;
    if (x == 0) return 16;
    return (__clzll((long long)x) - 16) / 3;
}

struct Cube {
    float lo[3], hi[3];
};

__device__ __forceinline__ float midf(float lo, float hi) { return fmul(0.5f, fadd(lo, hi)); }

// Descend `levels` levels of `key` (digits of levels 0..levels-1) from the
// root cube, reproducing the bounds of the reference's nodes (tree.c:159-163,
// 263-270, 331-335).
__device__ Cube cube_of(const float* __restrict__ root, uint64_t key, int levels) {
    Cube c;
    for (int a = 0; a < 3; a++) {
        c.lo[a] = root[a];
        c.hi[a] = root[3 + a];
    }
    for (int L = 0; L < levels; L++) {
        const uint32_t o = (uint32_t)(key >> (3 * (15 - L))) & 7u;
        for (int a = 0; a < 3; a++) {
            const float m = midf(c.lo[a], c.hi[a]);
            if ((o >> a) & 1u) c.lo[a] = m; else c.hi[a] = m;
        }
    }
    return c;
}

// Digits of levels [from, 16) with the "<=" rule, starting in cube c; tie bits.
__device__ uint64_t descend(const float x[3], Cube c, uint64_t key, int from, uint32_t& ties) {
    for (int L = from; L < 16; L++) {
        uint32_t o = 0;
        bool tie = false;
        for (int a = 0; a < 3; a++) {
            const float m = midf(c.lo[a], c.hi[a]);
            const bool up = m <= x[a];
            tie |= (m == x[a]);
            o |= (up ? 1u : 0u) << a;
            if (up) c.lo[a] = m; else c.hi[a] = m;
        }
        key |= (uint64_t)o << (3 * (15 - L));
        if (tie) ties |= 1u << L;
    }
    return key;
}

// Besides the keys: clears the sort's work words (SortClear), which saves
// the sort a launch.
__global__ void k_keys(const float* __restrict__ pos, const float* __restrict__ mas, uint32_t n,
                       const float* __restrict__ bounds, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                       uint32_t* __restrict__ nin, uint2* __restrict__ ties, uint32_t* __restrict__ tie_count,
                       uint32_t* __restrict__ mmax, uint32_t* __restrict__ nan_in, uint32_t* d_status,
                       SortClear sc) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t j = i; j < sc.nhist + sc.ncounters + sc.nstatus; j += gridDim.x * blockDim.x) {
        if (j < sc.nhist) sc.hist[j] = 0u;
        else if (j < sc.nhist + sc.ncounters) sc.counters[j - sc.nhist] = 0u;
        else sc.status[j - sc.nhist - sc.ncounters] = 0u;
    }
    bool inside = false;
    // largest |mass| (its bits: non-negative floats order as integers), the
    // scale of the monopoles' fixed-point sums
    uint32_t mb = i < n ? (__float_as_uint(mas[i]) & 0x7FFFFFFFu) : 0u;
    mb = __reduce_max_sync(0xffffffffu, mb);
    if ((threadIdx.x & 31) == 0 && mb) atomicMax(mmax, mb);
    if (i < n) {
        const float x[3] = {pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u]};
        Cube c;
        for (int a = 0; a < 3; a++) {
            c.lo[a] = bounds[a];
            c.hi[a] = bounds[3 + a];
        }
        // tree.c:141-146: skipped only when a comparison with the closed
        // root cube says outside, so a NaN coordinate is inserted: every
        // midpoint comparison is false and it takes octant 0 at every level
        // (key 0, the first sorted slot)
        inside = !(c.lo[0] > x[0] || x[0] > c.hi[0] || c.lo[1] > x[1] || x[1] > c.hi[1] || c.lo[2] > x[2] ||
                   x[2] > c.hi[2]);
        uint64_t key = KEY_OUT;
        if (inside) {
            if (isnan(x[0]) || isnan(x[1]) || isnan(x[2])) atomicOr(nan_in, 1u);
            uint32_t tb = 0;
            key = descend(x, c, 0ull, 0, tb);
            if (tb) {
                const uint32_t slot = atomicAdd(tie_count, 1u);
                if (slot < TIE_CAP) ties[slot] = make_uint2(i, tb);
                else atomicOr(d_status, SFGPU_STATUS_TIES);
            }
        }
        keys[i] = key;
        vals[i] = i;
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, inside);
    if ((threadIdx.x & 31) == 0 && bal) atomicAdd(nin, (uint32_t)__popc(bal));
}

// first index in [lo, hi) whose key >> shift is >= target
__device__ __forceinline__ uint32_t lower_bound_shift(const uint64_t* __restrict__ K, uint32_t lo, uint32_t hi,
                                                      int shift, uint64_t target) {
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((K[mid] >> shift) < target) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint64_t prefix_of(uint64_t key, int L) { return L == 0 ? 0ull : key >> (3 * (16 - L)); }

// Sorted-key search through a table of every stride-th key in shared memory:
// the table narrows the answer to one stride (no global loads), a binary
// search of that stride finishes it (log2(stride) dependent loads instead of
// log2(nin)).
constexpr uint32_t NSAMP = 1024;

struct KeySamples {
    uint32_t stride, count, nin;
};

__device__ __forceinline__ KeySamples load_key_samples(const uint64_t* __restrict__ K, uint32_t nin,
                                                       uint64_t* samp) {
    KeySamples ks;
    ks.nin = nin;
    ks.stride = max(1u, (nin + NSAMP - 1) / NSAMP);
    ks.count = (nin + ks.stride - 1) / ks.stride;
    for (uint32_t j = threadIdx.x; j < ks.count; j += blockDim.x) samp[j] = K[(size_t)j * ks.stride];
    return ks;
}

// first index in [0, nin) whose key >> shift is >= target
__device__ __forceinline__ uint32_t search_keys(const uint64_t* __restrict__ K, const uint64_t* samp,
                                                const KeySamples& ks, int shift, uint64_t target) {
    uint32_t lo = 0, hi = ks.count;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((samp[mid] >> shift) < target) lo = mid + 1; else hi = mid;
    }
    if (lo == 0) return 0u;
    const uint32_t a = (lo - 1) * ks.stride + 1;
    const uint32_t b = (lo == ks.count) ? ks.nin : lo * ks.stride;
    return lower_bound_shift(K, a, b, shift, target);
}

// First index in [from, end) whose key >> shift is >= target, where
// K[from] >> shift < target: probes from+1, from+3, from+7, ... then bisects
// the last gap, O(log d) loads for an answer d slots away.
__device__ __forceinline__ uint32_t gallop_up(const uint64_t* __restrict__ K, uint32_t from, uint32_t end, int shift,
                                              uint64_t target) {
    uint32_t prev = from, step = 1;
    while (true) {
        const uint32_t probe = prev + step;
        if (probe >= end || probe < prev) return lower_bound_shift(K, prev + 1, end, shift, target);
        if ((K[probe] >> shift) >= target) return lower_bound_shift(K, prev + 1, probe, shift, target);
        prev = probe;
        step <<= 1;
    }
}
// First index in [0, from] whose key >> shift is >= target, where
// K[from] >> shift >= target: probes from-1, from-2, from-4, ... backwards.
__device__ __forceinline__ uint32_t gallop_down(const uint64_t* __restrict__ K, uint32_t from, int shift,
                                                uint64_t target) {
    uint32_t cur = from, step = 1;
    while (true) {
        if (cur < step) return lower_bound_shift(K, 0, cur, shift, target);
        const uint32_t probe = cur - step;
        if ((K[probe] >> shift) < target) return lower_bound_shift(K, probe + 1, cur, shift, target);
        cur = probe;
        step <<= 1;
    }
}

// The run of keys with K[i] >> shift == pre around `home` (whose key has that
// prefix): the TIE_WIN neighbours on each side are loaded at once (one memory
// latency; deep cells rarely hold more), and only a run reaching past them
// is galloped further.
constexpr int TIE_WIN = 8;
__device__ __forceinline__ void run_near(const uint64_t* __restrict__ K, uint32_t home, uint32_t end, int shift,
                                         uint64_t pre, uint32_t& lo, uint32_t& hi) {
    uint32_t eqa = 0u, eqb = 0u;
#pragma unroll
    for (int j = 0; j < TIE_WIN; j++) {
        const bool ina = home >= (uint32_t)(j + 1);
        const bool inb = home + 1u + (uint32_t)j < end;
        const uint64_t ka = ina ? K[home - 1u - (uint32_t)j] : 0ull;
        const uint64_t kb = inb ? K[home + 1u + (uint32_t)j] : 0ull;
        eqa |= (uint32_t)(ina && (ka >> shift) == pre) << j;
        eqb |= (uint32_t)(inb && (kb >> shift) == pre) << j;
    }
    // sorted keys: the equal neighbours on each side are a prefix of the bits
    const int dl = __ffs(~eqa) - 1, du = __ffs(~eqb) - 1;
    lo = dl < TIE_WIN ? home - (uint32_t)dl : gallop_down(K, home - TIE_WIN, shift, pre);
    hi = du < TIE_WIN ? home + 1u + (uint32_t)du : gallop_up(K, home + TIE_WIN, end, shift, pre + 1);
}

// Exact digits for bodies lying on a midplane (one block; see file comment).
// Reads the sorted provisional keys (Ks, Vs); the bodies whose digits change
// are listed for k_tie_merge: their old slots ascending (gpos), their new
// (key, body) ascending (gkey, gbody), their number in *moved_out.
constexpr int FIX_THREADS = 1024;

__global__ void __launch_bounds__(FIX_THREADS) k_tie_fix(const float* __restrict__ pos, const float* __restrict__ bounds,
                                                         const uint64_t* __restrict__ K, const uint32_t* __restrict__ V,
                                                         const uint32_t* __restrict__ nin_p, const uint2* __restrict__ ties,
                                                         const uint32_t* __restrict__ tie_count, uint32_t leaf_cap,
                                                         uint32_t depth_max, uint32_t* __restrict__ moved_out,
                                                         uint32_t* __restrict__ gpos, uint64_t* __restrict__ gkey,
                                                         uint32_t* __restrict__ gbody, uint32_t n,
                                                         uint64_t* __restrict__ copyK, uint32_t* __restrict__ copyV) {
    __shared__ uint64_t prov[TIE_CAP];
    __shared__ uint64_t cur[TIE_CAP];
    __shared__ uint32_t body[TIE_CAP];
    __shared__ uint32_t mask[TIE_CAP];
    __shared__ uint64_t samp[NSAMP];
    __shared__ uint32_t home[TIE_CAP];  // a sorted slot holding the body's provisional key
    const uint32_t T = min(*tie_count, TIE_CAP);
    if (T == 0) {
        if (threadIdx.x == 0) *moved_out = 0u;
        return;
    }
    const uint32_t nin = *nin_p;
    const KeySamples ks = load_key_samples(K, nin, samp);
    for (uint32_t t = threadIdx.x; t < T; t += FIX_THREADS) {
        const uint2 e = ties[t];
        body[t] = e.x;
        mask[t] = e.y;
        const float x[3] = {pos[3u * e.x], pos[3u * e.x + 1u], pos[3u * e.x + 2u]};
        Cube c = cube_of(bounds, 0ull, 0);
        uint32_t tb = 0;
        prov[t] = descend(x, c, 0ull, 0, tb);
        cur[t] = prov[t];
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < T; t += FIX_THREADS) home[t] = search_keys(K, samp, ks, 0, prov[t]);
    __syncthreads();

    // Speculation: while no body moves, every cell count is the provisional
    // one, so each body settles its own tie levels in order without waiting
    // for the others (the usual case: deep ties inside leaves).  A body that
    // would move ends the speculation; the level-by-level pass below then
    // decides everything from scratch.
    __shared__ int s_move;
    if (threadIdx.x == 0) s_move = 0;
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < T; t += FIX_THREADS) {
        const uint32_t mk = mask[t];
        const uint32_t p = body[t];
        for (int L = 0; L < (int)depth_max && L < 16; L++) {
            if (!((mk >> L) & 1u)) continue;
            uint32_t lo = 0u, hi = nin;
            if (L > 0) run_near(K, home[t], nin, 3 * (16 - L), prefix_of(prov[t], L), lo, hi);
            if (hi - lo <= leaf_cap) break;  // a leaf: deeper digits unused
            uint32_t seen = 0;
            for (uint32_t k = lo; k < hi && seen < leaf_cap; k += 4) {
                uint32_t v4[4];
#pragma unroll
                for (int j = 0; j < 4; j++) v4[j] = (k + (uint32_t)j < hi) ? V[k + (uint32_t)j] : 0xFFFFFFFFu;
#pragma unroll
                for (int j = 0; j < 4; j++) seen += (v4[j] < p) ? 1u : 0u;
            }
            const bool strict = seen < leaf_cap;
            const float x[3] = {pos[3u * p], pos[3u * p + 1u], pos[3u * p + 2u]};
            const Cube c = cube_of(bounds, prov[t], L);
            uint32_t o = 0;
            for (int a = 0; a < 3; a++) {
                const float m = midf(c.lo[a], c.hi[a]);
                o |= ((strict ? (m < x[a]) : (m <= x[a])) ? 1u : 0u) << a;
            }
            if (o != ((uint32_t)(prov[t] >> (3 * (15 - L))) & 7u)) {
                s_move = 1;
                break;
            }
        }
    }
    __syncthreads();
    if (!s_move) {
        if (threadIdx.x == 0) *moved_out = 0u;
        return;
    }

    // Levels in order; within a level every midplane body is settled by its
    // own thread: membership of a level-L cell can only have been changed by
    // moves at shallower levels, collected in `moved`.
    __shared__ uint32_t moved[TIE_CAP];
    __shared__ uint32_t n_moved, n_moved_next;
    if (threadIdx.x == 0) n_moved = n_moved_next = 0u;
    __syncthreads();
    for (int L = 0; L < (int)depth_max && L < 16; L++) {
        for (uint32_t t = threadIdx.x; t < T; t += FIX_THREADS) {
            if (!((mask[t] >> L) & 1u)) continue;
            const uint64_t pre = prefix_of(cur[t], L);
            const int shift = 3 * (16 - L);
            // the level-L cell's slots: galloped from the body's own slot while
            // it has not moved (deep cells are short runs), else searched
            uint32_t lo = 0u, hi = nin;
            if (L > 0) {
                if (prefix_of(prov[t], L) == pre) {
                    run_near(K, home[t], nin, shift, pre, lo, hi);
                } else {
                    lo = search_keys(K, samp, ks, shift, pre);
                    hi = search_keys(K, samp, ks, shift, pre + 1);
                }
            }
            const uint32_t p = body[t];
            uint32_t add = 0, sub = 0, radd = 0, rsub = 0;
            for (uint32_t m = 0; m < n_moved; m++) {
                const uint32_t u = moved[m];
                const bool pin = prefix_of(prov[u], L) == pre;
                const bool cin = prefix_of(cur[u], L) == pre;
                if (cin && !pin) { add++; if (body[u] < p) radd++; }
                if (pin && !cin) { sub++; if (body[u] < p) rsub++; }
            }
            const uint32_t count = (hi - lo) + add - sub;
            if (count <= leaf_cap) {
                mask[t] = 0u;  // the cell is a leaf for good: deeper digits unused
                continue;
            }
            // rank of p among the cell's bodies in index order, decided up to
            // leaf_cap (stop once enough smaller indices are seen)
            const uint32_t need = leaf_cap + rsub;
            uint32_t seen = 0;
            for (uint32_t k = lo; k < hi && seen < need; k += 4) {  // four independent loads a round
                uint32_t v4[4];
#pragma unroll
                for (int j = 0; j < 4; j++) v4[j] = (k + (uint32_t)j < hi) ? V[k + (uint32_t)j] : 0xFFFFFFFFu;
#pragma unroll
                for (int j = 0; j < 4; j++) seen += (v4[j] < p) ? 1u : 0u;
            }
            const uint32_t rank = seen + radd - rsub;
            const bool strict = rank < leaf_cap;
            const float x[3] = {pos[3u * p], pos[3u * p + 1u], pos[3u * p + 2u]};
            Cube c = cube_of(bounds, cur[t], L);
            uint32_t o = 0;
            for (int a = 0; a < 3; a++) {
                const float m = midf(c.lo[a], c.hi[a]);
                const bool up = strict ? (m < x[a]) : (m <= x[a]);
                o |= (up ? 1u : 0u) << a;
            }
            const uint32_t old = (uint32_t)(cur[t] >> (3 * (15 - L))) & 7u;
            if (o != old) {
                uint64_t key = (L == 0 ? 0ull : (pre << (3 * (16 - L))));
                key |= (uint64_t)o << (3 * (15 - L));
                Cube cc = cube_of(bounds, key, L + 1);
                uint32_t tb = 0;
                key = descend(x, cc, key, L + 1, tb);
                cur[t] = key;
                // bit 31 marks bodies already in `moved`: each is listed once,
                // however many levels it moves at (its correction is by its
                // current key, so a second entry would count it twice)
                const uint32_t listed = mask[t] & 0x80000000u;
                mask[t] = (mask[t] & ((2u << L) - 1u)) | (tb & ~((2u << L) - 1u) & 0xFFFFu) | 0x80000000u;
                if (!listed) {
                    const uint32_t slot = atomicAdd(&n_moved_next, 1u);
                    if (slot < TIE_CAP) moved[slot] = t;
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) n_moved = min(n_moved_next, TIE_CAP);
        __syncthreads();
    }
    const uint32_t M = n_moved;
    if (threadIdx.x == 0) *moved_out = M;
    // the moved bodies' old slots, ranked ascending, and their new (key,
    // body), ranked ascending
    for (uint32_t m = threadIdx.x; m < M; m += FIX_THREADS) {
        const uint32_t t = moved[m];
        uint32_t k = search_keys(K, samp, ks, 0, prov[t]);
        while (k < nin && V[k] != body[t]) k++;
        uint32_t r_key = 0;
        for (uint32_t q = 0; q < M; q++) {
            const uint32_t u = moved[q];
            if (cur[u] < cur[t] || (cur[u] == cur[t] && body[u] < body[t])) r_key++;
        }
        gkey[r_key] = cur[t];
        gbody[r_key] = body[t];
        mask[t] = k;  // reuse: old slot
    }
    __syncthreads();
    for (uint32_t m = threadIdx.x; m < M; m += FIX_THREADS) {
        const uint32_t t = moved[m];
        uint32_t r = 0;
        for (uint32_t q = 0; q < M; q++)
            if (mask[moved[q]] < mask[t]) r++;
        gpos[r] = mask[t];
    }
    // when the sort left the provisional order in the tree's own arrays, the
    // merge needs it as a separate source (rare: only when a body moved)
    if (M > 0 && copyK)
        for (uint32_t k = threadIdx.x; k < n; k += FIX_THREADS) {
            copyK[k] = K[k];
            copyV[k] = V[k];
        }
}

// (K, V) = the sorted provisional (Ks, Vs) with the moved bodies taken out
// of their old slots and merged back at their new keys.  When nothing moved:
// a plain copy, or nothing at all when the provisional order already sits
// in (K, V) (copy_unmoved = 0).  Replaces a second sort.
constexpr int MERGE_THREADS = 256;

__global__ void __launch_bounds__(MERGE_THREADS) k_tie_merge(const uint64_t* __restrict__ Ks,
                                                             const uint32_t* __restrict__ Vs,
                                                             uint64_t* __restrict__ K, uint32_t* __restrict__ V,
                                                             uint32_t n, const uint32_t* __restrict__ nin_p,
                                                             const uint32_t* __restrict__ moved,
                                                             const uint32_t* __restrict__ gpos,
                                                             const uint64_t* __restrict__ gkey,
                                                             const uint32_t* __restrict__ gbody, int copy_unmoved) {
    const uint32_t M = min(*moved, TIE_CAP);
    const uint32_t stride = gridDim.x * MERGE_THREADS;
    const uint32_t g = blockIdx.x * MERGE_THREADS + threadIdx.x;
    if (M == 0) {
        if (copy_unmoved)
            for (uint32_t k = g; k < n; k += stride) {
                K[k] = Ks[k];
                V[k] = Vs[k];
            }
        return;
    }
    __shared__ uint32_t mpos[TIE_CAP];
    __shared__ uint64_t mkey[TIE_CAP];
    __shared__ uint32_t mbody[TIE_CAP];
    for (uint32_t m = threadIdx.x; m < M; m += MERGE_THREADS) {
        mpos[m] = gpos[m];
        mkey[m] = gkey[m];
        mbody[m] = gbody[m];
    }
    __syncthreads();
    const uint32_t nin = *nin_p;
    auto below_pos = [&](uint32_t k) {  // moved bodies with old slot < k
        uint32_t lo = 0, hi = M;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (mpos[mid] < k) lo = mid + 1; else hi = mid;
        }
        return lo;
    };
    auto below_key = [&](uint64_t key, uint32_t b) {  // moved bodies with (new key, body) < (key, b)
        uint32_t lo = 0, hi = M;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (mkey[mid] < key || (mkey[mid] == key && mbody[mid] < b)) lo = mid + 1; else hi = mid;
        }
        return lo;
    };
    for (uint32_t k = g; k < n; k += stride) {
        if (k >= nin) {  // bodies outside the root cube keep their slots
            K[k] = Ks[k];
            V[k] = Vs[k];
            continue;
        }
        const uint32_t bp = below_pos(k);
        if (bp < M && mpos[bp] == k) continue;  // a moved body's old slot
        const uint64_t key = Ks[k];
        const uint32_t b = Vs[k];
        const uint32_t dst = k - bp + below_key(key, b);
        K[dst] = key;
        V[dst] = b;
    }
    for (uint32_t m = g; m < M; m += stride) {
        // stayed bodies before the new key: binary search on (Ks, Vs), minus moved slots below it
        const uint64_t key = mkey[m];
        const uint32_t b = mbody[m];
        uint32_t lo = 0, hi = nin;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (Ks[mid] < key || (Ks[mid] == key && Vs[mid] < b)) lo = mid + 1; else hi = mid;
        }
        const uint32_t dst = lo - below_pos(lo) + m;
        K[dst] = key;
        V[dst] = b;
    }
}

// Split nodes from the sorted keys, in one pass: s(k), the number of split
// nodes whose range starts at sorted position k, is the run of levels L
// with "k begins a level-L run (K[k-1] differs in the first L digits) and
// K[k+leaf_cap] shares them"; split nodes are numbered by the exclusive
// prefix of s (depth-first preorder), each tile of positions taking its
// prefix from the tiles before it through a decoupled look-back, and every
// split node is written out as (start position, level) right away.
constexpr int SS_THREADS = 256;
constexpr int SS_ITEMS = 4;
constexpr uint32_t SS_TILE = SS_THREADS * SS_ITEMS;
constexpr uint32_t SS_AGG = 1u << 30, SS_INC = 2u << 30, SS_VAL = (1u << 30) - 1u;

__global__ void __launch_bounds__(SS_THREADS) k_split_scan(
    const uint64_t* __restrict__ K, uint32_t n, const uint32_t* __restrict__ nin_p, uint32_t leaf_cap,
    uint32_t depth_max, uint32_t* __restrict__ sbase, uint32_t* __restrict__ split_start,
    uint8_t* __restrict__ split_level, uint32_t split_cap, uint32_t* __restrict__ nsplit_p, uint32_t nodes_max,
    uint32_t* tile_status, uint32_t* ticket, uint32_t* d_status, uint32_t spin_limit) {
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t wsum[SS_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);  // tiles in launch order: the look-back cannot wait on an unstarted tile
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t ntiles = (n + SS_TILE - 1) / SS_TILE;
    const uint32_t nin = *nin_p;
    const uint32_t k0 = tile * SS_TILE + (uint32_t)threadIdx.x * SS_ITEMS;
    uint32_t c[SS_ITEMS];
    int lv[SS_ITEMS];
    uint32_t tsum = 0;
#pragma unroll
    for (int i = 0; i < SS_ITEMS; i++) {
        const uint32_t k = k0 + (uint32_t)i;
        c[i] = 0u;
        lv[i] = -1;
        if (k < nin) {
            const uint64_t key = K[k];
            const int a = (k == 0) ? -1 : cpl_levels(K[k - 1], key);
            int b = -1;
            if (k + leaf_cap < nin) {
                const int cl = cpl_levels(key, K[k + leaf_cap]);
                if (cl >= (int)depth_max && a < (int)depth_max) atomicOr(d_status, SFGPU_STATUS_TREE_DEPTH);
                b = min(cl, (int)depth_max - 1);
            }
            c[i] = (uint32_t)max(0, b - a);
            lv[i] = a;
        }
        tsum += c[i];
    }
    // block exclusive scan of the per-thread sums
    uint32_t x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    uint32_t wbefore = 0, agg = 0;
#pragma unroll
    for (int w = 0; w < SS_THREADS / 32; w++) {
        wbefore += w < warp ? wsum[w] : 0u;
        agg += wsum[w];
    }
    const uint32_t excl = wbefore + x - tsum;
    // decoupled look-back over the preceding tiles (warp 0, 32 tiles a round)
    if (warp == 0) {
        volatile uint32_t* st = tile_status;
        uint32_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) st[0] = SS_INC | (agg & SS_VAL);
        } else {
            if (lane == 0) st[tile] = SS_AGG | (agg & SS_VAL);
            int64_t look = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (true) {
                const int64_t j = look - lane;
                const uint32_t w = j >= 0 ? st[j] : 0u;
                const uint32_t fl = w & ~SS_VAL;
                const uint32_t inc = __ballot_sync(0xffffffffu, j >= 0 && fl == SS_INC);
                const uint32_t gap = __ballot_sync(0xffffffffu, j >= 0 && fl == 0u);
                const int fi = inc ? __ffs(inc) - 1 : 32, fz = gap ? __ffs(gap) - 1 : 32;
                const int take = fi < fz ? fi + 1 : fz;  // the nearest words up to an inclusive one or a gap
                prefix += __reduce_add_sync(0xffffffffu, lane < take ? (w & SS_VAL) : 0u);
                if (fi < fz) break;
                look -= take;
                if (fz < 32 && ++spins > spin_limit) {
                    if (lane == 0) atomicOr(d_status, SFGPU_STATUS_SPIN);
                    break;
                }
            }
            if (lane == 0) st[tile] = SS_INC | ((prefix + agg) & SS_VAL);
        }
        if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    uint32_t run = s_prefix + excl;
#pragma unroll
    for (int i = 0; i < SS_ITEMS; i++) {
        const uint32_t k = k0 + (uint32_t)i;
        if (k < n) sbase[k] = run;
        for (uint32_t j = 0; j < c[i]; j++) {
            const uint32_t id = run + j;
            if (id < split_cap) {
                split_start[id] = k;
                split_level[id] = (uint8_t)(lv[i] + 1 + (int)j);
            }
        }
        run += c[i];
    }
    if (tile == ntiles - 1 && threadIdx.x == 0) {  // the total, and tree.c:180's node limit
        const uint32_t total = s_prefix + agg;
        *nsplit_p = total;
        if (1ull + 8ull * (uint64_t)total >= nodes_max || total > split_cap) atomicOr(d_status, SFGPU_STATUS_TREE_NODES);
    }
}

__device__ __forceinline__ void write_node(NodeArrays nd, uint32_t v, const Cube& c, uint32_t bodies,
                                           uint32_t first_child, uint32_t parent, uint32_t start, float third) {
    const float mx = midf(c.lo[0], c.hi[0]), my = midf(c.lo[1], c.hi[1]), mz = midf(c.lo[2], c.hi[2]);
    // gravity.c:370-374: w = (1/3) * ((dx + dy) + dz), compared as w*w
    const float w = fmul(third, fadd(fadd(fsub(c.hi[0], c.lo[0]), fsub(c.hi[1], c.lo[1])), fsub(c.hi[2], c.lo[2])));
    nd.geo[NODE_REC * v] = make_float4(mx, my, mz, fmul(w, w));
    nd.lo[NODE_REC * v] = make_float4(c.lo[0], c.lo[1], c.lo[2], c.hi[0]);
    nd.hi[NODE_REC * v] = make_float4(c.hi[1], c.hi[2], __uint_as_float(bodies), __uint_as_float(first_child));
    nd.parent[v] = parent;
    nd.start[v] = start;
}

// Monopoles from exact integer sums.  m x, m y, m z and m of every body are
// turned into 64-bit fixed-point integers whose scales (powers of two) are
// set from N, the largest mass and the root cube's extent so that no sum of
// up to N bodies can overflow; the quantisation is 2^-(62 - log2 N) of the
// largest term, far below FP64 rounding of the same sums.  Integer sums are
// exact and associative, so prefix differences are exact, any summation
// order gives the same bits, and nothing runs on GB300's slow FP64 pipe
// except one division per node.
struct FixScale {
    int kx, km;  // q(m x) = m x 2^kx, q(m) = m 2^km
};

__device__ __forceinline__ int ceil_log2_u32(uint32_t v) { return v <= 1u ? 0 : 32 - __clz(v - 1u); }

__device__ __forceinline__ FixScale fix_scale(uint32_t n, uint32_t mmax_bits, const float* __restrict__ bounds) {
    float xmax = 0.0f;
    for (int k = 0; k < 6; k++) xmax = fmaxf(xmax, fabsf(bounds[k]));
    int em = 0, ex = 0;
    frexpf(__uint_as_float(mmax_bits), &em);  // m_max < 2^em
    frexpf(xmax, &ex);                        // |x| <= xmax < 2^ex
    const int room = 62 - ceil_log2_u32(n);
    FixScale f;
    f.kx = room - em - ex;
    f.km = room - em;
    return f;
}

// round(M * 2^s) for |M| < 2^48
__device__ __forceinline__ long long shift_round(long long M, int s) {
    if (s >= 0) return M << s;
    if (s <= -63) return 0;
    return (M + (1ll << (-s - 1))) >> (-s);
}

// exact m * x * 2^k as a rounded integer: 24-bit mantissas multiplied in int64
__device__ __forceinline__ long long fix_mul(float m, float x, int k) {
    int em = 0, ex = 0;
    const float fm = frexpf(m, &em), fx = frexpf(x, &ex);  // m = fm 2^em, fm in [0.5, 1)
    const long long Mm = (long long)(fm * 16777216.0f), Mx = (long long)(fx * 16777216.0f);
    return shift_round(Mm * Mx, em + ex - 48 + k);
}

struct fix4 {
    long long x, y, z, m;
};

// Sorted bodies for the walk, and the fixed-point prefix sums of (m x, m y,
// m z, m) over the sorted slots (zero outside the root cube), in two levels:
// pre[k] = the sum over the slots of k's 32-slot chunk before k (a warp scan),
// cpre[c] = the sum over the chunks before c (the last block to finish scans
// the chunk totals, so no separate launch), cpre[nc] = the total.
constexpr int GATHER_THREADS = 256;

__device__ __forceinline__ long long warp_incl_scan(long long x, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

__global__ void __launch_bounds__(GATHER_THREADS) k_gather(const uint32_t* __restrict__ V, uint32_t n,
                                                           const uint32_t* __restrict__ nin_p,
                                                           const uint32_t* __restrict__ mmax,
                                                           const float* __restrict__ bounds,
                                                           const float* __restrict__ pos,
                                                           const float* __restrict__ mas, float4* __restrict__ sp,
                                                           fix4* __restrict__ pre, fix4* __restrict__ cpre,
                                                           uint32_t* done) {
    const uint32_t k = blockIdx.x * GATHER_THREADS + threadIdx.x;
    const int lane = threadIdx.x & 31;
    long long q[4] = {0, 0, 0, 0};
    if (k < n) {
        const uint32_t p = V[k];
        const float x = pos[3u * p], y = pos[3u * p + 1u], z = pos[3u * p + 2u], w = mas[p];
        sp[k] = make_float4(x, y, z, w);
        if (k < *nin_p) {
            const FixScale f = fix_scale(n, *mmax, bounds);
            q[0] = fix_mul(w, x, f.kx);
            q[1] = fix_mul(w, y, f.kx);
            q[2] = fix_mul(w, z, f.kx);
            q[3] = fix_mul(w, 1.0f, f.km);
        }
    }
    long long incl[4];
#pragma unroll
    for (int c = 0; c < 4; c++) incl[c] = warp_incl_scan(q[c], lane);
    if (k < n) pre[k] = fix4{incl[0] - q[0], incl[1] - q[1], incl[2] - q[2], incl[3] - q[3]};
    if (lane == 31 && (k & ~31u) < n) cpre[k >> 5] = fix4{incl[0], incl[1], incl[2], incl[3]};  // chunk total
    // the last block: exclusive scan of the chunk totals, in place
    __shared__ bool s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(done, 1u) == gridDim.x - 1;
        if (s_last) *done = 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t nc = (n + 31u) >> 5;
    __shared__ long long wsum[4][GATHER_THREADS / 32];
    long long carry[4] = {0, 0, 0, 0};
    for (uint32_t c0 = 0; c0 < nc; c0 += GATHER_THREADS) {
        const uint32_t c = c0 + threadIdx.x;
        long long v[4] = {0, 0, 0, 0};
        if (c < nc) {
            const long long* t = reinterpret_cast<const long long*>(&cpre[c]);
            for (int j = 0; j < 4; j++) v[j] = __ldcg(t + j);
        }
        long long in[4];
        for (int j = 0; j < 4; j++) {
            in[j] = warp_incl_scan(v[j], lane);
            if (lane == 31) wsum[j][threadIdx.x >> 5] = in[j];
        }
        __syncthreads();
        long long ex[4], tot[4];
        for (int j = 0; j < 4; j++) {
            long long w = 0, all = 0;
            for (int u = 0; u < GATHER_THREADS / 32; u++) {
                if (u < (int)(threadIdx.x >> 5)) w += wsum[j][u];
                all += wsum[j][u];
            }
            ex[j] = carry[j] + w + in[j] - v[j];
            tot[j] = all;
        }
        if (c < nc) cpre[c] = fix4{ex[0], ex[1], ex[2], ex[3]};
        for (int j = 0; j < 4; j++) carry[j] += tot[j];
        __syncthreads();
    }
    if (threadIdx.x == 0) cpre[nc] = fix4{carry[0], carry[1], carry[2], carry[3]};
}

// sum over the sorted slots [0, i)
__device__ __forceinline__ fix4 slot_prefix(const fix4* __restrict__ pre, const fix4* __restrict__ cpre, uint32_t i,
                                            uint32_t n) {
    if (i >= n) return cpre[(n + 31u) >> 5];
    const fix4 a = cpre[i >> 5], b = pre[i];
    return fix4{a.x + b.x, a.y + b.y, a.z + b.z, a.m + b.m};
}

// tree.c:302-310: centre of mass = sum(m x) / sum(m), from the exact sums
// over the sorted slots [s, s + cnt)
__device__ __forceinline__ float4 node_monopole(uint32_t s, uint32_t cnt, uint32_t n, const uint32_t* __restrict__ mmax,
                                                const float* __restrict__ bounds, const fix4* __restrict__ msum,
                                                const fix4* __restrict__ cpre, bool nan_in) {
    if (!cnt) return make_float4(0.f, 0.f, 0.f, 0.f);
    const fix4 a = slot_prefix(msum, cpre, s, n), b = slot_prefix(msum, cpre, s + cnt, n);
    const long long sx = b.x - a.x, sy = b.y - a.y, sz = b.z - a.z, sm = b.m - a.m;
    const FixScale f = fix_scale(n, *mmax, bounds);
    const double m = ldexp((double)sm, -f.km);
    // bodies with a NaN coordinate hold the first sorted slots (key 0): in
    // the reference their m x makes every node on their path NaN
    if (nan_in && s == 0u) return make_float4(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff),
                                              __int_as_float(0x7fffffff), (float)m);
    if (sm > 0) {
        const double inv = ldexp(1.0 / (double)sm, f.km - f.kx);  // 2^km / (sm 2^kx)
        return make_float4((float)((double)sx * inv), (float)((double)sy * inv), (float)((double)sz * inv),
                           (float)m);
    }
    return make_float4((float)ldexp((double)sx, -f.kx), (float)ldexp((double)sy, -f.kx),
                       (float)ldexp((double)sz, -f.kx), (float)m);
}

// One split node per 8 threads, thread o writing the node of octant o: its
// first body is the first sorted key at or past octant o of the split cell
// (one table-narrowed search, no chain of gallops), its end the next
// octant's start.  Thread 0 of the group also places the split node itself
// (its id under its parent), which every thread of the group needs.  With
// the fixed-point prefix sums (msum non-NULL) every node written also gets
// its monopole here.
constexpr int FILL_THREADS = 128;

__global__ void __launch_bounds__(FILL_THREADS) k_split_fill(const uint64_t* __restrict__ K, const uint32_t* __restrict__ nin_p,
                             const uint32_t* __restrict__ sbase, const uint32_t* __restrict__ nsplit_p,
                             uint32_t split_cap, const uint32_t* __restrict__ split_start,
                             const uint8_t* __restrict__ split_level, const float* __restrict__ bounds,
                             uint32_t leaf_cap, uint32_t depth_max, NodeArrays nd, float third,
                             uint32_t* __restrict__ split_node, uint32_t n, const uint32_t* __restrict__ mmax,
                             const fix4* __restrict__ msum, const fix4* __restrict__ cpre,
                             const uint32_t* __restrict__ nan_in_p) {
    __shared__ uint64_t samp[NSAMP];
    const uint32_t ns = min(*nsplit_p, split_cap);
    const uint32_t nin = *nin_p;
    const uint32_t g = blockIdx.x * FILL_THREADS + threadIdx.x;
    const uint32_t s = g >> 3;
    const uint32_t o = g & 7u;
    if (g == 0) {  // the root record (tree.c:112-115: bounds = the root cube)
        Cube r;
        for (int a = 0; a < 3; a++) {
            r.lo[a] = bounds[a];
            r.hi[a] = bounds[3 + a];
        }
        write_node(nd, 0, r, nin, (nin > leaf_cap && depth_max > 0) ? 1u : NODE_NONE, 0u, 0u, third);
        if (msum) nd.com[0] = node_monopole(0u, nin, n, mmax, bounds, msum, cpre, *nan_in_p != 0u);
    }
    if ((blockIdx.x * FILL_THREADS) / 8u >= ns) return;  // the whole block is past the split nodes
    const KeySamples ks = load_key_samples(K, nin, samp);
    __syncthreads();
    const bool live = s < ns;
    uint32_t k = 0, cend = 0;
    int L = 0;
    uint64_t pre = 0;
    if (live) {
        k = split_start[s];
        L = split_level[s];
        pre = prefix_of(K[k], L);
        // end of octant o = first key at or past octant o+1 (for o = 7 the
        // next level-L cell, or nin)
        cend = search_keys(K, samp, ks, 3 * (15 - L), (pre << 3) + (uint64_t)o + 1);
    }
    uint32_t cstart = __shfl_up_sync(0xffffffffu, cend, 1, 8);
    if (o == 0) cstart = k;
    if (!live) return;
    // node id of this split node (the children's parent); the node record
    // itself is written by the parent's group
    uint32_t self = 0;
    if (L > 0) {
        const uint32_t kp = (L == 1) ? 0u : search_keys(K, samp, ks, 3 * (17 - L), pre >> 3);
        const int ap = (kp == 0) ? -1 : cpl_levels(K[kp - 1], K[kp]);
        const uint32_t sp = sbase[kp] + (uint32_t)(L - 1 - (ap + 1));
        self = 1u + 8u * sp + (uint32_t)(pre & 7ull);
    }
    if (o == 0) split_node[s] = self;
    const Cube c = cube_of(bounds, K[k], L);
    const uint32_t cnt = cend - cstart;
    Cube cc;
    for (int a = 0; a < 3; a++) {
        const float mid = midf(c.lo[a], c.hi[a]);
        const bool up = (o >> a) & 1u;
        cc.lo[a] = up ? mid : c.lo[a];
        cc.hi[a] = up ? c.hi[a] : mid;
    }
    uint32_t fc = NODE_NONE;
    if (cnt > leaf_cap && L + 1 < (int)depth_max) {
        const int ac = (cstart == 0) ? -1 : cpl_levels(K[cstart - 1], K[cstart]);
        const uint32_t sid = sbase[cstart] + (uint32_t)(L + 1 - (ac + 1));
        // beyond capacity (node overflow, flagged by k_split_emit) the
        // child stays a leaf so nothing reads past the node arrays
        fc = sid < split_cap ? 1u + 8u * sid : NODE_NONE;
    }
    write_node(nd, 1u + 8u * s + o, cc, cnt, fc, self, cstart, third);
    if (msum)
        nd.com[NODE_REC * (1u + 8u * s + o)] = node_monopole(cstart, cnt, n, mmax, bounds, msum, cpre,
                                                             *nan_in_p != 0u);
}

// ---- reference-order monopoles (EXACT arithmetic) ----------------------------
// The reference accumulates each node's sum(m x) and sum(m) in FP32 as bodies
// arrive (tree.c:166-169, 256-259), i.e. in body-index order over the node's
// members, then scales by 1/sum(m) (tree.c:302-310).  Reproduced here: every
// leaf sorts its members by index; going up one level at a time, every split
// node merges its eight children's index-ordered lists (children's ranges are
// adjacent) and adds up its members in that order.
__device__ __forceinline__ float4 ref_com(float sx, float sy, float sz, float sm) {
    const float inv = (0.0f < sm) ? fdiv(1.0f, sm) : 1.0f;
    return make_float4(fmul(sx, inv), fmul(sy, inv), fmul(sz, inv), sm);
}

__global__ void k_ref_leaf_sums(const uint32_t* __restrict__ nsplit_p, uint32_t split_cap, NodeArrays nd,
                                const uint32_t* __restrict__ V, uint32_t* __restrict__ X,
                                const float* __restrict__ pos, const float* __restrict__ mas) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nn = 1u + 8u * min(*nsplit_p, split_cap);
    if (v >= nn) return;
    const float4 H = nd.hi[NODE_REC * v];
    if (__float_as_uint(H.w) != NODE_NONE) return;  // split node: merged later
    const uint32_t cnt = __float_as_uint(H.z);
    const uint32_t s0 = nd.start[v];
    for (uint32_t a = 0; a < cnt; a++) {  // insertion sort by body index
        const uint32_t x = V[s0 + a];
        uint32_t b = a;
        while (b > 0 && X[s0 + b - 1] > x) {
            X[s0 + b] = X[s0 + b - 1];
            b--;
        }
        X[s0 + b] = x;
    }
    float sx = 0.f, sy = 0.f, sz = 0.f, sm = 0.f;
    for (uint32_t a = 0; a < cnt; a++) {
        const uint32_t p = X[s0 + a];
        const float m = mas[p];
        sx = fadd(sx, fmul(m, pos[3u * p]));
        sy = fadd(sy, fmul(m, pos[3u * p + 1u]));
        sz = fadd(sz, fmul(m, pos[3u * p + 2u]));
        sm = fadd(sm, m);
    }
    nd.com[NODE_REC * v] = cnt ? ref_com(sx, sy, sz, sm) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// A CTA per split node of a level: the node's members in index order are
// the merge of its eight children's index-ordered lists, each member's place
// being its rank in its own list plus, for every other child, the number of
// members with a smaller index (a binary search), so all members move at
// once; then warp 0 adds them up in that order: lanes load and multiply 32
// members side by side and the sums take them one by one through shuffles,
// the FP32 chain the reference's insertion order makes.
constexpr int REF_THREADS = 256;

__device__ __forceinline__ uint32_t count_below(const uint32_t* __restrict__ L, uint32_t len, uint32_t x) {
    uint32_t lo = 0, hi = len;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (L[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// the FP32 running sums of m x, m y, m z and m over `cnt` members (warp 0),
// the member of step a being idx(a) when use(it); lane 0 returns the totals
template <typename IdxF, typename UseF>
__device__ __forceinline__ float4 ref_sum_in_order(uint32_t cnt, IdxF idx, UseF use, const float* __restrict__ pos,
                                                   const float* __restrict__ mas) {
    const int lane = threadIdx.x & 31;
    float sx = 0.f, sy = 0.f, sz = 0.f, sm = 0.f;
    for (uint32_t a0 = 0; a0 < cnt; a0 += 32) {
        const uint32_t a = a0 + (uint32_t)lane;
        float mx = 0.f, my = 0.f, mz = 0.f, m = 0.f;
        bool u = false;
        if (a < cnt) {
            const uint32_t p = idx(a);
            u = use(p);
            if (u) {
                m = mas[p];
                mx = fmul(m, pos[3u * p]);  // tree.c:166-169: m x, then +=
                my = fmul(m, pos[3u * p + 1u]);
                mz = fmul(m, pos[3u * p + 2u]);
            }
        }
        const uint32_t ub = __ballot_sync(0xffffffffu, u);
        const int lim = (int)min(32u, cnt - a0);
        for (int l = 0; l < lim; l++) {
            const float tx = __shfl_sync(0xffffffffu, mx, l), ty = __shfl_sync(0xffffffffu, my, l);
            const float tz = __shfl_sync(0xffffffffu, mz, l), tm = __shfl_sync(0xffffffffu, m, l);
            if ((ub >> l) & 1u) {
                sx = fadd(sx, tx);
                sy = fadd(sy, ty);
                sz = fadd(sz, tz);
                sm = fadd(sm, tm);
            }
        }
    }
    return make_float4(sx, sy, sz, sm);
}

__device__ __forceinline__ void ref_level_node(uint32_t s, NodeArrays nd, const uint32_t* __restrict__ split_node,
                                               uint32_t* __restrict__ X, uint32_t* __restrict__ Y,
                                               const float* __restrict__ pos, const float* __restrict__ mas,
                                               uint32_t* cst, uint32_t* cen) {
    const uint32_t v = split_node[s];
    const uint32_t fc = 1u + 8u * s;
    const uint32_t s0 = nd.start[v];
    const uint32_t cnt = __float_as_uint(nd.hi[NODE_REC * v].z);
    if (threadIdx.x < 8) {
        cst[threadIdx.x] = nd.start[fc + threadIdx.x];
        cen[threadIdx.x] = cst[threadIdx.x] + __float_as_uint(nd.hi[NODE_REC * (fc + threadIdx.x)].z);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < cnt; k += REF_THREADS) {
        const uint32_t q = s0 + k;
        int o = 0;
        while (o < 7 && q >= cen[o]) o++;
        const uint32_t x = X[q];
        uint32_t rank = q - cst[o];
        for (int c = 0; c < 8; c++)
            if (c != o) rank += count_below(X + cst[c], cen[c] - cst[c], x);
        Y[s0 + rank] = x;
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < cnt; k += REF_THREADS) X[s0 + k] = Y[s0 + k];
    __syncthreads();
    if (threadIdx.x < 32) {
        const float4 t = ref_sum_in_order(
            cnt, [&](uint32_t a) { return X[s0 + a]; }, [](uint32_t) { return true; }, pos, mas);
        if (threadIdx.x == 0) nd.com[NODE_REC * v] = ref_com(t.x, t.y, t.z, t.w);
    }
    __syncthreads();  // cst / cen are reused by the CTA's next node
}

__global__ void __launch_bounds__(REF_THREADS) k_ref_level(int level, const uint32_t* __restrict__ nsplit_p,
                                                           uint32_t split_cap, const uint8_t* __restrict__ split_level,
                                                           const uint32_t* __restrict__ split_node, NodeArrays nd,
                                                           uint32_t* __restrict__ X, uint32_t* __restrict__ Y,
                                                           const float* __restrict__ pos,
                                                           const float* __restrict__ mas) {
    const uint32_t ns = min(*nsplit_p, split_cap);
    __shared__ uint32_t cst[8], cen[8];
    for (uint32_t s = blockIdx.x; s < ns; s += gridDim.x) {  // the same s on every thread of the CTA
        if (split_level[s] != level) continue;
        ref_level_node(s, nd, split_node, X, Y, pos, mas, cst, cen);
    }
}

// The root's members in index order are simply the bodies inside the root
// cube, by index (tree.c:141-146, the closed test that lets NaN in).
__global__ void k_ref_root(uint32_t n, const float* __restrict__ bounds, NodeArrays nd, const float* __restrict__ pos,
                           const float* __restrict__ mas) {
    if (__float_as_uint(nd.hi[0].w) == NODE_NONE) return;  // a leaf root: k_ref_leaf_sums has it
    const float b[6] = {bounds[0], bounds[1], bounds[2], bounds[3], bounds[4], bounds[5]};
    const float4 t = ref_sum_in_order(
        n, [](uint32_t a) { return a; },
        [&](uint32_t p) {
            const float x = pos[3u * p], y = pos[3u * p + 1u], z = pos[3u * p + 2u];
            return !(b[0] > x || x > b[3] || b[1] > y || y > b[4] || b[2] > z || z > b[5]);
        },
        pos, mas);
    if (threadIdx.x == 0) nd.com[0] = ref_com(t.x, t.y, t.z, t.w);
}

}  // namespace

int sf_tree_alloc(TreeWork** out, uint32_t n, const sfgpu_params& p) {
    TreeWork* t = new TreeWork();
    *out = t;
    t->n = n;
    t->nodes_max = p.nodes_max;
    t->split_cap = p.nodes_max >= 9 ? (p.nodes_max - 1) / 8 : 0;
    const size_t nn = std::max<size_t>(n, 1);
    const size_t nodes = std::max<uint32_t>(p.nodes_max, 16u);
    SF_CUDA(cudaMalloc(&t->keys, sizeof(uint64_t) * nn));
    SF_CUDA(cudaMalloc(&t->vals, sizeof(uint32_t) * nn));
    if (sf_sort_alloc(t->sort, nn) != SFGPU_OK) return SFGPU_FAILURE;
    if (p.spin_limit) t->sort.spin_limit = p.spin_limit;
    // counters: [0] bodies inside, [1] ties, [2] moved, [3] split nodes,
    // [4] largest mass bits, [5] gather ticket, [6] split-scan ticket, [7]
    // a body inside the tree has a NaN coordinate, then one look-back word
    // per split-scan tile
    const size_t ncount = 8 + (nn + SS_TILE - 1) / SS_TILE;
    SF_CUDA(cudaMalloc(&t->counters, sizeof(uint32_t) * ncount));
    SF_CUDA(cudaMemset(t->counters, 0, sizeof(uint32_t) * ncount));
    SF_CUDA(cudaMalloc(&t->ties, sizeof(uint2) * TIE_CAP));
    SF_CUDA(cudaMalloc(&t->tie_pos, sizeof(uint32_t) * TIE_CAP));
    SF_CUDA(cudaMalloc(&t->tie_key, sizeof(uint64_t) * TIE_CAP));
    SF_CUDA(cudaMalloc(&t->tie_body, sizeof(uint32_t) * TIE_CAP));
    SF_CUDA(cudaMalloc(&t->sbase, sizeof(uint32_t) * nn));
    SF_CUDA(cudaMalloc(&t->split_start, sizeof(uint32_t) * std::max<uint32_t>(t->split_cap, 1)));
    SF_CUDA(cudaMalloc(&t->split_level, sizeof(uint8_t) * std::max<uint32_t>(t->split_cap, 1)));
    SF_CUDA(cudaMalloc(&t->split_node, sizeof(uint32_t) * std::max<uint32_t>(t->split_cap, 1)));
    if (p.math == SFGPU_MATH_EXACT) {
        SF_CUDA(cudaMalloc(&t->ordA, sizeof(uint32_t) * nn));
        SF_CUDA(cudaMalloc(&t->ordB, sizeof(uint32_t) * nn));
    }
    SF_CUDA(cudaMalloc(&t->nd.geo, sizeof(float4) * NODE_REC * nodes));  // one 64-byte record per node
    t->nd.lo = t->nd.geo + 1;
    t->nd.hi = t->nd.geo + 2;
    t->nd.com = t->nd.geo + 3;
    SF_CUDA(cudaMalloc(&t->nd.parent, sizeof(uint32_t) * nodes));
    SF_CUDA(cudaMalloc(&t->nd.start, sizeof(uint32_t) * nodes));
    SF_CUDA(cudaMalloc(&t->sp, sizeof(float4) * nn));
    SF_CUDA(cudaMalloc(&t->msum, 32 * nn));              // fix4 per sorted slot
    SF_CUDA(cudaMalloc(&t->cpre, 32 * (nn / 32 + 2)));   // fix4 per 32 slots, + the total
    SF_CUDA(cudaMalloc(&t->walk_part, sizeof(float4) * sf_walk_scratch_floats4((uint32_t)nn)));
    return SFGPU_OK;
}

void sf_tree_free(TreeWork* t) {
    if (!t) return;
    cudaFree(t->keys);
    cudaFree(t->vals);
    sf_sort_free(t->sort);
    cudaFree(t->counters);
    cudaFree(t->ties);
    cudaFree(t->tie_pos);
    cudaFree(t->tie_key);
    cudaFree(t->tie_body);
    cudaFree(t->sbase);
    cudaFree(t->split_start);
    cudaFree(t->split_level);
    cudaFree(t->split_node);
    cudaFree(t->ordA);
    cudaFree(t->ordB);
    cudaFree(t->nd.geo);
    cudaFree(t->nd.parent);
    cudaFree(t->nd.start);
    cudaFree(t->sp);
    cudaFree(t->walk_part);
    cudaFree(t->msum);
    cudaFree(t->cpre);
    delete t;
}

// Build the tree of the slab's current positions inside s->d_bounds.
int sf_tree_build(sfgpu_sim* s) {
    TreeWork* t = s->tree;
    const uint32_t n = s->n;
    cudaStream_t st = s->stream;
    const float* pos = s->slab;
    const float* mas = s->slab + (size_t)9 * n;
    const float third = (float)(1.0 / 3.0);
    uint32_t* nin = t->counters + 0;
    uint32_t* tie_count = t->counters + 1;
    uint32_t* resort = t->counters + 2;
    uint32_t* nsplit = t->counters + 3;
    SF_CUDA(cudaMemsetAsync(t->counters, 0, sizeof(uint32_t) * (8 + sf_ceil_div(n, SS_TILE)), st));
    const uint32_t nb = sf_ceil_div(n, 256);
    int tk = s->timer.begin(st, "tree_keys");
    const SortClear sclr = sf_sort_clear_words(t->sort, n, KEY_BITS);
    k_keys<<<nb, 256, 0, st>>>(pos, mas, n, s->d_bounds, t->keys, t->vals, nin, t->ties, tie_count, t->counters + 4,
                               t->counters + 7, s->d_status, sclr);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    tk = s->timer.begin(st, "tree_sort");
    // the sorted provisional keys stay in the sort's other buffer (7 passes);
    // k_tie_merge writes the final order into (t->keys, t->vals)
    uint64_t* ks = t->keys;
    uint32_t* vs = t->vals;
    if (sf_sort_pairs_keep(t->keys, t->vals, n, KEY_BITS, t->sort, st, s->d_status, &ks, &vs) != SFGPU_OK)
        return SFGPU_FAILURE;
    // the sorted provisional order is in the tree's own arrays (small N, and
    // N <= 1) or in the sort's other buffer (the tile passes)
    const bool in_place = ks == t->keys;
    s->timer.end(st, tk);
    tk = s->timer.begin(st, "tree_ties");
    k_tie_fix<<<1, FIX_THREADS, 0, st>>>(pos, s->d_bounds, ks, vs, nin, t->ties, tie_count, s->p.leaf_cap,
                                         s->p.depth_max, resort, t->tie_pos, t->tie_key, t->tie_body, n,
                                         in_place ? t->sort.keys_b : nullptr, in_place ? t->sort.vals_b : nullptr);
    SF_CHECK_LAUNCH();
    const uint32_t mgb = std::max<uint32_t>(1u, std::min<uint32_t>(sf_ceil_div(n, MERGE_THREADS),
                                                                   (uint32_t)sf_num_sms() * 8u));
    k_tie_merge<<<mgb, MERGE_THREADS, 0, st>>>(in_place ? t->sort.keys_b : ks, in_place ? t->sort.vals_b : vs,
                                                t->keys, t->vals, n, nin, resort, t->tie_pos, t->tie_key,
                                                t->tie_body, in_place ? 0 : 1);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    const bool exact = s->p.math == SFGPU_MATH_EXACT && s->p.form == SFGPU_FORM_PLAIN;
    // the gather (bodies and prefix sums in sorted order) and the split
    // scan (from the sorted keys) are independent: the gather runs on the
    // second stream, joined before the node records need its sums (with
    // per-stage timing both stay on the main stream)
    const bool fork = !s->timer.enabled;
    cudaStream_t gs = fork ? s->aux : st;
    if (fork) {
        SF_CUDA(cudaEventRecord(s->ev_fork, st));
        SF_CUDA(cudaStreamWaitEvent(gs, s->ev_fork, 0));
    }
    tk = s->timer.begin(st, "tree_monopoles");
    k_gather<<<sf_ceil_div(n, GATHER_THREADS), GATHER_THREADS, 0, gs>>>(t->vals, n, nin, t->counters + 4,
                                                                       s->d_bounds, pos, mas, t->sp,
                                                                       (fix4*)t->msum, (fix4*)t->cpre,
                                                                       t->counters + 5);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    if (fork) SF_CUDA(cudaEventRecord(s->ev_join, gs));
    tk = s->timer.begin(st, "tree_nodes");
    k_split_scan<<<sf_ceil_div(n, SS_TILE), SS_THREADS, 0, st>>>(t->keys, n, nin, s->p.leaf_cap, s->p.depth_max,
                                                                  t->sbase, t->split_start, t->split_level,
                                                                  t->split_cap, nsplit, t->nodes_max,
                                                                  t->counters + 8, t->counters + 6, s->d_status,
                                                                  t->sort.spin_limit);
    SF_CHECK_LAUNCH();
    if (fork) SF_CUDA(cudaStreamWaitEvent(st, s->ev_join, 0));
    const uint32_t sb = sf_ceil_div((uint64_t)std::max<uint32_t>(t->split_cap, 1) * 8u, FILL_THREADS);
    k_split_fill<<<sb, FILL_THREADS, 0, st>>>(t->keys, nin, t->sbase, nsplit, t->split_cap, t->split_start, t->split_level,
                                     s->d_bounds, s->p.leaf_cap, s->p.depth_max, t->nd, third, t->split_node, n,
                                     t->counters + 4, exact ? nullptr : (const fix4*)t->msum,
                                     (const fix4*)t->cpre, t->counters + 7);
    SF_CHECK_LAUNCH();
    s->timer.end(st, tk);
    if (exact) {
        tk = s->timer.begin(st, "tree_monopoles");
        const uint32_t mb = sf_ceil_div(1u + 8u * t->split_cap, 256);
        k_ref_leaf_sums<<<mb, 256, 0, st>>>(nsplit, t->split_cap, t->nd, t->vals, t->ordA, pos, mas);
        SF_CHECK_LAUNCH();
        // CTAs stride over the split nodes, working those of the level;
        // level 0, the root, by its own single-warp scan
        const uint32_t sm = std::max<uint32_t>(1u, std::min<uint32_t>(t->split_cap, (uint32_t)sf_num_sms() * 8u));
        for (int L = (int)s->p.depth_max - 1; L >= 1; L--) {
            k_ref_level<<<sm, REF_THREADS, 0, st>>>(L, nsplit, t->split_cap, t->split_level, t->split_node, t->nd,
                                                     t->ordA, t->ordB, pos, mas);
            SF_CHECK_LAUNCH();
        }
        k_ref_root<<<1, 32, 0, st>>>(n, s->d_bounds, t->nd, pos, mas);
        SF_CHECK_LAUNCH();
        s->timer.end(st, tk);
    }
    return SFGPU_OK;
}

int sf_stage_tree_solve(sfgpu_sim* s, bool radius_ready) {
    int tk = s->timer.begin(s->stream, "bounds");
    // kick_drift already reduced the radii and set the root cube
    if (!radius_ready && sf_stage_radius(s) != SFGPU_OK) return SFGPU_FAILURE;
    s->timer.end(s->stream, tk);
    if (sf_tree_build(s) != SFGPU_OK) return SFGPU_FAILURE;
    tk = s->timer.begin(s->stream, "walk");
    if (sf_walk_launch(s) != SFGPU_OK) return SFGPU_FAILURE;
    s->timer.end(s->stream, tk);
    return SFGPU_OK;
}

// ---- inspection -------------------------------------------------------------
int sf_tree_keys(sfgpu_sim* s, uint64_t* keys, uint32_t* index, uint32_t* n_inside) {
    if (!s->tree) {
        sf_set_error("the simulation has no tree");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    if (keys) SF_CUDA(cudaMemcpy(keys, s->tree->keys, sizeof(uint64_t) * s->n, cudaMemcpyDeviceToHost));
    if (index) SF_CUDA(cudaMemcpy(index, s->tree->vals, sizeof(uint32_t) * s->n, cudaMemcpyDeviceToHost));
    if (n_inside) SF_CUDA(cudaMemcpy(n_inside, s->tree->counters, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return SFGPU_OK;
}

int sf_tree_num_nodes(sfgpu_sim* s, uint32_t* num_nodes) {
    if (!s->tree) {
        sf_set_error("the simulation has no tree");
        return SFGPU_FAILURE;
    }
    uint32_t ns = 0;
    SF_CUDA(cudaStreamSynchronize(s->stream));
    SF_CUDA(cudaMemcpy(&ns, s->tree->counters + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    *num_nodes = 1u + 8u * std::min(ns, s->tree->split_cap);
    return SFGPU_OK;
}
