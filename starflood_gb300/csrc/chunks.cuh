// chunks.cuh -- cost-balanced dealing of 32-body chunks to persistent warps.
//
// The SPH passes run one warp per chunk of 32 consecutive sorted bodies, and
// a chunk's cost follows the local density: on a Plummer sphere the core
// chunks cost tens of times what the halo chunks cost.  Launched as one
// block per few chunks, the heavy blocks pile up on some SMs while others
// idle (ncu: the busiest SM active 1.8 to 4 times as long as the least
// busy); persistent warps taking the heaviest chunks first from one counter
// do not fix it either, because each SM's ~40 resident warps take their
// first ~40 chunks at once and those totals differ by a third from SM to
// SM.  So before each pass one block orders the chunks by cost level,
// heaviest first (a counting sort over half-octave levels), and position p
// of that order belongs to SM bin p mod B in snake order (rounds of B
// alternately forward and backward), so the bins' totals are nearly equal.
// The cost is the chunk's measured duration in the same pass of the
// previous step (clock cycles, recorded by the warp that ran it: the sorted
// order, and so each chunk's bodies, changes little from step to step), or
// before the first, an estimate written where the cell grid is built.  A
// warp takes the chunks of its own SM's bin in order, heaviest first; when
// the bin is empty (or its SM has no bin) it takes whatever is left through
// a global counter over all positions, from the light end.  A chunk is
// claimed by a compare-and-swap on its position's word, so each is done
// exactly once whichever way it is reached, and its arithmetic is
// unchanged: the results are the same bits whichever warp takes it.
#pragma once

#include "internal.cuh"

namespace sfchunk {
namespace {  // a copy per translation unit (the kernel included)

constexpr int LEVELS = 64;  // half-octave cost levels
constexpr int KINDS = 2;    // passes with their own measured costs: 0 density, 1 force / momentum

struct ChunkQueue {
    uint32_t* est = nullptr;    // [nchunks] cost estimate written where the grid is built
    uint32_t* cost = nullptr;   // [KINDS][nchunks] measured cost of the last run of each pass kind
    uint32_t* have = nullptr;   // [KINDS] the pass kind has run (its costs are valid)
    uint32_t* order = nullptr;  // [nchunks] chunk ids, heaviest first
    uint32_t* claim = nullptr;  // [nchunks] per position: claimed in this pass (cleared by the ordering)
    uint32_t* ctr = nullptr;    // [0, B) next round of each SM bin, [B] global position, [B + 1] warps done
    uint32_t nchunks = 0;
    uint32_t bins = 0;          // B: the SM count
};

inline int alloc(ChunkQueue& q, uint32_t n) {
    q.nchunks = sf_ceil_div(std::max<uint32_t>(n, 1u), 32u);
    q.bins = (uint32_t)sf_num_sms();
    SF_CUDA(cudaMalloc(&q.est, sizeof(uint32_t) * q.nchunks));
    SF_CUDA(cudaMalloc(&q.cost, sizeof(uint32_t) * KINDS * q.nchunks));
    SF_CUDA(cudaMalloc(&q.have, sizeof(uint32_t) * KINDS));
    SF_CUDA(cudaMalloc(&q.order, sizeof(uint32_t) * q.nchunks));
    SF_CUDA(cudaMalloc(&q.claim, sizeof(uint32_t) * q.nchunks));
    SF_CUDA(cudaMalloc(&q.ctr, sizeof(uint32_t) * (q.bins + 2)));
    SF_CUDA(cudaMemset(q.est, 0, sizeof(uint32_t) * q.nchunks));
    SF_CUDA(cudaMemset(q.have, 0, sizeof(uint32_t) * KINDS));
    SF_CUDA(cudaMemset(q.claim, 0, sizeof(uint32_t) * q.nchunks));
    SF_CUDA(cudaMemset(q.ctr, 0, sizeof(uint32_t) * (q.bins + 2)));
    return SFGPU_OK;
}

inline void release(ChunkQueue& q) {
    cudaFree(q.est);
    cudaFree(q.cost);
    cudaFree(q.have);
    cudaFree(q.order);
    cudaFree(q.claim);
    cudaFree(q.ctr);
    q = ChunkQueue{};
}

__device__ __forceinline__ uint32_t cost_level(uint32_t v) {
    if (v < 2u) return v;
    const uint32_t top = 31u - (uint32_t)__clz(v);
    return min((uint32_t)LEVELS - 1u, 2u * top + ((v >> (top - 1u)) & 1u));
}

// Called by every lane of a warp whose lanes hold the bodies of one chunk
// (sorted slots k = 32 c .. 32 c + 31, lanes past the end with cost 0).
__device__ __forceinline__ void note_cost(const ChunkQueue& q, uint32_t chunk, uint32_t cost) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cost += __shfl_xor_sync(0xffffffffu, cost, o);
    if ((threadIdx.x & 31) == 0) q.est[chunk] = cost;
}

// The cost of a chunk a warp has just run (lane 0), for the next ordering
// of the same pass kind.
__device__ __forceinline__ void record(const ChunkQueue& q, int kind, uint32_t chunk, long long cycles) {
    if ((threadIdx.x & 31) == 0) {
        q.cost[(size_t)kind * q.nchunks + chunk] = (uint32_t)min(cycles, 0xFFFFFFFFll);
        if (q.have[kind] == 0u) q.have[kind] = 1u;
    }
}

// One block: chunk ids into q.order by descending cost level (measured if
// the pass kind has run, else estimated); clears the claims.
__global__ void __launch_bounds__(1024) k_chunk_order(ChunkQueue q, int kind) {
    __shared__ uint32_t s_pos[LEVELS];
    __shared__ uint32_t s_hist[LEVELS];
    const bool measured = q.have[kind] != 0u;
    const uint32_t* src = measured ? q.cost + (size_t)kind * q.nchunks : q.est;
    if (threadIdx.x < LEVELS) s_hist[threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < q.nchunks; c += blockDim.x) atomicAdd(&s_hist[cost_level(src[c])], 1u);
    __syncthreads();
    if (threadIdx.x < 32) {  // positions by descending level: lane l holds levels 2l, 2l + 1
        const uint32_t h0 = s_hist[2 * threadIdx.x], h1 = s_hist[2 * threadIdx.x + 1];
        uint32_t x = h0 + h1;  // sum over levels >= 2l
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_down_sync(0xffffffffu, x, o);
            if (threadIdx.x + o < 32) x += y;
        }
        s_pos[2 * threadIdx.x + 1] = x - h0 - h1;  // level 2l + 1 comes first
        s_pos[2 * threadIdx.x] = x - h0;
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < q.nchunks; c += blockDim.x) {
        const uint32_t pos = atomicAdd(&s_pos[cost_level(src[c])], 1u);
        q.order[pos] = c;
        q.claim[c] = 0u;
    }
}

// A warp's walk through the queue: its own SM's bin first, then the global
// counter.
struct Taker {
    uint32_t bin;   // this SM's bin, or bins (none)
    bool global;    // the bin is empty: take from the global counter
};
__device__ __forceinline__ Taker taker(const ChunkQueue& q) {
    uint32_t sm;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
    return Taker{sm < q.bins ? sm : q.bins, sm >= q.bins};
}

// The warp's next chunk, or 0xFFFFFFFF when none is left.
__device__ __forceinline__ uint32_t next(const ChunkQueue& q, Taker& t) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        uint32_t pos = 0xFFFFFFFFu;
        if (lane == 0) {
            if (!t.global) {
                const uint32_t r = atomicAdd(&q.ctr[t.bin], 1u);
                const uint32_t p = r * q.bins + ((r & 1u) ? q.bins - 1u - t.bin : t.bin);
                if (p < q.nchunks) pos = p;
            }
            if (pos == 0xFFFFFFFFu) {  // from the light end, where the bins arrive last
                const uint32_t g = atomicAdd(&q.ctr[q.bins], 1u);
                if (g < q.nchunks) pos = q.nchunks - 1u - g;
            }
        }
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (pos == 0xFFFFFFFFu) {
            t.global = true;
            return 0xFFFFFFFFu;
        }
        bool won = false;
        if (lane == 0) won = atomicCAS(&q.claim[pos], 0u, 1u) == 0u;
        if (__shfl_sync(0xffffffffu, won, 0)) return q.order[pos];
        // taken already (through its bin or the global counter): go on
    }
}

// Every warp of the launch calls this once, after its last chunk: the last
// one out puts the counters back for the next pass (every other warp has
// taken its last ticket before counting itself out).
__device__ __forceinline__ void warp_exit(const ChunkQueue& q, uint32_t warps) {
    if ((threadIdx.x & 31) == 0) {
        __threadfence();
        if (atomicAdd(&q.ctr[q.bins + 1u], 1u) == warps - 1u) {
            for (uint32_t b = 0; b <= q.bins + 1u; b++) q.ctr[b] = 0u;
        }
    }
}

// Blocks of `threads` for one resident wave of `kernel` (at least 1).
template <typename K>
uint32_t wave_blocks(K kernel, int threads, uint32_t max_blocks) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, 0);
    const uint32_t b = (uint32_t)sf_num_sms() * (uint32_t)std::max(occ, 1);
    return std::max<uint32_t>(1u, std::min(b, max_blocks));
}

}  // namespace
}  // namespace sfchunk
