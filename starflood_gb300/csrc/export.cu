// export.cu -- the tree in the reference's node_t numbering (tree.h:16-25).
//
// The reference numbers nodes in creation order: the root is 0 and a split
// appends the 8 children of the split cell at num_nodes .. num_nodes+7
// (tree.c:263-273).  A cell splits when its (leaf_cap+1)-th body arrives,
// i.e. at the insertion of the (leaf_cap+1)-th smallest body index among its
// members, and one insertion splits cells top-down.  So the reference id of
// the children of split cell s is 1 + 8 r(s) + octant, with r(s) the rank of
// s by (trigger index, level).  Here: one warp per split finds its trigger,
// the splits are radix sorted by (trigger, level), and every node record is
// written at its reference id: parent, bodies, branch[8] (children, or a
// leaf's bodies in index order), bounds, params (centre of mass, mass).
#include "internal.cuh"
#include "tree.cuh"

namespace {

constexpr int TOPK = 17;  // leaf_cap + 1 <= 17

// trigger of each split: the (cap+1)-th smallest body index of its range
__global__ void k_trigger(const uint32_t* __restrict__ nsplit_p, uint32_t split_cap,
                          const uint32_t* __restrict__ split_node, const uint8_t* __restrict__ split_level,
                          NodeArrays nd, const uint32_t* __restrict__ V, uint32_t cap, uint64_t* __restrict__ key,
                          uint32_t* __restrict__ val) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t ns = min(*nsplit_p, split_cap);
    if (warp >= ns) return;
    const uint32_t v = split_node[warp];
    const uint32_t s0 = nd.start[v];
    const uint32_t cnt = __float_as_uint(nd.hi[NODE_REC * v].z);
    uint32_t best[TOPK];
    int nb = 0;
    for (uint32_t a = lane; a < cnt; a += 32) {  // each lane keeps its cap+1 smallest
        const uint32_t x = V[s0 + a];
        if (nb < (int)cap + 1) {
            int b = nb++;
            while (b > 0 && best[b - 1] > x) {
                best[b] = best[b - 1];
                b--;
            }
            best[b] = x;
        } else if (x < best[cap]) {
            int b = (int)cap;
            while (b > 0 && best[b - 1] > x) {
                best[b] = best[b - 1];
                b--;
            }
            best[b] = x;
        }
    }
    int head = 0;
    uint32_t last = 0;
    for (uint32_t round = 0; round <= cap; round++) {  // merge the lanes' lists
        const uint32_t mine = head < nb ? best[head] : 0xFFFFFFFFu;
        const uint32_t m = __reduce_min_sync(0xffffffffu, mine);
        const uint32_t who = __ballot_sync(0xffffffffu, mine == m && m != 0xFFFFFFFFu);
        if (who && lane == __ffs(who) - 1) head++;
        last = m;
    }
    if (lane == 0) {
        key[warp] = ((uint64_t)last << 5) | (uint64_t)split_level[warp];
        val[warp] = warp;
    }
}

__global__ void k_rank(const uint32_t* __restrict__ sorted_val, uint32_t ns, uint32_t* __restrict__ rank) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ns) rank[sorted_val[i]] = i;
}

__device__ __forceinline__ uint32_t ref_id(uint32_t v, const uint32_t* __restrict__ rank) {
    if (v == 0) return 0;
    const uint32_t s = (v - 1u) >> 3, o = (v - 1u) & 7u;
    return 1u + 8u * rank[s] + o;
}

__global__ void k_export(uint32_t nn, NodeArrays nd, const uint32_t* __restrict__ V,
                         const uint32_t* __restrict__ rank, uint32_t* __restrict__ parent,
                         uint32_t* __restrict__ bodies, uint32_t* __restrict__ branch, float* __restrict__ bounds,
                         float* __restrict__ params) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn) return;
    const uint32_t R = ref_id(v, rank);
    const float4 Lo = nd.lo[NODE_REC * v], H = nd.hi[NODE_REC * v], C = nd.com[NODE_REC * v];
    const uint32_t cnt = __float_as_uint(H.z);
    const uint32_t first = __float_as_uint(H.w);
    parent[R] = v == 0 ? 0u : ref_id(nd.parent[v], rank);
    bodies[R] = cnt;
    uint32_t br[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (first != NODE_NONE) {
        for (int o = 0; o < 8; o++) br[o] = ref_id(first + o, rank);
    } else {
        const uint32_t s0 = nd.start[v];
        const uint32_t m = min(cnt, 8u);
        for (uint32_t a = 0; a < m; a++) {  // the leaf's bodies in index order
            const uint32_t x = V[s0 + a];
            uint32_t b = a;
            while (b > 0 && br[b - 1] > x) {
                br[b] = br[b - 1];
                b--;
            }
            br[b] = x;
        }
    }
    for (int o = 0; o < 8; o++) branch[8u * R + o] = br[o];
    const float b6[6] = {Lo.x, Lo.y, Lo.z, Lo.w, H.x, H.y};
    for (int a = 0; a < 6; a++) bounds[6u * R + a] = b6[a];
    params[4u * R + 0] = C.x;
    params[4u * R + 1] = C.y;
    params[4u * R + 2] = C.z;
    params[4u * R + 3] = C.w;
}

}  // namespace

int sf_tree_export(sfgpu_sim* s, uint32_t* parent, uint32_t* bodies, uint32_t* branch8, float* bounds6,
                   float* params4) {
    TreeWork* t = s->tree;
    if (!t) {
        sf_set_error("the simulation has no tree");
        return SFGPU_FAILURE;
    }
    if (s->p.leaf_cap > 8) {
        sf_set_error("node_t holds 8 bodies per leaf: export needs leaf_cap <= 8");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    uint32_t ns = 0;
    SF_CUDA(cudaMemcpy(&ns, t->counters + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (ns > t->split_cap) {
        sf_set_error("the last build overflowed the node capacity");
        return SFGPU_FAILURE;
    }
    const uint32_t nn = 1u + 8u * ns;
    uint64_t* key = nullptr;
    uint32_t *val = nullptr, *rank = nullptr, *d_par = nullptr, *d_bod = nullptr, *d_br = nullptr;
    float *d_bnd = nullptr, *d_prm = nullptr;
    SortWork sw;
    int rc = SFGPU_FAILURE;
    cudaError_t e = cudaSuccess;
#define EXP_TRY(call)                                                                   \
    do {                                                                                \
        e = (call);                                                                     \
        if (e != cudaSuccess) goto done;                                                \
    } while (0)
    EXP_TRY(cudaMalloc(&key, sizeof(uint64_t) * (ns + 1)));
    EXP_TRY(cudaMalloc(&val, sizeof(uint32_t) * (ns + 1)));
    EXP_TRY(cudaMalloc(&rank, sizeof(uint32_t) * (ns + 1)));
    EXP_TRY(cudaMalloc(&d_par, sizeof(uint32_t) * nn));
    EXP_TRY(cudaMalloc(&d_bod, sizeof(uint32_t) * nn));
    EXP_TRY(cudaMalloc(&d_br, sizeof(uint32_t) * 8 * nn));
    EXP_TRY(cudaMalloc(&d_bnd, sizeof(float) * 6 * nn));
    EXP_TRY(cudaMalloc(&d_prm, sizeof(float) * 4 * nn));
    if (ns) {
        const uint32_t threads = 32u * ns;
        k_trigger<<<sf_ceil_div(threads, 256), 256, 0, s->stream>>>(t->counters + 3, t->split_cap, t->split_node,
                                                                    t->split_level, t->nd, t->vals, s->p.leaf_cap,
                                                                    key, val);
        EXP_TRY(cudaGetLastError());
        if (sf_sort_alloc(sw, ns) != SFGPU_OK) goto done_msg;
        if (sf_sort_pairs(key, val, ns, 37, sw, s->stream, s->d_status) != SFGPU_OK) goto done_msg;
        k_rank<<<sf_ceil_div(ns, 256), 256, 0, s->stream>>>(val, ns, rank);
        EXP_TRY(cudaGetLastError());
    }
    k_export<<<sf_ceil_div(nn, 256), 256, 0, s->stream>>>(nn, t->nd, t->vals, rank, d_par, d_bod, d_br, d_bnd, d_prm);
    EXP_TRY(cudaGetLastError());
    EXP_TRY(cudaStreamSynchronize(s->stream));
    if (parent) EXP_TRY(cudaMemcpy(parent, d_par, sizeof(uint32_t) * nn, cudaMemcpyDeviceToHost));
    if (bodies) EXP_TRY(cudaMemcpy(bodies, d_bod, sizeof(uint32_t) * nn, cudaMemcpyDeviceToHost));
    if (branch8) EXP_TRY(cudaMemcpy(branch8, d_br, sizeof(uint32_t) * 8 * nn, cudaMemcpyDeviceToHost));
    if (bounds6) EXP_TRY(cudaMemcpy(bounds6, d_bnd, sizeof(float) * 6 * nn, cudaMemcpyDeviceToHost));
    if (params4) EXP_TRY(cudaMemcpy(params4, d_prm, sizeof(float) * 4 * nn, cudaMemcpyDeviceToHost));
    rc = SFGPU_OK;
done:
    if (e != cudaSuccess) sf_set_error("tree export: %s", cudaGetErrorString(e));
done_msg:
#undef EXP_TRY
    sf_sort_free(sw);
    cudaFree(key);
    cudaFree(val);
    cudaFree(rank);
    cudaFree(d_par);
    cudaFree(d_bod);
    cudaFree(d_br);
    cudaFree(d_bnd);
    cudaFree(d_prm);
    return rc;
}
