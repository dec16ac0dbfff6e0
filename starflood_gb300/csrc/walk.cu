// walk.cu -- Barnes-Hut monopole walk, solve_gravity_part_tree
// (src/gravity.c:242-663).
//
// A warp takes 32 consecutive bodies of the key order (spatially close) and
// walks the union of their trees with one shared stack of (node, lane mask)
// entries.  At an internal node each lane in the mask runs the reference's
// opening test with the reference's FP32 rounding (so the set of cells every
// body interacts with is exactly the reference's); lanes that do not open
// take the node as a monopole, the others continue into its children, which
// are pushed in reverse octant order.  Each lane therefore meets its cells in
// the same depth-first octant order as the reference's stackless walk
// (gravity.c:306-579), which lets the EXACT variant reproduce its Kahan sums.
// Leaves (bodies <= leaf_cap) are always monopoles; empty cells are skipped;
// the reference's self-exclusion (gravity.c:473-490) is applied to every
// cell whose closed bounds contain the body.
#include "internal.cuh"
#include "tree.cuh"

namespace {

constexpr int WALK_WARPS = 4;
constexpr int WALK_THREADS = WALK_WARPS * 32;
constexpr int STACK = 8 * 17 + 8;

enum WalkKind { WALK_FAST = 0, WALK_EXACT = 1, WALK_COMP = 2 };

template <int KIND, bool STATS>
__global__ void __launch_bounds__(WALK_THREADS) k_walk(const float4* __restrict__ sp, const uint32_t* __restrict__ V,
                                                       uint32_t n, NodeArrays nd, ForceConsts fc, uint32_t leaf_cap,
                                                       float* __restrict__ acc, float* __restrict__ pot,
                                                       uint32_t* __restrict__ st_int, uint32_t* __restrict__ st_open,
                                                       unsigned long long* __restrict__ tot, uint32_t* d_status) {
    __shared__ uint32_t s_node[WALK_WARPS][STACK];
    __shared__ uint32_t s_mask[WALK_WARPS][STACK];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const uint32_t k = blockIdx.x * WALK_THREADS + threadIdx.x;
    const bool live = k < n;
    const float4 b = live ? sp[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rx = b.x, ry = b.y, rz = b.z, mi = b.w;
    const uint32_t live_mask = __ballot_sync(0xffffffffu, live);
    if (!live_mask) return;

    KSum ax{0.f, 0.f}, ay{0.f, 0.f}, az{0.f, 0.f}, ph{0.f, 0.f};
    uint32_t n_int = 0, n_open = 0;
    int top = 0;
    if (lane == 0) {
        s_node[w][0] = 0u;
        s_mask[w][0] = live_mask;
    }
    top = 1;
    __syncwarp();
    uint32_t guard = 0;
    while (top > 0) {
        top--;
        const uint32_t v = s_node[w][top];
        const uint32_t M = s_mask[w][top];
        __syncwarp();
        if (++guard > fc.walk_limit) {  // cannot happen for a well-formed tree under the default limit
            if (lane == 0) atomicOr(d_status, SFGPU_STATUS_WALK);
            break;
        }
        const float4 H = nd.hi[NODE_REC * v];
        const uint32_t bodies = __float_as_uint(H.z);
        if (bodies == 0u) continue;  // gravity.c:324-328
        const bool me = (M >> lane) & 1u;
        uint32_t take = M;
        if (bodies > leaf_cap) {
            const float4 G = nd.geo[NODE_REC * v];
            bool open = false;
            if (me) {
                // gravity.c:352-377, 448: open when theta <= (w*w)/d2
                const float ox = fsub(G.x, rx), oy = fsub(G.y, ry), oz = fsub(G.z, rz);
                const float d2 = fadd(fadd(fmul(ox, ox), fmul(oy, oy)), fmul(oz, oz));
                const float ratio = (0.0f < d2) ? fdiv(G.w, d2) : 0.0f;
                open = fc.theta <= ratio;
                n_open++;
            }
            const uint32_t om = __ballot_sync(0xffffffffu, me && open);
            take = M & ~om;
            if (om) {
                const uint32_t first = __float_as_uint(H.w);
                if (top + 8 > STACK || first == NODE_NONE) {
                    if (lane == 0) atomicOr(d_status, SFGPU_STATUS_WALK);
                    take = M;  // fall back to the monopole rather than overflow
                } else {
                    if (lane < 8) {
                        s_node[w][top + lane] = first + 7u - (uint32_t)lane;
                        s_mask[w][top + lane] = om;
                    }
                    top += 8;
                }
            }
            __syncwarp();
        }
        if ((take >> lane) & 1u) {
            const float4 C = nd.com[NODE_REC * v];
            const float4 Lo = nd.lo[NODE_REC * v];
            float cx = C.x, cy = C.y, cz = C.z, mj = C.w;
            // gravity.c:473-490: take body i out of a cell that contains it
            if (Lo.x <= rx && rx <= Lo.w && Lo.y <= ry && ry <= H.x && Lo.z <= rz && rz <= H.y && 1u < bodies) {
                cx = fmul(cx, mj);
                cy = fmul(cy, mj);
                cz = fmul(cz, mj);
                cx = fsub(cx, fmul(mi, rx));
                cy = fsub(cy, fmul(mi, ry));
                cz = fsub(cz, fmul(mi, rz));
                mj = fsub(mj, mi);
                const float f = (0.0f < mj) ? fdiv(1.0f, mj) : 1.0f;
                cx = fmul(cx, f);
                cy = fmul(cy, f);
                cz = fmul(cz, f);
            }
            if (KIND == WALK_EXACT) {
                // gravity.c:493-548 with Kahan sums: accumulates sum F, F = phi/s r_ij
                const float dx = fsub(rx, cx), dy = fsub(ry, cy), dz = fsub(rz, cz);
                const float r2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
                const float s = fadd(r2, fc.eps2);
                const float inv2 = fdiv(1.0f, s);
                const float inv1 = fdiv(1.0f, fsqrt(s));
                const float phi = fmul(mj, inv1);
                const float f = fmul(phi, inv2);
                ax.add(fmul(f, dx));
                ay.add(fmul(f, dy));
                az.add(fmul(f, dz));
                ph.add(phi);
            } else {
                // accumulates S = sum m_j (r_j - r_i) / s^1.5 = -sum F
                const float dx = cx - rx, dy = cy - ry, dz = cz - rz;
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, fc.eps2)));
                const float inv = rsqrtf(r2);
                const float mphi = mj * inv;
                const float f = mphi * (inv * inv);
                if (KIND == WALK_COMP) {
                    ax.add(f * dx);
                    ay.add(f * dy);
                    az.add(f * dz);
                    ph.add(mphi);
                } else {
                    ax.s = fmaf(f, dx, ax.s);
                    ay.s = fmaf(f, dy, ay.s);
                    az.s = fmaf(f, dz, az.s);
                    ph.s += mphi;
                }
            }
            n_int++;
        }
    }
    if (live) {
        const uint32_t p = V[k];
        if (KIND == WALK_EXACT) {
            // gravity.c:656-659
            const float scale = fc.physical ? fc.neg_g : fmul(fc.neg_g, mi);
            acc[3u * p + 0u] = fmul(scale, ax.s);
            acc[3u * p + 1u] = fmul(scale, ay.s);
            acc[3u * p + 2u] = fmul(scale, az.s);
            pot[p] = fmul(fc.neg_g, ph.s);
        } else {
            const float g = -fc.neg_g;
            const float scale = fc.physical ? g : g * mi;
            acc[3u * p + 0u] = scale * (ax.s + (KIND == WALK_COMP ? -ax.c : 0.f));
            acc[3u * p + 1u] = scale * (ay.s + (KIND == WALK_COMP ? -ay.c : 0.f));
            acc[3u * p + 2u] = scale * (az.s + (KIND == WALK_COMP ? -az.c : 0.f));
            pot[p] = fc.neg_g * (ph.s + (KIND == WALK_COMP ? -ph.c : 0.f));
        }
        if (STATS) {
            st_int[p] = n_int;
            st_open[p] = n_open;
        }
    }
    // totals for the flop count
    unsigned long long ci = n_int, co = n_open;
    for (int o = 16; o > 0; o >>= 1) {
        ci += __shfl_xor_sync(0xffffffffu, ci, o);
        co += __shfl_xor_sync(0xffffffffu, co, o);
    }
    if (lane == 0) {
        atomicAdd(&tot[0], ci);
        atomicAdd(&tot[1], co);
    }
}

template <int KIND>
int launch_kind(sfgpu_sim* s, bool stats) {
    TreeWork* t = s->tree;
    const ForceConsts fc = sf_force_consts(s->p);
    const uint32_t grid = sf_ceil_div(s->n, WALK_THREADS);
    float* acc = s->slab + (size_t)6 * s->n;
    float* pot = s->slab + (size_t)10 * s->n;
    if (stats)
        k_walk<KIND, true><<<grid, WALK_THREADS, 0, s->stream>>>(t->sp, t->vals, s->n, t->nd, fc, s->p.leaf_cap, acc,
                                                                 pot, s->stat_int, s->stat_open, s->walk_tot,
                                                                 s->d_status);
    else
        k_walk<KIND, false><<<grid, WALK_THREADS, 0, s->stream>>>(t->sp, t->vals, s->n, t->nd, fc, s->p.leaf_cap, acc,
                                                                  pot, nullptr, nullptr, s->walk_tot, s->d_status);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

// ---- split walk (FAST / COMPENSATED) ----------------------------------------
// The walk above runs one warp per 32 bodies: 2048 warps for 65,536 bodies,
// about 13 per SM, each a chain of dependent node loads.  Here SPLIT warps
// share a group of 32 bodies, warp p walking only the subtree of root octant
// p (warp 0 also takes the root itself as a monopole for lanes that do not
// open it).  Partial sums go to scratch and k_walk_reduce adds them in octant
// order.  All four node vectors are loaded at once per visit, and the
// opening test compares by products, falling back to the IEEE divide only
// within 2^-19 of theta, so every decision equals the reference's.
constexpr int SPLIT = 8;

__device__ __forceinline__ bool opens(const float4& G, float rx, float ry, float rz, const ForceConsts& fc,
                                      float th_lo, float th_hi) {
    const float ox = fsub(G.x, rx), oy = fsub(G.y, ry), oz = fsub(G.z, rz);
    const float d2 = fadd(fadd(fmul(ox, ox), fmul(oy, oy)), fmul(oz, oz));
    if (!(0.0f < d2)) return fc.theta <= 0.0f;
    // G.w / d2 against theta by products (each within 2^-24 of exact, far
    // inside the 2^-19 margins of th_lo, th_hi); the IEEE quotient only in
    // between
    if (G.w > fmul(th_hi, d2)) return true;
    if (G.w < fmul(th_lo, d2)) return false;
    return fc.theta <= fdiv(G.w, d2);
}

// The same test for two (cell, body) pairs at once, each element rounded as
// the scalar test: differences and products on paired FP32 instructions
// (a - b as a + (-b), which IEEE defines to be the same), the sums of the
// squares scalar (measured on GB300: ptxas fuses a paired product into a
// following paired add, even one written as add.rn.f32x2, which rounds d^2
// differently in about a fifth of the cases), so both decisions equal
// opens().
__device__ __forceinline__ bool open_decide(float w, float d2, float hi, float lo, const ForceConsts& fc) {
    if (!(0.0f < d2)) return fc.theta <= 0.0f;
    if (w > hi) return true;
    if (w < lo) return false;
    return fc.theta <= fdiv(w, d2);
}
__device__ __forceinline__ void opens2(float2 gx, float2 gy, float2 gz, float2 gw, float2 rx, float2 ry, float2 rz,
                                       const ForceConsts& fc, float th_lo, float th_hi, bool& o0, bool& o1) {
    const float2 ox = __fadd2_rn(gx, make_float2(-rx.x, -rx.y));
    const float2 oy = __fadd2_rn(gy, make_float2(-ry.x, -ry.y));
    const float2 oz = __fadd2_rn(gz, make_float2(-rz.x, -rz.y));
    const float2 px = __fmul2_rn(ox, ox), py = __fmul2_rn(oy, oy), pz = __fmul2_rn(oz, oz);
    const float2 d2 = make_float2(fadd(fadd(px.x, py.x), pz.x), fadd(fadd(px.y, py.y), pz.y));
    const float2 hi = __fmul2_rn(make_float2(th_hi, th_hi), d2);
    const float2 lo = __fmul2_rn(make_float2(th_lo, th_lo), d2);
    o0 = open_decide(gw.x, d2.x, hi.x, lo.x, fc);
    o1 = open_decide(gw.y, d2.y, hi.y, lo.y, fc);
}

template <int KIND>
__device__ __forceinline__ void monopole(const float4& C, const float4& Lo, const float4& H, uint32_t bodies, float rx,
                                         float ry, float rz, float mi, float eps2, KSum& ax, KSum& ay, KSum& az,
                                         KSum& ph) {
    float cx = C.x, cy = C.y, cz = C.z, mj = C.w;
    if (Lo.x <= rx && rx <= Lo.w && Lo.y <= ry && ry <= H.x && Lo.z <= rz && rz <= H.y && 1u < bodies) {
        cx = fsub(fmul(cx, mj), fmul(mi, rx));
        cy = fsub(fmul(cy, mj), fmul(mi, ry));
        cz = fsub(fmul(cz, mj), fmul(mi, rz));
        mj = fsub(mj, mi);
        const float f = (0.0f < mj) ? fdiv(1.0f, mj) : 1.0f;
        cx = fmul(cx, f);
        cy = fmul(cy, f);
        cz = fmul(cz, f);
    }
    const float dx = cx - rx, dy = cy - ry, dz = cz - rz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    const float inv = rsqrtf(r2);
    const float mphi = mj * inv;
    const float f = mphi * (inv * inv);
    if (KIND == WALK_COMP) {
        ax.add(f * dx);
        ay.add(f * dy);
        az.add(f * dz);
        ph.add(mphi);
    } else {
        ax.s = fmaf(f, dx, ax.s);
        ay.s = fmaf(f, dy, ay.s);
        az.s = fmaf(f, dz, az.s);
        ph.s += mphi;
    }
}

// One thread walks one body's tree, stacklessly, in the reference's order:
// into the first child when a cell opens, on to the next sibling (children
// are numbered contiguously), up through the parent links when the last
// sibling is done (gravity.c:306-579 keeps the same walk state as a path of
// octants).  With SPLIT > 1, SPLIT warps share 32 bodies and warp o walks
// only the subtree of root octant o; partial sums are added by
// k_walk_reduce.
template <int KIND, int SPLIT_, bool STATS>
__global__ void __launch_bounds__(WALK_THREADS) k_walk_body(const float4* __restrict__ sp,
                                                            const uint32_t* __restrict__ V, uint32_t n,
                                                            NodeArrays nd, ForceConsts fc, float th_lo, float th_hi,
                                                            uint32_t leaf_cap, float4* __restrict__ part,
                                                            float* __restrict__ acc, float* __restrict__ pot,
                                                            uint32_t* __restrict__ st_int,
                                                            uint32_t* __restrict__ st_open,
                                                            unsigned long long* __restrict__ tot,
                                                            uint32_t* d_status) {
    const int lane = threadIdx.x & 31;
    const uint32_t gw = blockIdx.x * WALK_WARPS + (threadIdx.x >> 5);
    const uint32_t group = gw / SPLIT_;
    const uint32_t oct = gw % SPLIT_;
    const uint32_t k = group * 32u + lane;
    const bool live = k < n;
    const float4 b = live ? sp[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rx = b.x, ry = b.y, rz = b.z, mi = b.w;
    KSum ax{0.f, 0.f}, ay{0.f, 0.f}, az{0.f, 0.f}, ph{0.f, 0.f};
    uint32_t n_int = 0, n_open = 0;

    if (live) {
        const float4 H = __ldg(&nd.hi[NODE_REC * 0]);
        const uint32_t bodies = __float_as_uint(H.z);
        const uint32_t first = __float_as_uint(H.w);
        bool descend_root = false;
        if (bodies > 0u) {
            if (bodies > leaf_cap) {
                if (oct == 0) n_open++;
                descend_root = opens(__ldg(&nd.geo[NODE_REC * 0]), rx, ry, rz, fc, th_lo, th_hi) && first != NODE_NONE;
            }
            if (!descend_root && oct == 0) {
                monopole<KIND>(__ldg(&nd.com[NODE_REC * 0]), __ldg(&nd.lo[NODE_REC * 0]), H, bodies, rx, ry, rz, mi, fc.eps2, ax, ay, az,
                               ph);
                n_int++;
            }
        }
        if (descend_root) {
            // SPLIT_ == 1: walk all of the root's children; else only octant oct
            const uint32_t stop = SPLIT_ == 1 ? 0u : first + oct;
            uint32_t v = SPLIT_ == 1 ? first : first + oct;
            uint32_t guard = 0;
            while (true) {
                if (++guard > fc.walk_limit) {
                    atomicOr(d_status, SFGPU_STATUS_WALK);
                    break;
                }
                const float4 Hv = __ldg(&nd.hi[NODE_REC * v]);
                const float4 G = __ldg(&nd.geo[NODE_REC * v]);
                const float4 C = __ldg(&nd.com[NODE_REC * v]);
                const float4 Lo = __ldg(&nd.lo[NODE_REC * v]);
                const uint32_t bv = __float_as_uint(Hv.z);
                bool down = false;
                if (bv > 0u) {
                    if (bv > leaf_cap) {
                        n_open++;
                        const uint32_t fcv = __float_as_uint(Hv.w);
                        down = fcv != NODE_NONE && opens(G, rx, ry, rz, fc, th_lo, th_hi);
                        if (down) v = fcv;
                        else if (fcv == NODE_NONE) atomicOr(d_status, SFGPU_STATUS_WALK);
                    }
                    if (!down) {
                        monopole<KIND>(C, Lo, Hv, bv, rx, ry, rz, mi, fc.eps2, ax, ay, az, ph);
                        n_int++;
                    }
                }
                if (down) continue;
                // the subtree of v is done: next sibling, or climb
                bool done = false;
                while (true) {
                    if (v == stop) {
                        done = true;
                        break;
                    }
                    if (((v - 1u) & 7u) != 7u) {
                        v += 1u;
                        break;
                    }
                    v = __ldg(&nd.parent[v]);
                }
                if (done) break;
            }
        }
    }
    if (live) {
        float4 r;
        if (KIND == WALK_COMP)
            r = make_float4(ax.s - ax.c, ay.s - ay.c, az.s - az.c, ph.s - ph.c);
        else
            r = make_float4(ax.s, ay.s, az.s, ph.s);
        const uint32_t p = V[k];
        if (SPLIT_ == 1) {
            const float g = -fc.neg_g;
            const float scale = fc.physical ? g : g * mi;
            acc[3u * p + 0u] = scale * r.x;
            acc[3u * p + 1u] = scale * r.y;
            acc[3u * p + 2u] = scale * r.z;
            pot[p] = fc.neg_g * r.w;
            if (STATS) {
                st_int[p] = n_int;
                st_open[p] = n_open;
            }
        } else {
            part[(size_t)oct * n + k] = r;
            if (STATS) {
                atomicAdd(&st_int[p], n_int);
                atomicAdd(&st_open[p], n_open);
            }
        }
    }
    unsigned long long ci = n_int, co = n_open;
    for (int o = 16; o > 0; o >>= 1) {
        ci += __shfl_xor_sync(0xffffffffu, ci, o);
        co += __shfl_xor_sync(0xffffffffu, co, o);
    }
    if (lane == 0 && (ci | co)) {
        atomicAdd(&tot[0], ci);
        atomicAdd(&tot[1], co);
    }
}

// acc = G m_i sum_p S_p (S = -sum F), pot = -G sum_p phi_p, octant order.
template <int KIND>
__global__ void k_walk_reduce(const float4* __restrict__ part, const float4* __restrict__ sp,
                              const uint32_t* __restrict__ V, uint32_t n, ForceConsts fc, float* __restrict__ acc,
                              float* __restrict__ pot) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float mi = sp[k].w;
    const uint32_t p = V[k];
    const float g = -fc.neg_g;
    if (KIND == WALK_COMP) {
        double x = 0, y = 0, z = 0, w = 0;
        for (int o = 0; o < SPLIT; o++) {
            const float4 t = part[(size_t)o * n + k];
            x += t.x;
            y += t.y;
            z += t.z;
            w += t.w;
        }
        const double scale = fc.physical ? (double)g : (double)g * (double)mi;
        acc[3u * p + 0u] = (float)(scale * x);
        acc[3u * p + 1u] = (float)(scale * y);
        acc[3u * p + 2u] = (float)(scale * z);
        pot[p] = (float)((double)fc.neg_g * w);
    } else {
        float4 s = part[k];
        for (int o = 1; o < SPLIT; o++) {
            const float4 t = part[(size_t)o * n + k];
            s.x += t.x;
            s.y += t.y;
            s.z += t.z;
            s.w += t.w;
        }
        const float scale = fc.physical ? g : g * mi;
        acc[3u * p + 0u] = scale * s.x;
        acc[3u * p + 1u] = scale * s.y;
        acc[3u * p + 2u] = scale * s.z;
        pot[p] = fc.neg_g * s.w;
    }
}

template <int KIND, int SPLIT_>
int launch_body(sfgpu_sim* s, bool stats) {
    TreeWork* t = s->tree;
    const ForceConsts fc = sf_force_consts(s->p);
    const float th_lo = fc.theta * (1.0f - 1.0f / 524288.0f);
    const float th_hi = fc.theta * (1.0f + 1.0f / 524288.0f);
    const uint32_t groups = sf_ceil_div(s->n, 32);
    const uint32_t grid = sf_ceil_div((uint64_t)groups * SPLIT_, WALK_WARPS);
    float* acc = s->slab + (size_t)6 * s->n;
    float* pot = s->slab + (size_t)10 * s->n;
    if (stats) {
        if (SPLIT_ > 1) {
            SF_CUDA(cudaMemsetAsync(s->stat_int, 0, sizeof(uint32_t) * s->n, s->stream));
            SF_CUDA(cudaMemsetAsync(s->stat_open, 0, sizeof(uint32_t) * s->n, s->stream));
        }
        k_walk_body<KIND, SPLIT_, true><<<grid, WALK_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, s->p.leaf_cap, t->walk_part, acc, pot, s->stat_int,
            s->stat_open, s->walk_tot, s->d_status);
    } else {
        k_walk_body<KIND, SPLIT_, false><<<grid, WALK_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, s->p.leaf_cap, t->walk_part, acc, pot, nullptr, nullptr,
            s->walk_tot, s->d_status);
    }
    SF_CHECK_LAUNCH();
    if (SPLIT_ > 1) {
        k_walk_reduce<KIND><<<sf_ceil_div(s->n, 256), 256, 0, s->stream>>>(t->walk_part, t->sp, t->vals, s->n, fc,
                                                                           acc, pot);
        SF_CHECK_LAUNCH();
    }
    return SFGPU_OK;
}

// ---- group walk (FAST / COMPENSATED, the default) -----------------------------
// A warp walks the tree for its group of bodies (16 by default, consecutive
// in key order), but the lanes work on up to 32 stack entries (cell, mask of
// bodies still walking it)
// at once, so the loads of many cells are in flight together.  Each entry is
// classified against the bounding box of the group: with margins of 2^-12 on
// theta, far larger than the FP32 rounding of the reference's ratio, "every
// body accepts" (w^2 < theta d_min^2) and "every body opens"
// (w^2 >= theta d_max^2) are certain to agree with each body's own FP32
// decision; only the remaining "mixed" cells are tested body by body with the
// reference's arithmetic.  Accepted (cell, mask) pairs go to a list in shared
// memory that all 32 lanes then run through with dense monopole
// interactions (one body per lane; with 16- or 8-body groups the sub-warps
// share the entries).  Every body ends up with exactly the cells the reference
// gives it (the per-body interaction counts are checked in the tests).
// Bodies per group of the group walk unless sfgpu_params.walk_group says
// otherwise.  On the 65,536-body uniform sphere (one GB300): 32 bodies
// 0.157 ms, 16 bodies 0.137 ms per walk.
constexpr uint32_t WALK_GROUP_DEFAULT = 16;
constexpr int GW_WARPS = 4;
constexpr int GW_THREADS = GW_WARPS * 32;
constexpr int GW_STACK = 512;
constexpr int GW_GSTACK = 128;  // sibling-group entries per warp of k_walk_sib
constexpr int GW_LIST = 112;  // accepted cells whose bounds miss the group box
constexpr int GW_MIN_BLOCKS = 7;  // resident blocks per SM the register budget is cut for
constexpr int GW_SLOW = 48;   // accepted cells that may contain a body (self-exclusion test)
constexpr int PART_LEVELS = 3;  // k_walk_sib walks a group in parts that share their top 3 octants

// Per-warp lists in shared memory.  The fast list holds the monopole itself
// (centre of mass and mass) and the mask of the bodies taking it, entries
// stored in pairs so that one 128-bit load brings (x0, x1, y0, y1) and
// another (z0, z1, m0, m1) of two consecutive entries; the slow list holds
// node ids for the few accepted cells whose closed bounds meet the group's
// box, where the reference's self-exclusion test must run.
struct GroupLists {
    float* xy;  // entry e: x at 4 (e/2) + e%2, y at 4 (e/2) + 2 + e%2
    float* zm;  // entry e: z at 4 (e/2) + e%2, m at 4 (e/2) + 2 + e%2
    uint32_t* msk;
    uint32_t* qn;
    uint32_t* qm;
};
__device__ __forceinline__ int lx_of(int e) { return 4 * (e >> 1) + (e & 1); }

// Fast list: every lane runs every entry, its mask bit selecting the result,
// so the inner loop has no per-lane branch.  FAST kind evaluates two entries
// per instruction (paired FP32); COMP kind adds each interaction to Kahan
// sums in list order.
// With 16- or 8-body groups the 2 or 4 sub-warps hold the same bodies and
// take entries in turn (FAST: entry pairs), `lane` being the body slot and
// `half` the sub-warp.
// COUNT: count each body's interactions here (per-body statistics);
// otherwise the caller counts whole entries as they are listed.
template <int KIND, int GB, bool COUNT>
__device__ __forceinline__ void flush_fast(const GroupLists& L, int count, int lane, int half, float rx, float ry,
                                           float rz, float eps2, float2& a2x, float2& a2y, float2& a2z, float2& p2,
                                           KSum& ax, KSum& ay, KSum& az, KSum& ph, uint32_t& n_int) {
    constexpr int H = 32 / GB;  // half-warps sharing the list
    if (KIND == WALK_COMP) {
        for (int e = half; e < count; e += H) {
            const uint32_t M = L.msk[e];
            if ((M >> lane) & 1u) {
                const int ix = lx_of(e);
                const float dx = L.xy[ix] - rx, dy = L.xy[ix + 2] - ry, dz = L.zm[ix] - rz;
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                const float inv = rsqrtf(r2);
                const float mphi = L.zm[ix + 2] * inv;
                const float f = mphi * (inv * inv);
                ax.add(f * dx);
                ay.add(f * dy);
                az.add(f * dz);
                ph.add(mphi);
                if (COUNT) n_int++;
            }
        }
        return;
    }
    const float2 nrx = make_float2(-rx, -rx), nry = make_float2(-ry, -ry), nrz = make_float2(-rz, -rz);
    const float2 e2 = make_float2(eps2, eps2);
#pragma unroll 2
    for (int e = 2 * half; e < count; e += 2 * H) {  // count is a multiple of 2H (padded by the caller)
        const float4 A = reinterpret_cast<const float4*>(L.xy)[e >> 1];
        const float4 B = reinterpret_cast<const float4*>(L.zm)[e >> 1];
        const float2 X = make_float2(A.x, A.y), Y = make_float2(A.z, A.w);
        const float2 Z = make_float2(B.x, B.y), M2 = make_float2(B.z, B.w);
        const uint2 MK = *reinterpret_cast<const uint2*>(&L.msk[e]);
        const bool t0 = (MK.x >> lane) & 1u, t1 = (MK.y >> lane) & 1u;
        // a body not taking an entry sees it massless: its terms are +0
        const float2 Mj = make_float2(t0 ? M2.x : 0.f, t1 ? M2.y : 0.f);
        const float2 dx = __fadd2_rn(X, nrx);
        const float2 dy = __fadd2_rn(Y, nry);
        const float2 dz = __fadd2_rn(Z, nrz);
        float2 r2 = __ffma2_rn(dz, dz, e2);
        r2 = __ffma2_rn(dy, dy, r2);
        r2 = __ffma2_rn(dx, dx, r2);
        const float2 inv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
        const float2 mphi = __fmul2_rn(Mj, inv);
        const float2 f = __fmul2_rn(mphi, __fmul2_rn(inv, inv));
        a2x = __ffma2_rn(f, dx, a2x);
        a2y = __ffma2_rn(f, dy, a2y);
        a2z = __ffma2_rn(f, dz, a2z);
        p2 = __fadd2_rn(p2, mphi);
        if (COUNT) n_int += (uint32_t)t0 + (uint32_t)t1;
    }
}

template <int KIND, int GB, bool COUNT>
__device__ __forceinline__ void flush_slow(const GroupLists& L, int count, const NodeArrays& nd, int lane, int half,
                                           float rx, float ry, float rz, float mi, float eps2, KSum& ax, KSum& ay,
                                           KSum& az, KSum& ph, uint32_t& n_int) {
    for (int e = half; e < count; e += 32 / GB) {
        const uint32_t v = L.qn[e];
        const uint32_t M = L.qm[e];
        const float4 C = __ldg(&nd.com[NODE_REC * v]);
        const float4 Lo = __ldg(&nd.lo[NODE_REC * v]);
        const float4 H = __ldg(&nd.hi[NODE_REC * v]);
        if ((M >> lane) & 1u) {
            monopole<KIND>(C, Lo, H, __float_as_uint(H.z), rx, ry, rz, mi, eps2, ax, ay, az, ph);
            if (COUNT) n_int++;
        }
    }
}

// Appends the cells of the lanes with am != 0 (their C, Lo, H loaded) to the
// fast or the slow list.
__device__ __forceinline__ void append_cells(const GroupLists& L, uint32_t am, uint32_t v, const float4& C,
                                             const float4& Lo, const float4& H, float bx0, float by0, float bz0,
                                             float bx1, float by1, float bz1, int lane, int& count, int& qcount) {
    const uint32_t lt = (1u << lane) - 1u;
    // the reference's self-exclusion needs a body inside the closed bounds
    // of a cell with more than one body: impossible when the bounds miss
    // the group's box
    const bool slow = am != 0u && __float_as_uint(H.z) > 1u && !(Lo.w < bx0 || bx1 < Lo.x || H.x < by0 ||
                                                                  by1 < Lo.y || H.y < bz0 || bz1 < Lo.z);
    const uint32_t sb = __ballot_sync(0xffffffffu, slow);
    const uint32_t fb = __ballot_sync(0xffffffffu, am != 0u && !slow);
    if (slow) {
        const int q = qcount + __popc(sb & lt);
        L.qn[q] = v;
        L.qm[q] = am;
    } else if (am) {
        const int q = count + __popc(fb & lt);
        const int ix = lx_of(q);
        L.xy[ix] = C.x;
        L.xy[ix + 2] = C.y;
        L.zm[ix] = C.z;
        L.zm[ix + 2] = C.w;
        L.msk[q] = am;
    }
    count += __popc(fb);
    qcount += __popc(sb);
}

// kick_1 of sim_step and the energies (simulation.c:420-497), applied by the
// walk's epilogue to each body as soon as its force is known, when no SPH
// force follows the walk: one pass and one launch fewer per step.  The
// per-body arithmetic is k_kick_energy's; the block partials (float-float
// within warps, FP64 across them) are added in block order by the last
// block, which also advances the device step counter.
struct WalkKick {
    float* vel;
    float* ken;
    float* pen;
    double* vel64;      // FP64 velocities (precision form) or NULL
    double dt64;
    float half_dt;
    float g_over_eps;   // G / eps: the self term of the corrected potential
    int physical;
    double* part;       // [gridDim.x][4]
    uint32_t* done;     // last-block ticket
    double* sums;       // [0] T, [1] V, [2] corrected kinetic, [3] corrected potential
    uint32_t* d_step;
};

__device__ __forceinline__ void walk_kick_body(const WalkKick& wk, uint32_t p, float mi, const float a[3], float potp,
                                               ff (&e)[4]) {
    float v[3];
    double v64[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const size_t q = 3u * (size_t)p + c;
        if (wk.vel64) {
            v64[c] = wk.vel64[q] + 0.5 * wk.dt64 * (double)a[c];
            wk.vel64[q] = v64[c];
            v[c] = (float)v64[c];
        } else {
            v[c] = fadd(wk.vel[q], fmul(wk.half_dt, a[c]));  // simulation.c:424
            v64[c] = v[c];
        }
        wk.vel[q] = v[c];
    }
    // simulation.c:443-450
    const float v2 = fadd(fadd(fmul(v[0], v[0]), fmul(v[1], v[1])), fmul(v[2], v[2]));
    const float k_i = fmul(fmul(0.5f, mi), v2);
    const float p_i = fmul(mi, potp);
    wk.ken[p] = k_i;
    wk.pen[p] = p_i;
    if (wk.vel64) {
        const double v2d = v64[0] * v64[0] + v64[1] * v64[1] + v64[2] * v64[2];
        e[2] = ff_from_double(wk.physical ? 0.5 * (double)mi * v2d : 0.5 * v2d);
    } else {
        e[2] = ff_from(wk.physical ? fmul(fmul(0.5f, mi), v2) : fmul(0.5f, v2));
    }
    e[3] = ff_from(fmul(fmul(0.5f, mi), fadd(potp, fmul(wk.g_over_eps, mi))));
    e[0] = ff_from(k_i);
    e[1] = ff_from(p_i);
}

// Block partials of e (every thread of the block calls this), then the last
// block's ordered FP64 totals.
__device__ void walk_kick_reduce(const WalkKick& wk, ff (&e)[4]) {
    __shared__ double wsum[4][GW_WARPS];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ff_warp_sum<4>(e);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 4; k++) wsum[k][warp] = ff_to_double(e[k]);
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            double t = 0.0;
            for (int u = 0; u < GW_WARPS; u++) t += wsum[k][u];
            wk.part[(size_t)blockIdx.x * 4 + k] = t;
        }
        __threadfence();
        s_last = atomicAdd(wk.done, 1u) == gridDim.x - 1;
        if (s_last) *wk.done = 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t q = threadIdx.x; q < gridDim.x; q += GW_THREADS)
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] += __ldcg(&wk.part[(size_t)q * 4 + k]);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; k++) {
        double x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) wsum[k][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            double t = 0.0;
            for (int u = 0; u < GW_WARPS; u++) t += wsum[k][u];
            wk.sums[k] = t;
        }
        *wk.d_step += 1u;
    }
}

template <int KIND, int GSPLIT, int GB, bool STATS, bool KICK = false>
__global__ void __launch_bounds__(GW_THREADS, GW_MIN_BLOCKS) k_walk_group(const float4* __restrict__ sp,
                                                           const uint32_t* __restrict__ V, uint32_t n, NodeArrays nd,
                                                           ForceConsts fc, float th_lo, float th_hi,
                                                           float th_acc, float th_open, uint32_t leaf_cap,
                                                           float4* __restrict__ part,
                                                           float* __restrict__ acc, float* __restrict__ pot,
                                                           uint32_t* __restrict__ st_int,
                                                           uint32_t* __restrict__ st_open,
                                                           unsigned long long* __restrict__ tot, uint32_t* d_status,
                                                           WalkKick wk) {
    __shared__ uint32_t s_node[GW_WARPS][GW_STACK];
    __shared__ uint32_t s_mask[GW_WARPS][GW_STACK];
    __shared__ __align__(16) float l_xy[GW_WARPS][2 * GW_LIST];
    __shared__ __align__(16) float l_zm[GW_WARPS][2 * GW_LIST];
    __shared__ __align__(16) uint32_t l_k[GW_WARPS][GW_LIST];
    __shared__ uint32_t q_node[GW_WARPS][GW_SLOW];
    __shared__ uint32_t q_mask[GW_WARPS][GW_SLOW];
    __shared__ float4 s_body[GW_WARPS][32];
    __shared__ float4 s_mg[GW_WARPS][32];     // a round's mixed cells: centre and w^2,
    __shared__ uint32_t s_mm[GW_WARPS][32];   // the bodies walking them,
    __shared__ uint32_t s_om[GW_WARPS][32];   // and the bodies that open them
    constexpr int FRONT = GSPLIT > 1 ? 80 : 1;
    __shared__ uint32_t f_node[GW_WARPS][FRONT];  // top-level frontiers: [0,8) level 1, [8,72) level 2
    __shared__ uint32_t f_mask[GW_WARPS][FRONT];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    float4* sbd = s_body[w];
    uint32_t* stn = s_node[w];
    uint32_t* stm = s_mask[w];
    const GroupLists L{l_xy[w], l_zm[w], l_k[w], q_node[w], q_mask[w]};
    static_assert(GB == 32 || ((GB == 16 || GB == 8) && GSPLIT == 1), "8- and 16-body groups walk unsplit");
    const uint32_t gw = blockIdx.x * GW_WARPS + w;
    const uint32_t group = gw / GSPLIT;
    const uint32_t oct = gw % GSPLIT;
    // body slot of the lane (both half-warps hold the same 16 bodies when GB = 16)
    const int bl = lane & (GB - 1), half = lane / GB;
    const uint32_t body_bits = GB == 32 ? 0xffffffffu : (1u << GB) - 1u;
    const uint32_t k = group * (uint32_t)GB + (uint32_t)bl;
    const bool live = k < n;
    const uint32_t live_mask = __ballot_sync(0xffffffffu, live) & body_bits;
    // with the fused kick every warp reaches the block reduction; a warp
    // past the last body walks nothing
    if (!live_mask && !KICK) return;
    const float4 b = sp[live ? k : min(group * (uint32_t)GB, n - 1u)];
    const float rx = b.x, ry = b.y, rz = b.z, mi = b.w;
    if (half == 0) sbd[bl] = b;
    __syncwarp();
    // bounding box of the group (dead lanes repeat the first body)
    float bx0 = rx, by0 = ry, bz0 = rz, bx1 = rx, by1 = ry, bz1 = rz;
    for (int o = 16; o > 0; o >>= 1) {
        bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
        by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
        bz0 = fminf(bz0, __shfl_xor_sync(0xffffffffu, bz0, o));
        bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
        by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
        bz1 = fmaxf(bz1, __shfl_xor_sync(0xffffffffu, bz1, o));
    }
    KSum ax{0.f, 0.f}, ay{0.f, 0.f}, az{0.f, 0.f}, ph{0.f, 0.f};
    float2 a2x = make_float2(0.f, 0.f), a2y = a2x, a2z = a2x, p2 = a2x;
    uint32_t n_int = 0, n_open = 0;
    unsigned long long open_total = 0;
    int top = 0, count = 0, qcount = 0;
    auto flush = [&](bool all) {
        if (all || count > GW_LIST - 36) {
            // FAST: pad to a multiple of 2 (4 with two half-warps) with
            // entries no lane takes
            constexpr int PAD = KIND == WALK_COMP ? 1 : 2 * (32 / GB);
            const int padded = (count + PAD - 1) / PAD * PAD;
            if (lane < padded - count) {
                const int ix = lx_of(count + lane);
                L.xy[ix] = L.xy[ix + 2] = L.zm[ix] = L.zm[ix + 2] = 0.f;
                L.msk[count + lane] = 0u;
            }
            count = padded;
            __syncwarp();
            flush_fast<KIND, GB, STATS>(L, count, bl, half, rx, ry, rz, fc.eps2, a2x, a2y, a2z, p2, ax, ay, az, ph,
                                        n_int);
            count = 0;
            __syncwarp();
        }
        if (all || qcount > GW_SLOW - 32) {
            flush_slow<KIND, GB, STATS>(L, qcount, nd, bl, half, rx, ry, rz, mi, fc.eps2, ax, ay, az, ph, n_int);
            qcount = 0;
            __syncwarp();
        }
    };
    if (GSPLIT == 1) {
        if (lane == 0) {
            stn[0] = 0u;
            stm[0] = live_mask;
        }
        top = live_mask ? 1 : 0;
    } else {
        // Every warp of the group walks the top two levels itself (exact
        // per-body tests); the up to 64 cells left at level 2 are dealt out
        // round-robin, warp `oct` keeping cells j with j % GSPLIT == oct, so
        // the expensive near-field cells spread over the warps.  Cells
        // accepted above level 2 (and the opening-test totals there) belong
        // to warp 0.
        uint32_t* fnd = f_node[w];
        uint32_t* fms = f_mask[w];
        int n_in = 1, in_base = 0, out_base = 0;  // level 0 writes the 8 level-1 slots [0, 8)
        for (int lvl = 0; lvl < 2; lvl++) {
            uint32_t v = 0u, M = 0u, first = NODE_NONE, bodies = 0u;
            float4 G = make_float4(0.f, 0.f, 0.f, 0.f), H = G, C = G, Lo = G;
            if (lane < n_in) {
                v = lvl == 0 ? 0u : fnd[in_base + lane];
                M = lvl == 0 ? live_mask : fms[in_base + lane];
                H = __ldg(&nd.hi[NODE_REC * v]);
                G = __ldg(&nd.geo[NODE_REC * v]);
                C = __ldg(&nd.com[NODE_REC * v]);
                Lo = __ldg(&nd.lo[NODE_REC * v]);
                bodies = __float_as_uint(H.z);
                first = __float_as_uint(H.w);
            }
            const bool internal = lane < n_in && bodies > leaf_cap;
            uint32_t om = 0u;
            if (internal && first != NODE_NONE) {
                uint32_t mm = M;
                while (mm) {
                    const int i = __ffs(mm) - 1;
                    mm &= mm - 1u;
                    const float4 bi = sbd[i];
                    if (opens(G, bi.x, bi.y, bi.z, fc, th_lo, th_hi)) om |= 1u << i;
                }
            }
            if (internal && oct == 0) open_total += __popc(M);
            if (STATS && oct == 0) {
                for (int l = 0; l < n_in; l++) {
                    const bool il = __shfl_sync(0xffffffffu, internal, l);
                    const uint32_t ml = __shfl_sync(0xffffffffu, M, l);
                    if (il && ((ml >> lane) & 1u)) n_open++;
                }
            }
            const uint32_t am = (oct == 0 && lane < n_in && bodies > 0u) ? (M & ~om) : 0u;
            const uint32_t lt = (1u << lane) - 1u;
            append_cells(L, am, v, C, Lo, H, bx0, by0, bz0, bx1, by1, bz1, lane, count, qcount);
            if (!STATS) n_int += __popc(am);
            const uint32_t ob = __ballot_sync(0xffffffffu, om != 0u);
            if (om) {
                const int base = out_base + 8 * __popc(ob & lt);
                for (int o = 0; o < 8; o++) {
                    fnd[base + o] = first + (uint32_t)o;
                    fms[base + o] = om;
                }
            }
            __syncwarp();
            n_in = 8 * __popc(ob);
            in_base = out_base;
            out_base = 8;  // level 1 writes the 64 level-2 slots [8, 72)
        }
        // level-2 cells: this warp's share onto its stack
        for (int j0 = 0; j0 < n_in; j0 += 32) {
            const int j = j0 + lane;
            const bool mine = j < n_in && (j % GSPLIT) == (int)oct;
            const uint32_t mb = __ballot_sync(0xffffffffu, mine);
            if (mine) {
                const int slot = top + __popc(mb & ((1u << lane) - 1u));
                stn[slot] = fnd[in_base + j];
                stm[slot] = fms[in_base + j];
            }
            top += __popc(mb);
        }
    }
    __syncwarp();
    uint32_t guard = 0;
    while (top > 0) {
        if (++guard > fc.walk_limit) {
            if (lane == 0) atomicOr(d_status, SFGPU_STATUS_WALK);
            break;
        }
        int pops = min(32, min(top, (GW_STACK - top) / 8));
        if (pops == 0) {  // no room for children: cannot happen with GW_STACK >> depth * 8
            if (lane == 0) atomicOr(d_status, SFGPU_STATUS_WALK);
            break;
        }
        uint32_t v = 0, M = 0;
        if (lane < pops) {
            v = stn[top - 1 - lane];
            M = stm[top - 1 - lane];
        }
        top -= pops;
        __syncwarp();
        // 0 drop, 1 accept, 2 open, 3 mixed
        int kind = 0;
        bool internal = false;
        float4 G = make_float4(0.f, 0.f, 0.f, 0.f), H = G, C = G, Lo = G;
        uint32_t first = NODE_NONE;
        if (lane < pops) {
            // the whole node record in one round trip (the monopole half is
            // needed by every accepted or mixed cell, most of the entries)
            H = __ldg(&nd.hi[NODE_REC * v]);
            G = __ldg(&nd.geo[NODE_REC * v]);
            C = __ldg(&nd.com[NODE_REC * v]);
            Lo = __ldg(&nd.lo[NODE_REC * v]);
            const uint32_t bodies = __float_as_uint(H.z);
            first = __float_as_uint(H.w);
            internal = bodies > leaf_cap;
            if (bodies == 0u) {
                kind = 0;
            } else if (bodies <= leaf_cap) {
                kind = 1;
            } else {
                open_total += __popc(M);
                // distances from the cell centre to the group's box (nearest, farthest)
                const float ex = fmaxf(0.f, fmaxf(bx0 - G.x, G.x - bx1));
                const float ey = fmaxf(0.f, fmaxf(by0 - G.y, G.y - by1));
                const float ez = fmaxf(0.f, fmaxf(bz0 - G.z, G.z - bz1));
                const float fx = fmaxf(fabsf(G.x - bx0), fabsf(G.x - bx1));
                const float fy = fmaxf(fabsf(G.y - by0), fabsf(G.y - by1));
                const float fz = fmaxf(fabsf(G.z - bz0), fabsf(G.z - bz1));
                const float dmin2 = (ex * ex + ey * ey + ez * ez) * (1.0f - 1.0f / 65536.0f);
                const float dmax2 = (fx * fx + fy * fy + fz * fz) * (1.0f + 1.0f / 65536.0f);
                if (dmin2 > 0.0f && G.w < th_acc * dmin2) kind = 1;
                else if (G.w >= th_open * dmax2 && first != NODE_NONE) kind = 2;
                else kind = 3;
            }
        }
        // cells every body opens -> their children
        const uint32_t lt = (1u << lane) - 1u;
        const uint32_t open_b = __ballot_sync(0xffffffffu, kind == 2);
        if (kind == 2) {
            const int base = top + 8 * __popc(open_b & lt);
            for (int o = 0; o < 8; o++) {
                stn[base + o] = first + 7u - (uint32_t)o;
                stm[base + o] = M;
            }
        }
        top += 8 * __popc(open_b);
        // mixed cells: the reference's test for each (cell, body) pair of
        // the masks.  Either one lane per cell loops over its bodies, or the
        // warp goes through the cells one at a time with one lane per body,
        // whichever takes fewer rounds.
        const bool mixed = kind == 3 && first != NODE_NONE;
        const uint32_t mix_b = __ballot_sync(0xffffffffu, mixed);
        uint32_t om = 0u;
        if (mix_b) {
            constexpr int H = 32 / GB;  // sub-warps, each testing one cell per round
            const int rounds_cell = (__popc(mix_b) + H - 1) / H;
            const int rounds_body = __reduce_max_sync(0xffffffffu, mixed ? (uint32_t)__popc(M) : 0u);
            if (rounds_body <= rounds_cell) {
                if (mixed) {
                    uint32_t mm = M;
                    while (mm) {
                        const int i = __ffs(mm) - 1;
                        mm &= mm - 1u;
                        const float4 bi = sbd[i];
                        if (opens(G, bi.x, bi.y, bi.z, fc, th_lo, th_hi)) om |= 1u << i;
                    }
                }
            } else {
                // the mixed cells staged in shared memory in lane order;
                // sub-warp h tests cell j H + h in round j, one lane per body
                const int nmix = __popc(mix_b);
                const int slot = __popc(mix_b & lt);
                if (mixed) {
                    s_mg[w][slot] = G;
                    s_mm[w][slot] = M;
                }
                __syncwarp();
                for (int j0 = 0; j0 < nmix; j0 += H) {  // the same trip count on every lane
                    const int j = j0 + half;
                    bool t = false;
                    if (j < nmix) {
                        const uint32_t Mj = s_mm[w][j];
                        t = ((Mj >> bl) & 1u) && opens(s_mg[w][j], rx, ry, rz, fc, th_lo, th_hi);
                    }
                    const uint32_t ol = __ballot_sync(0xffffffffu, t);
                    if (bl == 0 && j < nmix) s_om[w][j] = (ol >> (half * GB)) & body_bits;
                }
                __syncwarp();
                if (mixed) om = s_om[w][slot];
            }
        }
        // accepted cells (all of the mask, or the bodies of a mixed cell
        // that do not open it) -> lists
        const uint32_t am = (kind == 1) ? M : ((kind == 3) ? (M & ~om) : 0u);
        append_cells(L, am, v, C, Lo, H, bx0, by0, bz0, bx1, by1, bz1, lane, count, qcount);
        if (!STATS) n_int += __popc(am);
        const uint32_t ob = __ballot_sync(0xffffffffu, om != 0u);
        if (om) {
            const int base = top + 8 * __popc(ob & lt);
            for (int o = 0; o < 8; o++) {
                stn[base + o] = first + 7u - (uint32_t)o;
                stm[base + o] = om;
            }
        }
        top += 8 * __popc(ob);
        __syncwarp();
        if (STATS) {  // opening tests (internal cells only) attributed to bodies
            for (int l = 0; l < pops; l++) {
                const bool il = __shfl_sync(0xffffffffu, internal, l);
                const uint32_t ml = __shfl_sync(0xffffffffu, M, l);
                if (il && half == 0 && ((ml >> bl) & 1u)) n_open++;
            }
        }
        flush(false);
    }
    flush(true);
    float sx = ax.s, sy = ay.s, sz = az.s, sw = ph.s;
    if (KIND == WALK_COMP) {
        sx -= ax.c;
        sy -= ay.c;
        sz -= az.c;
        sw -= ph.c;
    } else {
        sx += a2x.x + a2x.y;
        sy += a2y.x + a2y.y;
        sz += a2z.x + a2z.y;
        sw += p2.x + p2.y;
    }
    uint32_t n_int_body = n_int;
#pragma unroll
    for (int o = 16; o >= GB; o >>= 1) {  // the sub-warps' shares of the same bodies
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
        n_int_body += __shfl_xor_sync(0xffffffffu, n_int_body, o);
    }
    ff e[4] = {ff{0.f, 0.f}, ff{0.f, 0.f}, ff{0.f, 0.f}, ff{0.f, 0.f}};
    if (live && half == 0) {
        const uint32_t p = V[k];
        if (GSPLIT == 1) {
            const float g = -fc.neg_g;
            const float scale = fc.physical ? g : g * mi;
            const float a[3] = {scale * sx, scale * sy, scale * sz};
            acc[3u * p + 0u] = a[0];
            acc[3u * p + 1u] = a[1];
            acc[3u * p + 2u] = a[2];
            pot[p] = fc.neg_g * sw;
            if (KICK) walk_kick_body(wk, p, mi, a, fc.neg_g * sw, e);
            if (STATS) {
                st_int[p] = n_int_body;
                st_open[p] = n_open;
            }
        } else {
            part[(size_t)oct * n + k] = make_float4(sx, sy, sz, sw);
            if (STATS) {
                atomicAdd(&st_int[p], n_int_body);
                atomicAdd(&st_open[p], n_open);
            }
        }
    }
    unsigned long long ci = n_int;
    for (int o = 16; o > 0; o >>= 1) {
        ci += __shfl_xor_sync(0xffffffffu, ci, o);
        open_total += __shfl_xor_sync(0xffffffffu, open_total, o);
    }
    if (lane == 0) {
        atomicAdd(&tot[0], ci);
        atomicAdd(&tot[1], open_total);
    }
    if (KICK) walk_kick_reduce(wk, e);
}

// The default walk: the group walk above with a stack of sibling groups.
template <int KIND, int GB, bool STATS, bool KICK = false>
__global__ void __launch_bounds__(GW_THREADS, GW_MIN_BLOCKS) k_walk_sib(const float4* __restrict__ sp,
                                                           const uint32_t* __restrict__ V, uint32_t n, NodeArrays nd,
                                                           ForceConsts fc, float th_lo, float th_hi,
                                                           float th_acc, float th_open, uint32_t leaf_cap,
                                                           float4* __restrict__ part,
                                                           float* __restrict__ acc, float* __restrict__ pot,
                                                           uint32_t* __restrict__ st_int,
                                                           uint32_t* __restrict__ st_open,
                                                           unsigned long long* __restrict__ tot, uint32_t* d_status,
                                                           WalkKick wk, const uint64_t* __restrict__ skeys) {
    __shared__ uint2 s_stk[GW_WARPS][GW_GSTACK];  // sibling groups: (first child, mask)
    __shared__ __align__(16) float l_xy[GW_WARPS][2 * GW_LIST];
    __shared__ __align__(16) float l_zm[GW_WARPS][2 * GW_LIST];
    __shared__ __align__(16) uint32_t l_k[GW_WARPS][GW_LIST];
    __shared__ uint32_t q_node[GW_WARPS][GW_SLOW];
    __shared__ uint32_t q_mask[GW_WARPS][GW_SLOW];
    __shared__ float4 s_body[GW_WARPS][32];
    __shared__ float4 s_mg[GW_WARPS][32];     // a round's mixed cells: centre and w^2,
    __shared__ uint32_t s_mm[GW_WARPS][32];   // the bodies walking them,
    __shared__ uint32_t s_om[GW_WARPS][32];   // and the bodies that open them
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    float4* sbd = s_body[w];
    uint2* stk = s_stk[w];
    const GroupLists L{l_xy[w], l_zm[w], l_k[w], q_node[w], q_mask[w]};
    static_assert(GB == 32 || GB == 16 || GB == 8, "8-, 16- or 32-body groups");
    const uint32_t group = blockIdx.x * GW_WARPS + w;
    // body slot of the lane (both half-warps hold the same 16 bodies when GB = 16)
    const int bl = lane & (GB - 1), half = lane / GB;
    const uint32_t body_bits = GB == 32 ? 0xffffffffu : (1u << GB) - 1u;
    const uint32_t k = group * (uint32_t)GB + (uint32_t)bl;
    const bool live = k < n;
    const uint32_t live_mask = __ballot_sync(0xffffffffu, live) & body_bits;
    // with the fused kick every warp reaches the block reduction; a warp
    // past the last body walks nothing
    if (!live_mask && !KICK) return;
    const uint32_t kq = live ? k : min(group * (uint32_t)GB, n - 1u);
    const float4 b = sp[kq];
    const float rx = b.x, ry = b.y, rz = b.z, mi = b.w;
    if (half == 0) sbd[bl] = b;
    // The group is walked in parts: runs of its bodies that share the
    // octants of the top PART_LEVELS levels.  A group cut by such a cell
    // boundary (3 % of the 16-body groups of the uniform sphere, and those
    // of the sparse outskirts) would otherwise walk with a box spanning
    // both sides, find most cells mixed, and run several times as long as
    // the others (the longest warp sets the launch's duration).
    const uint32_t pfx = (uint32_t)(skeys[kq] >> (3 * (16 - PART_LEVELS)));
    const uint32_t pprev = __shfl_up_sync(0xffffffffu, pfx, 1);
    const uint32_t starts = __ballot_sync(0xffffffffu, live && (bl == 0 || pfx != pprev)) & body_bits;
    __syncwarp();
    float bx0 = rx, by0 = ry, bz0 = rz, bx1 = rx, by1 = ry, bz1 = rz;
    // bounding box of the part (lanes outside it repeat its first body)
    auto part_box = [&](uint32_t part, int s0) {
        const bool inp = (part >> bl) & 1u;
        const float4 r0 = sbd[s0];
        bx0 = bx1 = inp ? rx : r0.x;
        by0 = by1 = inp ? ry : r0.y;
        bz0 = bz1 = inp ? rz : r0.z;
        for (int o = 16; o > 0; o >>= 1) {
            bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
            by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
            bz0 = fminf(bz0, __shfl_xor_sync(0xffffffffu, bz0, o));
            bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
            by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
            bz1 = fmaxf(bz1, __shfl_xor_sync(0xffffffffu, bz1, o));
        }
    };
    KSum ax{0.f, 0.f}, ay{0.f, 0.f}, az{0.f, 0.f}, ph{0.f, 0.f};
    float2 a2x = make_float2(0.f, 0.f), a2y = a2x, a2z = a2x, p2 = a2x;
    uint32_t n_int = 0, n_open = 0;
    unsigned long long open_total = 0;
    int top = 0, count = 0, qcount = 0;
    auto flush = [&](bool all) {
        if (all || count > GW_LIST - 36) {
            // FAST: pad to a multiple of 2 (4 with two half-warps) with
            // entries no lane takes
            constexpr int PAD = KIND == WALK_COMP ? 1 : 2 * (32 / GB);
            const int padded = (count + PAD - 1) / PAD * PAD;
            if (lane < padded - count) {
                const int ix = lx_of(count + lane);
                L.xy[ix] = L.xy[ix + 2] = L.zm[ix] = L.zm[ix + 2] = 0.f;
                L.msk[count + lane] = 0u;
            }
            count = padded;
            __syncwarp();
            flush_fast<KIND, GB, STATS>(L, count, bl, half, rx, ry, rz, fc.eps2, a2x, a2y, a2z, p2, ax, ay, az, ph,
                                        n_int);
            count = 0;
            __syncwarp();
        }
        if (all || qcount > GW_SLOW - 32) {
            flush_slow<KIND, GB, STATS>(L, qcount, nd, bl, half, rx, ry, rz, mi, fc.eps2, ax, ay, az, ph, n_int);
            qcount = 0;
            __syncwarp();
        }
    };
    // The stack holds groups of 8 siblings (the children of an opened
    // cell: first child id, mask of the bodies that opened it); a round pops
    // up to 4 groups, lane l taking child l % 8 of group l / 8, so one push
    // per opened cell replaces eight.  The root is the first round's only
    // cell.  A round may push one group per lane: popping ng groups leaves
    // room when top + 7 ng <= GW_GSTACK.
    uint32_t guard = 0;
    uint32_t rest = live_mask;
    while (rest) {  // the group's parts, one walk each
    const int s0 = __ffs(rest) - 1;
    const uint32_t later = starts & ~((2u << s0) - 1u);  // part starts after s0
    const uint32_t part = rest & (later ? (1u << (__ffs(later) - 1)) - 1u : 0xffffffffu);
    rest &= ~part;
    part_box(part, s0);
    bool root_round = true;
    __syncwarp();
    while (root_round || top > 0) {
        if (++guard > fc.walk_limit) {
            if (lane == 0) atomicOr(d_status, SFGPU_STATUS_WALK);
            break;
        }
        uint32_t v = 0, M = 0;
        bool valid = false;
        if (root_round) {
            valid = lane == 0;
            M = part;
            root_round = false;
        } else {
            const int ng = min(4, min(top, (GW_GSTACK - top) / 7));
            if (ng == 0) {  // no room for children: cannot happen with GW_GSTACK >> 7 x depth x 4
                if (lane == 0) atomicOr(d_status, SFGPU_STATUS_WALK);
                break;
            }
            if ((lane >> 3) < ng) {
                const uint2 e = stk[top - 1 - (lane >> 3)];
                v = e.x + (uint32_t)(lane & 7);
                M = e.y;
                valid = true;
            }
            top -= ng;
            __syncwarp();
        }
        // 0 drop, 1 accept, 2 open, 3 mixed
        int kind = 0;
        bool internal = false;
        float4 G = make_float4(0.f, 0.f, 0.f, 0.f), H = G, C = G, Lo = G;
        uint32_t first = NODE_NONE;
        if (valid) {
            // the whole node record in one round trip (the monopole half is
            // needed by every accepted or mixed cell, most of the entries)
            H = __ldg(&nd.hi[NODE_REC * v]);
            G = __ldg(&nd.geo[NODE_REC * v]);
            C = __ldg(&nd.com[NODE_REC * v]);
            Lo = __ldg(&nd.lo[NODE_REC * v]);
            const uint32_t bodies = __float_as_uint(H.z);
            first = __float_as_uint(H.w);
            internal = bodies > leaf_cap;
            if (bodies == 0u) {
                kind = 0;
            } else if (bodies <= leaf_cap) {
                kind = 1;
            } else {
                open_total += __popc(M);
                // distances from the cell centre to the group's box (nearest, farthest)
                const float ex = fmaxf(0.f, fmaxf(bx0 - G.x, G.x - bx1));
                const float ey = fmaxf(0.f, fmaxf(by0 - G.y, G.y - by1));
                const float ez = fmaxf(0.f, fmaxf(bz0 - G.z, G.z - bz1));
                const float fx = fmaxf(fabsf(G.x - bx0), fabsf(G.x - bx1));
                const float fy = fmaxf(fabsf(G.y - by0), fabsf(G.y - by1));
                const float fz = fmaxf(fabsf(G.z - bz0), fabsf(G.z - bz1));
                const float dmin2 = (ex * ex + ey * ey + ez * ez) * (1.0f - 1.0f / 65536.0f);
                const float dmax2 = (fx * fx + fy * fy + fz * fz) * (1.0f + 1.0f / 65536.0f);
                if (dmin2 > 0.0f && G.w < th_acc * dmin2) kind = 1;
                else if (G.w >= th_open * dmax2 && first != NODE_NONE) kind = 2;
                else kind = 3;
            }
        }
        const uint32_t lt = (1u << lane) - 1u;
        // mixed cells: the reference's test for each (cell, body) pair of
        // the masks.  Either one lane per cell loops over its bodies, or the
        // warp goes through the cells one at a time with one lane per body,
        // whichever takes fewer rounds.
        const bool mixed = kind == 3 && first != NODE_NONE;
        const uint32_t mix_b = __ballot_sync(0xffffffffu, mixed);
        uint32_t om = 0u;
        if (mix_b) {
            constexpr int H = 32 / GB;  // sub-warps, each testing one cell per round
            const int rounds_cell = (__popc(mix_b) + H - 1) / H;
            const int rounds_body = __reduce_max_sync(0xffffffffu, mixed ? (uint32_t)__popc(M) : 0u);
            if (rounds_body <= rounds_cell) {
                if (mixed) {
                    uint32_t mm = M;
                    while (mm) {
                        const int i = __ffs(mm) - 1;
                        mm &= mm - 1u;
                        const float4 bi = sbd[i];
                        if (opens(G, bi.x, bi.y, bi.z, fc, th_lo, th_hi)) om |= 1u << i;
                    }
                }
            } else {
                // the mixed cells staged in shared memory in lane order;
                // sub-warp h tests cells j H + h and (j + 1) H + h in round
                // j / 2, one lane per body, the pair on paired FP32
                // instructions (walk 0.1022 -> 0.0985 ms at 65,536 bodies)
                const int nmix = __popc(mix_b);
                const int slot = __popc(mix_b & lt);
                if (mixed) {
                    s_mg[w][slot] = G;
                    s_mm[w][slot] = M;
                }
                __syncwarp();
                for (int j0 = 0; j0 < nmix; j0 += 2 * H) {  // two rounds at once, the same trip count on every lane
                    const int ja = j0 + half, jb = ja + H;
                    bool ta = false, tb = false;
                    if (ja < nmix) {
                        const bool inb = jb < nmix;
                        const float4 Ga = s_mg[w][ja], Gb = inb ? s_mg[w][jb] : Ga;
                        const uint32_t Ma = s_mm[w][ja], Mb = inb ? s_mm[w][jb] : 0u;
                        bool oa, ob;
                        opens2(make_float2(Ga.x, Gb.x), make_float2(Ga.y, Gb.y), make_float2(Ga.z, Gb.z),
                               make_float2(Ga.w, Gb.w), make_float2(rx, rx), make_float2(ry, ry), make_float2(rz, rz),
                               fc, th_lo, th_hi, oa, ob);
                        ta = ((Ma >> bl) & 1u) && oa;
                        tb = ((Mb >> bl) & 1u) && ob;
                    }
                    const uint32_t la = __ballot_sync(0xffffffffu, ta);
                    const uint32_t lb = __ballot_sync(0xffffffffu, tb);
                    if (bl == 0 && ja < nmix) s_om[w][ja] = (la >> (half * GB)) & body_bits;
                    if (bl == 0 && jb < nmix) s_om[w][jb] = (lb >> (half * GB)) & body_bits;
                }
                __syncwarp();
                if (mixed) om = s_om[w][slot];
            }
        }
        // accepted cells (all of the mask, or the bodies of a mixed cell
        // that do not open it) -> lists
        const uint32_t am = (kind == 1) ? M : ((kind == 3) ? (M & ~om) : 0u);
        append_cells(L, am, v, C, Lo, H, bx0, by0, bz0, bx1, by1, bz1, lane, count, qcount);
        if (!STATS) n_int += __popc(am);
        // children of the cells every body opens, and of the mixed cells
        // for the bodies that open them: one sibling group each
        const uint32_t pm = kind == 2 ? M : om;
        const uint32_t ob = __ballot_sync(0xffffffffu, pm != 0u);
        if (pm) stk[top + __popc(ob & lt)] = make_uint2(first, pm);
        top += __popc(ob);
        __syncwarp();
        if (STATS) {  // opening tests (internal cells only) attributed to bodies
            for (int l = 0; l < 32; l++) {
                const bool il = __shfl_sync(0xffffffffu, internal, l);
                const uint32_t ml = __shfl_sync(0xffffffffu, M, l);
                if (il && half == 0 && ((ml >> bl) & 1u)) n_open++;
            }
        }
        flush(false);
    }
    flush(true);
    }  // next part
    float sx = ax.s, sy = ay.s, sz = az.s, sw = ph.s;
    if (KIND == WALK_COMP) {
        sx -= ax.c;
        sy -= ay.c;
        sz -= az.c;
        sw -= ph.c;
    } else {
        sx += a2x.x + a2x.y;
        sy += a2y.x + a2y.y;
        sz += a2z.x + a2z.y;
        sw += p2.x + p2.y;
    }
    uint32_t n_int_body = n_int;
#pragma unroll
    for (int o = 16; o >= GB; o >>= 1) {  // the sub-warps' shares of the same bodies
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
        n_int_body += __shfl_xor_sync(0xffffffffu, n_int_body, o);
    }
    ff e[4] = {ff{0.f, 0.f}, ff{0.f, 0.f}, ff{0.f, 0.f}, ff{0.f, 0.f}};
    if (live && half == 0) {
        const uint32_t p = V[k];
        {
            const float g = -fc.neg_g;
            const float scale = fc.physical ? g : g * mi;
            const float a[3] = {scale * sx, scale * sy, scale * sz};
            acc[3u * p + 0u] = a[0];
            acc[3u * p + 1u] = a[1];
            acc[3u * p + 2u] = a[2];
            pot[p] = fc.neg_g * sw;
            if (KICK) walk_kick_body(wk, p, mi, a, fc.neg_g * sw, e);
            if (STATS) {
                st_int[p] = n_int_body;
                st_open[p] = n_open;
            }
        }
    }
    unsigned long long ci = n_int;
    for (int o = 16; o > 0; o >>= 1) {
        ci += __shfl_xor_sync(0xffffffffu, ci, o);
        open_total += __shfl_xor_sync(0xffffffffu, open_total, o);
    }
    if (lane == 0) {
        atomicAdd(&tot[0], ci);
        atomicAdd(&tot[1], open_total);
    }
    if (KICK) walk_kick_reduce(wk, e);
}

template <int KIND, int GSPLIT, int GB = 32>
int launch_group(sfgpu_sim* s, bool stats) {
    TreeWork* t = s->tree;
    const ForceConsts fc = sf_force_consts(s->p);
    const float th_lo = fc.theta * (1.0f - 1.0f / 524288.0f);
    const float th_hi = fc.theta * (1.0f + 1.0f / 524288.0f);
    const float th_acc = fc.theta * (1.0f - 1.0f / 4096.0f);
    const float th_open = fc.theta * (1.0f + 1.0f / 4096.0f);
    const uint32_t grid = sf_ceil_div((uint64_t)sf_ceil_div(s->n, GB) * GSPLIT, GW_WARPS);
    float* acc = s->slab + (size_t)6 * s->n;
    float* pot = s->slab + (size_t)10 * s->n;
    if (stats) {
        if (GSPLIT > 1) {
            SF_CUDA(cudaMemsetAsync(s->stat_int, 0, sizeof(uint32_t) * s->n, s->stream));
            SF_CUDA(cudaMemsetAsync(s->stat_open, 0, sizeof(uint32_t) * s->n, s->stream));
        }
        k_walk_group<KIND, GSPLIT, GB, true><<<grid, GW_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, th_acc, th_open, s->p.leaf_cap, t->walk_part, acc, pot,
            s->stat_int, s->stat_open, s->walk_tot, s->d_status, WalkKick{});
    } else if (GSPLIT == 1 && s->fuse_kick && s->red_cap * 2u >= grid * 4u) {
        WalkKick wk;
        wk.vel = s->slab + (size_t)3 * s->n;
        wk.ken = s->slab + (size_t)11 * s->n;
        wk.pen = s->slab + (size_t)12 * s->n;
        wk.vel64 = s->vel64;
        wk.dt64 = s->p.dt;
        wk.half_dt = 0.5f * (float)s->p.dt;
        wk.g_over_eps = (float)(s->p.G / s->p.eps);
        wk.physical = s->p.acc_mode == SFGPU_ACC_PHYSICAL;
        wk.part = (double*)s->red;
        wk.done = s->d_done + 1;
        wk.sums = s->sums;
        wk.d_step = s->d_step;
        k_walk_group<KIND, GSPLIT, GB, false, true><<<grid, GW_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, th_acc, th_open, s->p.leaf_cap, t->walk_part, acc, pot,
            nullptr, nullptr, s->walk_tot, s->d_status, wk);
        s->kicked = true;
    } else {
        k_walk_group<KIND, GSPLIT, GB, false><<<grid, GW_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, th_acc, th_open, s->p.leaf_cap, t->walk_part, acc, pot,
            nullptr, nullptr, s->walk_tot, s->d_status, WalkKick{});
    }
    SF_CHECK_LAUNCH();
    if (GSPLIT > 1) {
        k_walk_reduce<KIND><<<sf_ceil_div(s->n, 256), 256, 0, s->stream>>>(t->walk_part, t->sp, t->vals, s->n, fc,
                                                                           acc, pot);
        SF_CHECK_LAUNCH();
    }
    return SFGPU_OK;
}

template <int KIND, int GB>
int launch_sib(sfgpu_sim* s, bool stats) {
    TreeWork* t = s->tree;
    const ForceConsts fc = sf_force_consts(s->p);
    const float th_lo = fc.theta * (1.0f - 1.0f / 524288.0f);
    const float th_hi = fc.theta * (1.0f + 1.0f / 524288.0f);
    const float th_acc = fc.theta * (1.0f - 1.0f / 4096.0f);
    const float th_open = fc.theta * (1.0f + 1.0f / 4096.0f);
    const uint32_t grid = sf_ceil_div((uint64_t)sf_ceil_div(s->n, GB), GW_WARPS);
    float* acc = s->slab + (size_t)6 * s->n;
    float* pot = s->slab + (size_t)10 * s->n;
    if (stats) {
        k_walk_sib<KIND, GB, true><<<grid, GW_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, th_acc, th_open, s->p.leaf_cap, t->walk_part, acc, pot,
            s->stat_int, s->stat_open, s->walk_tot, s->d_status, WalkKick{}, t->keys);
    } else if (s->fuse_kick && s->red_cap * 2u >= grid * 4u) {
        WalkKick wk;
        wk.vel = s->slab + (size_t)3 * s->n;
        wk.ken = s->slab + (size_t)11 * s->n;
        wk.pen = s->slab + (size_t)12 * s->n;
        wk.vel64 = s->vel64;
        wk.dt64 = s->p.dt;
        wk.half_dt = 0.5f * (float)s->p.dt;
        wk.g_over_eps = (float)(s->p.G / s->p.eps);
        wk.physical = s->p.acc_mode == SFGPU_ACC_PHYSICAL;
        wk.part = (double*)s->red;
        wk.done = s->d_done + 1;
        wk.sums = s->sums;
        wk.d_step = s->d_step;
        k_walk_sib<KIND, GB, false, true><<<grid, GW_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, th_acc, th_open, s->p.leaf_cap, t->walk_part, acc, pot,
            nullptr, nullptr, s->walk_tot, s->d_status, wk, t->keys);
        s->kicked = true;
    } else {
        k_walk_sib<KIND, GB, false><<<grid, GW_THREADS, 0, s->stream>>>(
            t->sp, t->vals, s->n, t->nd, fc, th_lo, th_hi, th_acc, th_open, s->p.leaf_cap, t->walk_part, acc, pot,
            nullptr, nullptr, s->walk_tot, s->d_status, WalkKick{}, t->keys);
    }
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

template <int KIND>
int launch_fast(sfgpu_sim* s, bool stats) {
    // walk_split: 0 (default) group walk of walk_group bodies per warp (0 =
    // the default size, 8, 16 or 32) with a stack of sibling groups; 32 the
    // same walk with a stack of single cells; 1 one thread per body; 8 one
    // thread per body and root octant; 64 32-body group walk with the
    // level-2 frontier dealt over 8 warps per group.  The split variants pay
    // for their redundant top levels and imbalance more than they gain.
    const uint32_t split = s->p.walk_split;
    if (split == 1) return launch_body<KIND, 1>(s, stats);
    if (split == 8) return launch_body<KIND, SPLIT>(s, stats);
    if (split == 64) return launch_group<KIND, SPLIT>(s, stats);
    const uint32_t gb = s->p.walk_group ? s->p.walk_group : WALK_GROUP_DEFAULT;
    if (split == 32) {  // the group walk with a stack of single cells
        if (gb == 8) return launch_group<KIND, 1, 8>(s, stats);
        if (gb == 16) return launch_group<KIND, 1, 16>(s, stats);
        return launch_group<KIND, 1, 32>(s, stats);
    }
    if (gb == 8) return launch_sib<KIND, 8>(s, stats);
    if (gb == 16) return launch_sib<KIND, 16>(s, stats);
    return launch_sib<KIND, 32>(s, stats);
}

__device__ __forceinline__ uint32_t chk_mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
// n random cases of a body and two cells whose w^2 lies within 3 ulps of
// theta d^2 (so the IEEE-divide fallback decides many of them): opens2, as
// the walk pairs cells, against opens, mismatches counted in *bad.
__global__ void k_opens2_check(uint32_t n, uint32_t seed, float theta, float th_lo, float th_hi,
                               unsigned long long* bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto u = [&](uint32_t k) {
        return (float)(chk_mix(seed * 0x9E3779B9u ^ chk_mix(16u * i + k)) >> 8) * (1.0f / 16777216.0f);
    };
    ForceConsts fc{};
    fc.theta = theta;
    const float rx = fsub(fmul(2.0f, u(0)), 1.0f), ry = fsub(fmul(2.0f, u(1)), 1.0f), rz = fsub(fmul(2.0f, u(2)), 1.0f);
    float4 G[2];
    bool want[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
        const float gx = fsub(fmul(2.0f, u(3 + 4 * c)), 1.0f), gy = fsub(fmul(2.0f, u(4 + 4 * c)), 1.0f);
        const float gz = fsub(fmul(2.0f, u(5 + 4 * c)), 1.0f);
        const float ox = fsub(gx, rx), oy = fsub(gy, ry), oz = fsub(gz, rz);
        const float d2 = fadd(fadd(fmul(ox, ox), fmul(oy, oy)), fmul(oz, oz));
        const int k = (int)(chk_mix(seed ^ (0x51ED27u * (2u * i + (uint32_t)c))) % 7u) - 3;
        G[c] = make_float4(gx, gy, gz, __int_as_float(__float_as_int(fmul(theta, d2)) + k));
        want[c] = opens(G[c], rx, ry, rz, fc, th_lo, th_hi);
    }
    bool g0, g1;
    opens2(make_float2(G[0].x, G[1].x), make_float2(G[0].y, G[1].y), make_float2(G[0].z, G[1].z),
           make_float2(G[0].w, G[1].w), make_float2(rx, rx), make_float2(ry, ry), make_float2(rz, rz), fc, th_lo,
           th_hi, g0, g1);
    if (g0 != want[0] || g1 != want[1]) atomicAdd(bad, 1ull);
}

}  // namespace

size_t sf_walk_scratch_floats4(uint32_t n) { return (size_t)SPLIT * n; }

int sf_sph_neighbours2_check(uint32_t n, uint32_t seed, unsigned long long* d_bad, cudaStream_t st);

// Check of the paired FP32 decisions (no counterpart in the reference): the
// walk's opening test for two cells and the SPH density pass's neighbour test
// for two candidates, against their scalar forms on n random cases around
// the decision boundaries.  mismatches[0] walk, [1] SPH.
extern "C" int sfgpu_paired_check(uint32_t n, uint32_t seed, uint64_t* mismatches) {
    sf_clear_error();
    if (!mismatches || n == 0u) {
        sf_set_error("sfgpu_paired_check needs n > 0 and an output array");
        return SFGPU_FAILURE;
    }
    unsigned long long* d = nullptr;
    SF_CUDA(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
    cudaError_t e = cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    const float theta = 0.5f;
    const float th_lo = theta * (1.0f - 1.0f / 524288.0f), th_hi = theta * (1.0f + 1.0f / 524288.0f);
    if (e == cudaSuccess) {
        k_opens2_check<<<sf_ceil_div(n, 256), 256>>>(n, seed, theta, th_lo, th_hi, d);
        e = cudaGetLastError();
    }
    int rc = e == cudaSuccess ? sf_sph_neighbours2_check(n, seed, d + 1, 0) : SFGPU_FAILURE;
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        sf_set_error("sfgpu_paired_check: %s", cudaGetErrorString(e));
        return SFGPU_FAILURE;
    }
    mismatches[0] = h[0];
    mismatches[1] = h[1];
    return rc;
}

int sf_walk_launch(sfgpu_sim* s) {
    const bool stats = (s->p.flags & SFGPU_FLAG_STATS) && s->stat_int;
    if (s->p.math == SFGPU_MATH_EXACT && s->p.form == SFGPU_FORM_PLAIN) return launch_kind<WALK_EXACT>(s, stats);
    if (s->p.form == SFGPU_FORM_COMPENSATED) return launch_fast<WALK_COMP>(s, stats);
    return launch_fast<WALK_FAST>(s, stats);
}
