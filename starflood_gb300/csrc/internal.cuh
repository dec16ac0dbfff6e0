// internal.cuh -- shared declarations of the starflood_gb300 CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "sfgpu.h"

// ---------------------------------------------------------------------------
// error handling
// ---------------------------------------------------------------------------
void sf_set_error(const char* fmt, ...);
void sf_clear_error();

#define SF_CUDA(call)                                                               \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            sf_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call,                \
                         cudaGetErrorString(e_));                                   \
            return SFGPU_FAILURE;                                                   \
        }                                                                           \
    } while (0)

extern unsigned long long g_sf_launches;
#define SF_CHECK_LAUNCH()                                                           \
    do {                                                                            \
        __atomic_add_fetch(&g_sf_launches, 1ull, __ATOMIC_RELAXED);                 \
        cudaError_t e_ = cudaGetLastError();                                        \
        if (e_ != cudaSuccess) {                                                    \
            sf_set_error("%s:%d: kernel launch: %s", __FILE__, __LINE__,            \
                         cudaGetErrorString(e_));                                   \
            return SFGPU_FAILURE;                                                   \
        }                                                                           \
    } while (0)

// ---------------------------------------------------------------------------
// device helpers: reference-order FP32 arithmetic (no contraction into FMA)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// One MUFU instruction each (flush-to-zero): the force kernels call them on
// r^2 + eps^2, which is positive and far above the subnormal range for any
// eps > 0.
__device__ __forceinline__ float rsqrt_hw(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_hw(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// One j (coordinates and mass duplicated into pairs) against a pair of
// bodies (negated coordinates nx, ny, nz) on the paired FP32 instructions:
// a += m_j d / (d^2 + eps^2)^1.5, phi += m_j / (d^2 + eps^2)^0.5 with
// d = r_j - r_i.  RSQ 0: rsqrtf, 1/r^2 = rsqrt^2; 1: MUFU rsqrt; 2: MUFU
// rsqrt and MUFU reciprocal (13 -> 12 FP32 operations per interaction).
template <int RSQ>
__device__ __forceinline__ void pp_pair_step(float2 sx, float2 sy, float2 sz, float2 sw, float2 nx, float2 ny,
                                             float2 nz, float2 e2, float2& ax, float2& ay, float2& az, float2& ph) {
    const float2 dx = __fadd2_rn(sx, nx);
    const float2 dy = __fadd2_rn(sy, ny);
    const float2 dz = __fadd2_rn(sz, nz);
    float2 r2 = __ffma2_rn(dz, dz, e2);
    r2 = __ffma2_rn(dy, dy, r2);
    r2 = __ffma2_rn(dx, dx, r2);
    float2 inv, inv2;
    if (RSQ == 0) {
        inv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
        inv2 = __fmul2_rn(inv, inv);
    } else if (RSQ == 1) {
        inv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
        inv2 = __fmul2_rn(inv, inv);
    } else {
        inv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
        inv2 = make_float2(rcp_hw(r2.x), rcp_hw(r2.y));
    }
    const float2 mphi = __fmul2_rn(sw, inv);
    const float2 f = __fmul2_rn(mphi, inv2);
    ax = __ffma2_rn(f, dx, ax);
    ay = __ffma2_rn(f, dy, ay);
    az = __ffma2_rn(f, dz, az);
    ph = __fadd2_rn(ph, mphi);
}

// Kahan running sum (the idiom of src/gravity.c:521-533).
struct KSum {
    float s, c;
    __device__ __forceinline__ void add(float x) {
        const float y = fsub(x, c);
        const float t = fadd(s, y);
        const float z = fsub(t, s);
        c = fsub(z, y);
        s = t;
    }
};

// 32-byte FP64 quadruple (x, y, z, w), one aligned 256-bit load.
struct __align__(32) sfd4 {
    double x, y, z, w;
};
__host__ __device__ __forceinline__ sfd4 mk_d4(double x, double y, double z, double w) {
    sfd4 r;
    r.x = x;
    r.y = y;
    r.z = z;
    r.w = w;
    return r;
}

// Error-free transformation a + b = s + e (Knuth's two-sum).
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = __dadd_rn(a, b);
    const double bp = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bp)), __dsub_rn(b, bp));
}
__device__ __forceinline__ void two_sumf(float a, float b, float& s, float& e) {
    s = fadd(a, b);
    const float bp = fsub(s, a);
    e = fadd(fsub(a, fsub(s, bp)), fsub(b, bp));
}
// Float-float numbers (hi + lo, about 48 significant bits) for sums that
// need more than FP32 but should not run on GB300's FP64 pipe, which issues
// about one FP64 operation per SM per cycle against 128 FP32.
struct ff {
    float hi, lo;
};
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    float s, e;
    two_sumf(a.hi, b.hi, s, e);
    e = fadd(e, fadd(a.lo, b.lo));
    const float h = fadd(s, e);  // fast two-sum: |s| >= |e|
    return ff{h, fsub(e, fsub(h, s))};
}
__device__ __forceinline__ ff ff_from(float v) { return ff{v, 0.0f}; }
__device__ __forceinline__ ff ff_from_double(double v) {
    const float h = (float)v;
    return ff{h, (float)(v - (double)h)};
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }
// x^2 exactly (two-product with one FMA)
__device__ __forceinline__ ff ff_sqr(float x) {
    const float p = fmul(x, x);
    return ff{p, __fmaf_rn(x, x, -p)};
}
// square root of a float-float to about 46 bits: one Newton correction of
// the FP32 root (the residual a - s^2 computed exactly with a two-product)
__device__ __forceinline__ ff ff_sqrt(ff a) {
    const float s = __fsqrt_rn(a.hi);
    if (!(s > 0.0f)) return ff{s, 0.0f};
    const float p = fmul(s, s), pe = __fmaf_rn(s, s, -p);
    const float res = fadd(fsub(fsub(a.hi, p), pe), a.lo);
    const float t = __fdiv_rn(res, fmul(2.0f, s));
    const float h = fadd(s, t);
    return ff{h, fsub(t, fsub(h, s))};
}
// warp sum (fixed order) of NV float-float values; lane 0 gets the totals
template <int NV>
__device__ __forceinline__ void ff_warp_sum(ff (&v)[NV]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < NV; k++) {
            const ff w{__shfl_down_sync(0xffffffffu, v[k].hi, o), __shfl_down_sync(0xffffffffu, v[k].lo, o)};
            v[k] = ff_add(v[k], w);
        }
}

// double-double accumulate (hi, lo) += (b_hi, b_lo)
__device__ __forceinline__ double2 dd_add(double2 a, double2 b) {
    double s, e;
    two_sum(a.x, b.x, s, e);
    e = __dadd_rn(e, __dadd_rn(a.y, b.y));
    double hi, lo;
    two_sum(s, e, hi, lo);
    return make_double2(hi, lo);
}

// The output function of splitmix64 (Steele, Lea and Flood, OOPSLA 2014): a
// bijective 64-bit mix.  Summed (mod 2^64) over the body indices of a
// neighbour set it identifies the set regardless of the order the bodies are
// found in, so two searches can be compared set for set.
__host__ __device__ __forceinline__ uint64_t sf_mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// rng.h:13-40 (pcg4d), used for the root-cube jitter.
__host__ __device__ __forceinline__ void pcg4d(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
    a = a * 1664525u + 1013904223u;
    b = b * 1664525u + 1013904223u;
    c = c * 1664525u + 1013904223u;
    d = d * 1664525u + 1013904223u;
    a += b * d; b += c * a; c += a * b; d += b * c;
    a ^= a >> 16; b ^= b >> 16; c ^= c >> 16; d ^= d >> 16;
    a += b * d; b += c * a; c += a * b; d += b * c;
}

// ---------------------------------------------------------------------------
// constants derived from parameters exactly as the reference derives them
// ---------------------------------------------------------------------------
struct ForceConsts {
    float eps2;    // (real)(EPSILON*EPSILON)           gravity.c:754
    float neg_g;   // (real)(-G)                        gravity.c:808
    float theta;   // (real)TREE_THETA                  gravity.c:448
    float third;   // (real)(1.0/3.0)                   gravity.c:370
    int physical;  // SFGPU_ACC_PHYSICAL
    uint32_t walk_limit;  // rounds of a warp's walk loop before SFGPU_STATUS_WALK
};
ForceConsts sf_force_consts(const sfgpu_params& p);

// ---------------------------------------------------------------------------
// stage timer (CUDA events on the simulation's stream)
// ---------------------------------------------------------------------------
struct StageTimer {
    struct Rec {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<std::string> names;
    std::vector<double> ms;
    std::vector<uint32_t> launches;
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    bool enabled = false;
    int begin(cudaStream_t st, const char* name);
    void end(cudaStream_t st, int token);
    void collect();
    ~StageTimer();
};

// ---------------------------------------------------------------------------
// radix sort of (u64 key, u32 value) pairs on the low `bits` key bits (sort.cu)
// ---------------------------------------------------------------------------
struct SortWork {
    uint64_t* keys_b = nullptr;
    uint32_t* vals_b = nullptr;
    uint32_t* hist = nullptr;      // [passes][128]
    uint32_t* status = nullptr;    // [tiles][128] lookback words
    uint32_t* counters = nullptr;  // [passes] tile tickets
    size_t cap = 0;
    size_t tiles_cap = 0;
    uint32_t flags = 0;            // SORT_NO_BUCKETS: always the tile passes
    uint32_t spin_limit = 1u << 24;  // look-back rounds on an unpublished word before SFGPU_STATUS_SPIN
    uint32_t withheld = 0xFFFFFFFFu; // failure-detection check only: this tile of the first tile pass
                                     // never publishes its look-back words (0xFFFFFFFF: none)
};
constexpr uint32_t SORT_NO_BUCKETS = 1u;
constexpr uint32_t SORT_PRECLEARED = 2u;  // one-shot: the caller's kernel cleared the words of sf_sort_clear_words
// The work words the small-array sort path needs cleared before a call,
// for a kernel the caller launches anyway (empty when n takes the tile
// passes); sets SORT_PRECLEARED for the next sort call.
struct SortClear {
    uint32_t* hist = nullptr;
    uint32_t nhist = 0;
    uint32_t* counters = nullptr;
    uint32_t ncounters = 0;
    uint32_t* status = nullptr;
    uint32_t nstatus = 0;
};
SortClear sf_sort_clear_words(SortWork& w, uint32_t n, int bits);
constexpr uint32_t BUCKET_SORT_MAX = 1u << 17;  // sf_sort_pairs* use one pass + per-bucket CTAs up to here
int sf_sort_alloc(SortWork& w, size_t n);
void sf_sort_free(SortWork& w);
// Sorts keys/vals in place (result back in keys/vals).  d_n (device, may be
// NULL) overrides n as the element count when non-NULL (n is then the
// capacity).  `enable` (device flag, may be NULL) skips the sort when zero.
// The number of passes is ceil(bits/7); an odd count costs one extra copy.
int sf_sort_pairs(uint64_t* keys, uint32_t* vals, uint32_t n, int bits, SortWork& w,
                  cudaStream_t st, uint32_t* d_status, const uint32_t* d_n = nullptr,
                  const uint32_t* enable = nullptr);
// The same without the final copy: the result is left in (*out_keys,
// *out_vals), which is (keys, vals) for up to BUCKET_SORT_MAX pairs, else
// (keys, vals) after an even number of passes and (w.keys_b, w.vals_b)
// after an odd one.
int sf_sort_pairs_keep(uint64_t* keys, uint32_t* vals, uint32_t n, int bits, SortWork& w, cudaStream_t st,
                       uint32_t* d_status, uint64_t** out_keys, uint32_t** out_vals,
                       const uint32_t* enable = nullptr);

// ---------------------------------------------------------------------------
// simulation state
// ---------------------------------------------------------------------------
struct TreeWork;  // tree.cu
int sf_tree_alloc(TreeWork** tw, uint32_t n, const sfgpu_params& p);
void sf_tree_free(TreeWork* tw);

struct sfgpu_sim {
    uint32_t n = 0, dof = 13;
    sfgpu_params p{};
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;        // a second stream for independent stages of a step
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_pos = nullptr, ev_pos_done = nullptr;  // early position copy of the host-step graph
    float* host_pos_out = nullptr;  // set while a step is captured for sfgpu_host_step
    float* slab = nullptr;         // N*dof, reference layout
    double* pos64 = nullptr;       // COMPENSATED: FP64 positions (3N)
    double* vel64 = nullptr;       // COMPENSATED: FP64 velocities (3N)
    float* u = nullptr;            // CUBIC SPH: specific internal energy
    float* dudt = nullptr;         // CUBIC SPH: du/dt
    // PP scratch
    float4* pp_part = nullptr;
    size_t pp_part_cap = 0;        // float4 entries
    // reductions
    double2* red = nullptr;        // block partials
    uint32_t red_cap = 0;
    double* sums = nullptr;        // [0]=T [1]=V [2]=Tcorr [3]=U [4]=mean radius ...
    uint32_t* d_status = nullptr;
    uint32_t* d_step = nullptr;
    uint32_t* d_done = nullptr;    // last-block tickets of the fused reductions
    float* d_bounds = nullptr;     // root cube (6 floats)
    TreeWork* tree = nullptr;
    void* sph = nullptr;           // SphWork (sph.cu)
    void* sph_cubic = nullptr;     // CubicWork (sph_cubic.cu)
    // pinned host mirrors
    uint32_t* h_step = nullptr;
    double* h_sums = nullptr;
    uint32_t* h_status = nullptr;
    // per-particle walk counters (optional)
    uint32_t* stat_int = nullptr;
    uint32_t* stat_open = nullptr;
    unsigned long long* walk_tot = nullptr;  // [2]
    StageTimer timer;
    cudaGraphExec_t graph = nullptr;
    cudaGraphExec_t host_graph = nullptr;  // sfgpu_host_step: copies in, step, copies out
    const float* host_graph_slab = nullptr;
    int host_graph_solve = -1;
    bool host_graph_ok = true;
    uint32_t* h_step_in = nullptr;     // page-locked: the step number the host-step graph reads
    bool graph_ok = true;
    bool fuse_kick = false;        // set by a step: the walk may do kick_1 and the energies
    bool kicked = false;           // ... and did
    struct SnapshotWriter* snap = nullptr;  // snapshot.cu
    void* vis = nullptr;                    // VisScratch (vis.cu)
};
void sf_snapshot_free(sfgpu_sim* s);
int sf_refresh_fp64(sfgpu_sim* s);  // FP64 state (COMPENSATED) from the FP32 slab
void sf_vis_free(sfgpu_sim* s);

// stage entry points (each queues kernels on s->stream)
int sf_stage_gravity_pp(sfgpu_sim* s);
int sf_stage_tree_solve(sfgpu_sim* s, bool radius_ready);
int sf_stage_sph(sfgpu_sim* s);
int sf_stage_kick_drift(sfgpu_sim* s, bool want_radius);
int sf_stage_radius(sfgpu_sim* s);
int sf_stage_kick_energy(sfgpu_sim* s);
int sf_stage_momentum(sfgpu_sim* s);
int sf_sph_alloc(sfgpu_sim* s);
void sf_sph_free(sfgpu_sim* s);

// scratch (float4 entries) the PP launch needs for n bodies (pp.cu)
size_t sf_pp_scratch_need(const sfgpu_params& p, uint32_t n);
// the PP force on arbitrary device arrays (pp.cu)
int sf_pp_launch(const sfgpu_params& p, uint32_t n, const float* pos, const float* mas,
                 float* acc, float* pot, float4** part, size_t* part_cap, cudaStream_t st,
                 const double* pos64);

// tree inspection (tree.cu)
int sf_tree_keys(sfgpu_sim* s, uint64_t* keys, uint32_t* index, uint32_t* n_inside);
int sf_tree_num_nodes(sfgpu_sim* s, uint32_t* num_nodes);
int sf_tree_export(sfgpu_sim* s, uint32_t* parent, uint32_t* bodies, uint32_t* branch8,
                   float* bounds6, float* params4);

static inline uint32_t sf_ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }
int sf_num_sms();

#define SF_RED_BLOCK 256
