// scan.cu -- deterministic exclusive prefix sums (reduce, scan partials,
// downsweep).  Fixed association order, so results are reproducible.
#include "internal.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

template <typename T> struct Add;
template <> struct Add<uint32_t> {
    __device__ static uint32_t zero() { return 0u; }
    __device__ static uint32_t op(uint32_t a, uint32_t b) { return a + b; }
    __device__ static uint32_t shfl_up(uint32_t v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
    __device__ static uint32_t shfl(uint32_t v, int l) { return __shfl_sync(0xffffffffu, v, l); }
};
template <> struct Add<sfd4> {
    __device__ static sfd4 zero() { return mk_d4(0, 0, 0, 0); }
    __device__ static sfd4 op(sfd4 a, sfd4 b) {
        return mk_d4(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z),
                            __dadd_rn(a.w, b.w));
    }
    __device__ static sfd4 shfl_up(sfd4 v, int o) {
        return mk_d4(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o),
                     __shfl_up_sync(0xffffffffu, v.z, o), __shfl_up_sync(0xffffffffu, v.w, o));
    }
    __device__ static sfd4 shfl(sfd4 v, int l) {
        return mk_d4(__shfl_sync(0xffffffffu, v.x, l), __shfl_sync(0xffffffffu, v.y, l),
                     __shfl_sync(0xffffffffu, v.z, l), __shfl_sync(0xffffffffu, v.w, l));
    }
};

// Inclusive scan of one value per lane (Kogge-Stone by shuffles; the order of
// additions is fixed by lane index).
template <typename T>
__device__ __forceinline__ T warp_inclusive(T x, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = Add<T>::shfl_up(x, o);
        if (lane >= o) x = Add<T>::op(y, x);
    }
    return x;
}

// Block-wide exclusive scan of one value per thread: warp scans, then one
// warp scans the warp totals (fixed order).  sh holds >= 32 values.
template <typename T>
__device__ T block_exclusive(T v, T* sh, T& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const T incl = warp_inclusive<T>(v, lane);
    T excl = Add<T>::shfl_up(incl, 1);
    if (lane == 0) excl = Add<T>::zero();
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const T w = lane < nw ? sh[lane] : Add<T>::zero();
        const T wi = warp_inclusive<T>(w, lane);
        T we = Add<T>::shfl_up(wi, 1);
        if (lane == 0) we = Add<T>::zero();
        if (lane < nw) sh[lane] = we;
        if (lane == 31) sh[32] = wi;  // block total
    }
    __syncthreads();
    total = sh[32];
    const T r = Add<T>::op(sh[warp], excl);
    __syncthreads();
    return r;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_reduce(const T* __restrict__ in, uint32_t n,
                                                         T* __restrict__ partials) {
    __shared__ T sh[33];
    const size_t base = (size_t)blockIdx.x * SCAN_CHUNK + (size_t)threadIdx.x * SCAN_ITEMS;
    T acc = Add<T>::zero();
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < n) acc = Add<T>::op(acc, in[base + k]);
    T total;
    block_exclusive<T>(acc, sh, total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_partials(T* partials, uint32_t nb, T* total_out) {
    __shared__ T sh[33];
    T carry = Add<T>::zero();
    for (uint32_t b0 = 0; b0 < nb; b0 += SCAN_THREADS) {
        const uint32_t i = b0 + threadIdx.x;
        T v = i < nb ? partials[i] : Add<T>::zero();
        T tot;
        T ex = block_exclusive<T>(v, sh, tot);
        if (i < nb) partials[i] = Add<T>::op(carry, ex);
        carry = Add<T>::op(carry, tot);
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_downsweep(const T* __restrict__ in, T* out, uint32_t n,
                                                            const T* __restrict__ partials) {
    __shared__ T sh[33];
    const size_t base = (size_t)blockIdx.x * SCAN_CHUNK + (size_t)threadIdx.x * SCAN_ITEMS;
    T v[SCAN_ITEMS];
    T acc = Add<T>::zero();
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = (base + k < n) ? in[base + k] : Add<T>::zero();
        acc = Add<T>::op(acc, v[k]);
    }
    T tot;
    T ex = block_exclusive<T>(acc, sh, tot);
    T run = Add<T>::op(partials[blockIdx.x], ex);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = run;
        run = Add<T>::op(run, v[k]);
    }
}

template <typename T>
int scan_impl(const T* in, T* out, uint32_t n, T* d_total, ScanWork& w, cudaStream_t st) {
    const uint32_t nb = sf_ceil_div(n ? n : 1, SCAN_CHUNK);
    const size_t need = (size_t)nb * sizeof(T);
    if (w.cap_blocks < need) {
        sf_set_error("scan: work space not reserved");
        return SFGPU_FAILURE;
    }
    T* part = (T*)w.partials;
    k_reduce<T><<<nb, SCAN_THREADS, 0, st>>>(in, n, part);
    SF_CHECK_LAUNCH();
    k_scan_partials<T><<<1, SCAN_THREADS, 0, st>>>(part, nb, d_total);
    SF_CHECK_LAUNCH();
    k_downsweep<T><<<nb, SCAN_THREADS, 0, st>>>(in, out, n, part);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

}  // namespace

int sf_scan_reserve(ScanWork& w, uint32_t n, size_t elem) {
    const uint32_t nb = sf_ceil_div(n ? n : 1, SCAN_CHUNK);
    const size_t need = (size_t)nb * elem;
    if (w.cap_blocks >= need) return SFGPU_OK;
    if (w.partials) cudaFree(w.partials);
    w.partials = nullptr;
    SF_CUDA(cudaMalloc(&w.partials, need));
    w.cap_blocks = need;
    return SFGPU_OK;
}

int sf_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* d_total, ScanWork& w,
                cudaStream_t st, const uint32_t*) {
    return scan_impl<uint32_t>(in, out, n, d_total, w, st);
}


