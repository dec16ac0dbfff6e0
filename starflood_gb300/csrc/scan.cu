// scan.cu -- deterministic exclusive prefix sums (reduce, scan partials,
// downsweep).  Fixed association order, so results are reproducible.
#include "internal.cuh"

namespace {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

template <typename T> struct Add;
template <> struct Add<uint32_t> {
    __device__ static uint32_t zero() { return 0u; }
    __device__ static uint32_t op(uint32_t a, uint32_t b) { return a + b; }
};
template <> struct Add<sfd4> {
    __device__ static sfd4 zero() { return mk_d4(0, 0, 0, 0); }
    __device__ static sfd4 op(sfd4 a, sfd4 b) {
        return mk_d4(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z),
                            __dadd_rn(a.w, b.w));
    }
};

// Block-wide exclusive scan of one value per thread (Hillis-Steele in shared
// memory; order of additions fixed by thread index).
template <typename T>
__device__ T block_exclusive(T v, T* sh, T& total) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        T add = (t >= off) ? sh[t - off] : Add<T>::zero();
        __syncthreads();
        if (t >= off) sh[t] = Add<T>::op(add, sh[t]);
        __syncthreads();
    }
    T incl = sh[t];
    total = sh[blockDim.x - 1];
    __syncthreads();
    T excl = (t == 0) ? Add<T>::zero() : sh[t - 1];
    __syncthreads();
    (void)incl;
    return excl;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_reduce(const T* __restrict__ in, uint32_t n,
                                                         T* __restrict__ partials) {
    __shared__ T sh[SCAN_THREADS];
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
    __shared__ T sh[SCAN_THREADS];
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
    __shared__ T sh[SCAN_THREADS];
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

int sf_scan_d4(const sfd4* in, sfd4* out, uint32_t n, ScanWork& w, cudaStream_t st,
               const uint32_t*) {
    return scan_impl<sfd4>(in, out, n, out + n, w, st);
}
