// context.cu -- resident simulations (sfgpu_sim): allocation, host transfers,
// the sim_solv / sim_step sequences, CUDA-graph replay of whole steps,
// energies, status word, stage timers.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include "internal.cuh"
#include "tree.cuh"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[1024] = "";
unsigned long long g_sf_launches = 0;

extern "C" unsigned long long sfgpu_kernel_launches(void) { return __atomic_load_n(&g_sf_launches, __ATOMIC_RELAXED); }

extern "C" int sfgpu_host_register(void* ptr, size_t bytes) {
    sf_clear_error();
    SF_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    return SFGPU_OK;
}

extern "C" int sfgpu_host_unregister(void* ptr) {
    sf_clear_error();
    SF_CUDA(cudaHostUnregister(ptr));
    return SFGPU_OK;
}

extern "C" int sfgpu_flush_l2(void* stream) {
    // overwrite a buffer larger than the 129 MB L2 so the next kernel starts cold
    static void* buf = nullptr;
    const size_t bytes = (size_t)256 << 20;
    sf_clear_error();
    if (!buf) SF_CUDA(cudaMalloc(&buf, bytes));
    SF_CUDA(cudaMemsetAsync(buf, (int)(g_sf_launches & 0xff), bytes, (cudaStream_t)stream));
    return SFGPU_OK;
}

void sf_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}
void sf_clear_error() { g_err[0] = 0; }

extern "C" const char* sfgpu_last_error(void) { return g_err; }

int sf_num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    }
    return sms;
}

// ---------------------------------------------------------------------------
// stage timer
// ---------------------------------------------------------------------------
int StageTimer::begin(cudaStream_t st, const char* name) {
    if (!enabled) return -1;
    int idx = -1;
    for (size_t i = 0; i < names.size(); i++)
        if (names[i] == name) idx = (int)i;
    if (idx < 0) {
        names.emplace_back(name);
        ms.push_back(0.0);
        launches.push_back(0);
        idx = (int)names.size() - 1;
    }
    Rec r;
    r.stage = idx;
    for (int k = 0; k < 2; k++) {
        cudaEvent_t e;
        if (!pool.empty()) {
            e = pool.back();
            pool.pop_back();
        } else if (cudaEventCreate(&e) != cudaSuccess) {
            return -1;
        }
        (k == 0 ? r.a : r.b) = e;
    }
    cudaEventRecord(r.a, st);
    pending.push_back(r);
    return (int)pending.size() - 1;
}

void StageTimer::end(cudaStream_t st, int token) {
    if (token < 0 || token >= (int)pending.size()) return;
    cudaEventRecord(pending[token].b, st);
}

void StageTimer::collect() {
    for (auto& r : pending) {
        float t = 0.f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
            ms[r.stage] += t;
            launches[r.stage] += 1;
        }
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    pending.clear();
}

StageTimer::~StageTimer() {
    for (auto& r : pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
}

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------
extern "C" void sfgpu_params_default(sfgpu_params* p) {
    memset(p, 0, sizeof(*p));
    p->dt = 1.0;         // config.h TIMESTEP_SIZE 1.000e-0
    p->eps = 1.0e-3;     // config.h EPSILON 1.000e-3
    p->G = 1.0;          // config.h G 1.000
    p->theta = 0.5;      // config.h TREE_THETA 0.5
    p->solver = SFGPU_SOLVER_TREE;
    p->sph = SFGPU_SPH_OFF;
    p->math = SFGPU_MATH_FAST;
    p->form = SFGPU_FORM_PLAIN;
    p->acc_mode = SFGPU_ACC_REFERENCE;
    p->leaf_cap = 8;
    p->depth_max = 16;
    p->nodes_max = 262144;
    p->sph_gamma = 5.0 / 3.0;
    p->sph_alpha = 1.0;
    p->sph_beta = 2.0;
}

extern "C" uint32_t sfgpu_dof(const sfgpu_params* p) { return p && p->sph != SFGPU_SPH_OFF ? 16u : 13u; }

static int validate(const sfgpu_params* p) {
    if (!p) {
        sf_set_error("params is NULL");
        return SFGPU_FAILURE;
    }
    if (!(p->eps > 0.0)) {
        sf_set_error("eps must be > 0 (the softened branch of gravity.c:753 is the one implemented)");
        return SFGPU_FAILURE;
    }
    if (p->leaf_cap < 1 || p->leaf_cap > 16) {
        sf_set_error("leaf_cap must be in [1, 16]");
        return SFGPU_FAILURE;
    }
    if (p->depth_max < 1 || p->depth_max > 16) {
        sf_set_error("depth_max must be in [1, 16]");
        return SFGPU_FAILURE;
    }
    if (p->solver == SFGPU_SOLVER_TREE && p->nodes_max < 9) {
        sf_set_error("nodes_max must be >= 9");
        return SFGPU_FAILURE;
    }
    if (p->solver != SFGPU_SOLVER_PP && p->solver != SFGPU_SOLVER_TREE) {
        sf_set_error("unknown solver %d", p->solver);
        return SFGPU_FAILURE;
    }
    if (p->sph < SFGPU_SPH_OFF || p->sph > SFGPU_SPH_CUBIC) {
        sf_set_error("unknown sph mode %d", p->sph);
        return SFGPU_FAILURE;
    }
    if (p->walk_group != 0 && p->walk_group != 8 && p->walk_group != 16 && p->walk_group != 32) {
        sf_set_error("walk_group must be 0, 8, 16 or 32");
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

// ---------------------------------------------------------------------------
// lifetime
// ---------------------------------------------------------------------------
extern "C" int sfgpu_destroy(sfgpu_sim* s) {
    if (!s) return SFGPU_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    sf_snapshot_free(s);
    sf_vis_free(s);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->host_graph) cudaGraphExecDestroy(s->host_graph);
    cudaFreeHost(s->h_step_in);
    sf_tree_free(s->tree);
    sf_sph_free(s);
    cudaFree(s->slab);
    cudaFree(s->pos64);
    cudaFree(s->vel64);
    cudaFree(s->u);
    cudaFree(s->dudt);
    cudaFree(s->pp_part);
    cudaFree(s->red);
    cudaFree(s->sums);
    cudaFree(s->d_status);
    cudaFree(s->d_step);
    cudaFree(s->d_done);
    cudaFree(s->d_bounds);
    cudaFree(s->stat_int);
    cudaFree(s->stat_open);
    cudaFree(s->walk_tot);
    cudaFreeHost(s->h_step);
    cudaFreeHost(s->h_sums);
    cudaFreeHost(s->h_status);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->ev_pos) cudaEventDestroy(s->ev_pos);
    if (s->ev_pos_done) cudaEventDestroy(s->ev_pos_done);
    if (s->aux) cudaStreamDestroy(s->aux);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SFGPU_OK;
}

extern "C" int sfgpu_create(sfgpu_sim** out, uint32_t n, const sfgpu_params* p) {
    sf_clear_error();
    if (!out) {
        sf_set_error("out is NULL");
        return SFGPU_FAILURE;
    }
    *out = nullptr;
    if (validate(p) != SFGPU_OK) return SFGPU_FAILURE;
    if (n == 0) {
        sf_set_error("N must be > 0");
        return SFGPU_FAILURE;
    }
    sfgpu_sim* s = new sfgpu_sim();
    s->n = n;
    s->p = *p;
    s->dof = sfgpu_dof(p);
    s->timer.enabled = (p->flags & SFGPU_FLAG_TIMING) != 0;
    auto fail = [&]() {
        sfgpu_destroy(s);
        return SFGPU_FAILURE;
    };
#define TRY(call)                                                                           \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            sf_set_error("sfgpu_create: %s: %s", #call, cudaGetErrorString(e_));            \
            return fail();                                                                  \
        }                                                                                   \
    } while (0)
    TRY(cudaGetDevice(&s->device));
    TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    TRY(cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking));
    TRY(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
    TRY(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
    TRY(cudaEventCreateWithFlags(&s->ev_pos, cudaEventDisableTiming));
    TRY(cudaEventCreateWithFlags(&s->ev_pos_done, cudaEventDisableTiming));
    const size_t slab_bytes = sizeof(float) * (size_t)n * s->dof;
    TRY(cudaMalloc(&s->slab, slab_bytes));
    TRY(cudaMemsetAsync(s->slab, 0, slab_bytes, s->stream));  // simulation.c:118
    if (p->form == SFGPU_FORM_COMPENSATED) {
        TRY(cudaMalloc(&s->pos64, sizeof(double) * 3 * (size_t)n));
        TRY(cudaMalloc(&s->vel64, sizeof(double) * 3 * (size_t)n));
        TRY(cudaMemsetAsync(s->pos64, 0, sizeof(double) * 3 * (size_t)n, s->stream));
        TRY(cudaMemsetAsync(s->vel64, 0, sizeof(double) * 3 * (size_t)n, s->stream));
    }
    TRY(cudaMalloc(&s->sums, sizeof(double) * 16));
    TRY(cudaMemsetAsync(s->sums, 0, sizeof(double) * 16, s->stream));
    TRY(cudaMalloc(&s->d_status, sizeof(uint32_t)));
    TRY(cudaMemsetAsync(s->d_status, 0, sizeof(uint32_t), s->stream));
    TRY(cudaMalloc(&s->d_done, sizeof(uint32_t) * 4));
    TRY(cudaMemsetAsync(s->d_done, 0, sizeof(uint32_t) * 4, s->stream));
    TRY(cudaMalloc(&s->d_step, sizeof(uint32_t)));
    TRY(cudaMemsetAsync(s->d_step, 0, sizeof(uint32_t), s->stream));
    TRY(cudaMalloc(&s->d_bounds, sizeof(float) * 8));
    TRY(cudaMemsetAsync(s->d_bounds, 0, sizeof(float) * 8, s->stream));
    TRY(cudaMalloc(&s->walk_tot, sizeof(unsigned long long) * 2));
    TRY(cudaMemsetAsync(s->walk_tot, 0, sizeof(unsigned long long) * 2, s->stream));
    TRY(cudaMallocHost(&s->h_step, sizeof(uint32_t)));
    TRY(cudaMallocHost(&s->h_step_in, sizeof(uint32_t)));
    TRY(cudaMallocHost(&s->h_sums, sizeof(double) * 16));
    TRY(cudaMallocHost(&s->h_status, sizeof(uint32_t)));
    if (p->solver == SFGPU_SOLVER_TREE) {
        if (sf_tree_alloc(&s->tree, n, *p) != SFGPU_OK) return fail();
        if (p->flags & SFGPU_FLAG_STATS) {
            TRY(cudaMalloc(&s->stat_int, sizeof(uint32_t) * n));
            TRY(cudaMalloc(&s->stat_open, sizeof(uint32_t) * n));
        }
    }
    if (p->sph != SFGPU_SPH_OFF && sf_sph_alloc(s) != SFGPU_OK) return fail();
    // work space allocated up front, so steps can be captured into graphs
    if (p->solver == SFGPU_SOLVER_PP) {
        const size_t need = sf_pp_scratch_need(*p, n);
        if (need) {
            TRY(cudaMalloc(&s->pp_part, need * sizeof(float4)));
            s->pp_part_cap = need;
        }
    }
    // per-block partials: the KDK kernels (4 per 256 bodies) and the walk's
    // fused kick (4 per 16 bodies at the smallest group size)
    s->red_cap = 4 * sf_ceil_div(n, 16) + 8;
    TRY(cudaMalloc(&s->red, sizeof(double2) * s->red_cap));
    TRY(cudaStreamSynchronize(s->stream));
#undef TRY
    *out = s;
    return SFGPU_OK;
}

// ---------------------------------------------------------------------------
// host transfers
// ---------------------------------------------------------------------------
__global__ static void k_widen(const float* __restrict__ src, double* __restrict__ dst, size_t m) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

static int refresh_fp64(sfgpu_sim* s) {
    if (!s->pos64) return SFGPU_OK;
    const size_t m = 3 * (size_t)s->n;
    const uint32_t g = std::min<uint32_t>(sf_ceil_div(m, 256), 4096);
    k_widen<<<g, 256, 0, s->stream>>>(s->slab, s->pos64, m);
    k_widen<<<g, 256, 0, s->stream>>>(s->slab + m, s->vel64, m);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

int sf_refresh_fp64(sfgpu_sim* s) { return refresh_fp64(s); }

extern "C" int sfgpu_upload_arrays(sfgpu_sim* s, const float* slab, uint32_t first, uint32_t count) {
    sf_clear_error();
    if (!s || !slab || first + count > s->dof) {
        sf_set_error("sfgpu_upload_arrays: bad arguments");
        return SFGPU_FAILURE;
    }
    const size_t off = (size_t)first * s->n;
    SF_CUDA(cudaMemcpyAsync(s->slab + off, slab + off, sizeof(float) * (size_t)count * s->n,
                            cudaMemcpyHostToDevice, s->stream));
    if (first < 6) {
        if (refresh_fp64(s) != SFGPU_OK) return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    return SFGPU_OK;
}

extern "C" int sfgpu_upload(sfgpu_sim* s, const float* slab) {
    return sfgpu_upload_arrays(s, slab, 0, s ? s->dof : 0);
}

extern "C" int sfgpu_download_arrays(sfgpu_sim* s, float* slab, uint32_t first, uint32_t count) {
    sf_clear_error();
    if (!s || !slab || first + count > s->dof) {
        sf_set_error("sfgpu_download_arrays: bad arguments");
        return SFGPU_FAILURE;
    }
    const size_t off = (size_t)first * s->n;
    SF_CUDA(cudaMemcpyAsync(slab + off, s->slab + off, sizeof(float) * (size_t)count * s->n,
                            cudaMemcpyDeviceToHost, s->stream));
    SF_CUDA(cudaStreamSynchronize(s->stream));
    return SFGPU_OK;
}

extern "C" int sfgpu_download(sfgpu_sim* s, float* slab) {
    return sfgpu_download_arrays(s, slab, 0, s ? s->dof : 0);
}

// ---------------------------------------------------------------------------
// solve / step
// ---------------------------------------------------------------------------
__global__ static void k_set_step(uint32_t* d_step, uint32_t v) { *d_step = v; }

static int solve_body(sfgpu_sim* s, bool radius_ready) {
    if (s->p.solver == SFGPU_SOLVER_TREE) {
        if (sf_stage_tree_solve(s, radius_ready) != SFGPU_OK) return SFGPU_FAILURE;
    } else {
        const int tk = s->timer.begin(s->stream, "pp");
        if (sf_stage_gravity_pp(s) != SFGPU_OK) return SFGPU_FAILURE;
        s->timer.end(s->stream, tk);
    }
    if (s->p.sph != SFGPU_SPH_OFF) {
        const int tk = s->timer.begin(s->stream, "sph");
        if (sf_stage_sph(s) != SFGPU_OK) return SFGPU_FAILURE;
        s->timer.end(s->stream, tk);
    }
    return SFGPU_OK;
}

static int step_body(sfgpu_sim* s) {
    const bool tree = s->p.solver == SFGPU_SOLVER_TREE;
    int tk = s->timer.begin(s->stream, "kick_drift");
    if (sf_stage_kick_drift(s, tree) != SFGPU_OK) return SFGPU_FAILURE;
    s->timer.end(s->stream, tk);
    if (s->host_pos_out) {
        // the positions are final after the drift: their download runs on
        // the second stream beside the force solve
        SF_CUDA(cudaEventRecord(s->ev_pos, s->stream));
        SF_CUDA(cudaStreamWaitEvent(s->aux, s->ev_pos, 0));
        SF_CUDA(cudaMemcpyAsync(s->host_pos_out, s->slab, sizeof(float) * 3 * (size_t)s->n,
                                cudaMemcpyDeviceToHost, s->aux));
        SF_CUDA(cudaEventRecord(s->ev_pos_done, s->aux));
    }
    // without SPH the walk's epilogue may apply kick_1 and the energies
    // itself (sets kicked); SPH forces come after the walk, so not then
    s->fuse_kick = tree && s->p.sph == SFGPU_SPH_OFF;
    s->kicked = false;
    const int rc = solve_body(s, true);
    s->fuse_kick = false;
    if (rc != SFGPU_OK) return SFGPU_FAILURE;
    if (!s->kicked) {
        tk = s->timer.begin(s->stream, "kick_energy");
        if (sf_stage_kick_energy(s) != SFGPU_OK) return SFGPU_FAILURE;
        s->timer.end(s->stream, tk);
    }
    return SFGPU_OK;
}

extern "C" int sfgpu_solve(sfgpu_sim* s, uint32_t step_number) {
    sf_clear_error();
    if (!s) {
        sf_set_error("sim is NULL");
        return SFGPU_FAILURE;
    }
    k_set_step<<<1, 1, 0, s->stream>>>(s->d_step, step_number);
    SF_CHECK_LAUNCH();
    return solve_body(s, false);
}

extern "C" int sfgpu_step(sfgpu_sim* s, uint32_t step_number) {
    sf_clear_error();
    if (!s) {
        sf_set_error("sim is NULL");
        return SFGPU_FAILURE;
    }
    k_set_step<<<1, 1, 0, s->stream>>>(s->d_step, step_number);
    SF_CHECK_LAUNCH();
    return step_body(s);
}

extern "C" int sfgpu_run(sfgpu_sim* s, uint32_t first_step, uint32_t nsteps) {
    sf_clear_error();
    if (!s) {
        sf_set_error("sim is NULL");
        return SFGPU_FAILURE;
    }
    if (nsteps == 0) return SFGPU_OK;
    k_set_step<<<1, 1, 0, s->stream>>>(s->d_step, first_step);
    SF_CHECK_LAUNCH();
    const bool use_graph = !(s->p.flags & SFGPU_FLAG_NOGRAPH) && !s->timer.enabled && s->graph_ok;
    if (!use_graph) {
        for (uint32_t k = 0; k < nsteps; k++)
            if (step_body(s) != SFGPU_OK) return SFGPU_FAILURE;
        return SFGPU_OK;
    }
    if (!s->graph) {
        // step_body advances d_step itself (k_kick_energy), so one captured
        // step replays correctly for any step number.
        cudaGraph_t g = nullptr;
        SF_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = step_body(s);
        cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
        if (rc != SFGPU_OK || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            s->graph_ok = false;
            for (uint32_t k = 0; k < nsteps; k++)
                if (step_body(s) != SFGPU_OK) return SFGPU_FAILURE;
            return SFGPU_OK;
        }
        cudaError_t ie = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            s->graph = nullptr;
            s->graph_ok = false;
            cudaGetLastError();
            for (uint32_t k = 0; k < nsteps; k++)
                if (step_body(s) != SFGPU_OK) return SFGPU_FAILURE;
            return SFGPU_OK;
        }
    }
    for (uint32_t k = 0; k < nsteps; k++) SF_CUDA(cudaGraphLaunch(s->graph, s->stream));
    return SFGPU_OK;
}

__global__ static void k_copy_bounds(const float* __restrict__ src, float* __restrict__ dst) {
    if (threadIdx.x < 6) dst[threadIdx.x] = src[threadIdx.x];
}

extern "C" int sfgpu_tree_build(sfgpu_sim* s, const float bounds[6]) {
    sf_clear_error();
    if (!s || !s->tree || !bounds) {
        sf_set_error("sfgpu_tree_build needs a tree simulation and bounds");
        return SFGPU_FAILURE;
    }
    float* tmp = nullptr;
    SF_CUDA(cudaMalloc(&tmp, sizeof(float) * 8));
    cudaError_t e = cudaMemcpy(tmp, bounds, sizeof(float) * 6, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_copy_bounds<<<1, 32, 0, s->stream>>>(tmp, s->d_bounds);
        e = cudaGetLastError();
    }
    int rc = e == cudaSuccess ? sf_tree_build(s) : SFGPU_FAILURE;
    cudaStreamSynchronize(s->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) {
        sf_set_error("sfgpu_tree_build: %s", cudaGetErrorString(e));
        return SFGPU_FAILURE;
    }
    return rc;
}

extern "C" int sfgpu_gravity_tree(sfgpu_sim* s) {
    sf_clear_error();
    if (!s || !s->tree) {
        sf_set_error("sfgpu_gravity_tree needs a tree simulation");
        return SFGPU_FAILURE;
    }
    // the walk reads the sorted copy of the bodies made by the build; refresh
    // it for the current positions without rebuilding the topology
    return sf_walk_launch(s);
}

extern "C" int sfgpu_gravity_part(sfgpu_sim* s) {
    sf_clear_error();
    if (!s) return SFGPU_FAILURE;
    return sf_stage_gravity_pp(s);
}

extern "C" int sfgpu_solve_sph(sfgpu_sim* s) {
    sf_clear_error();
    if (!s || s->p.sph == SFGPU_SPH_OFF) {
        sf_set_error("sfgpu_solve_sph needs a simulation created with SPH enabled");
        return SFGPU_FAILURE;
    }
    return sf_stage_sph(s);
}

uint32_t* sf_sph_neighbour_counts(sfgpu_sim* s);

extern "C" int sfgpu_sph_neighbours(sfgpu_sim* s, uint32_t* counts) {
    sf_clear_error();
    uint32_t* d = s ? sf_sph_neighbour_counts(s) : nullptr;
    if (!d || !counts) {
        sf_set_error("sfgpu_sph_neighbours needs a simulation with SPH");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    SF_CUDA(cudaMemcpy(counts, d, sizeof(uint32_t) * s->n, cudaMemcpyDeviceToHost));
    return SFGPU_OK;
}

uint64_t* sf_sph_neighbour_hashes(sfgpu_sim* s);

extern "C" int sfgpu_sph_neighbour_hashes(sfgpu_sim* s, uint64_t* hashes) {
    sf_clear_error();
    uint64_t* d = s ? sf_sph_neighbour_hashes(s) : nullptr;
    if (!d || !hashes) {
        sf_set_error("sfgpu_sph_neighbour_hashes needs a simulation with SPH created with SFGPU_FLAG_STATS");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    SF_CUDA(cudaMemcpy(hashes, d, sizeof(uint64_t) * s->n, cudaMemcpyDeviceToHost));
    return SFGPU_OK;
}

extern "C" int sfgpu_sph_set_u(sfgpu_sim* s, const float* u) {
    sf_clear_error();
    if (!s || !s->u || !u) {
        sf_set_error("sfgpu_sph_set_u needs a simulation with cubic-spline SPH");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    SF_CUDA(cudaMemcpy(s->u, u, sizeof(float) * s->n, cudaMemcpyHostToDevice));
    return SFGPU_OK;
}

extern "C" int sfgpu_sph_get_u(sfgpu_sim* s, float* u, float* dudt) {
    sf_clear_error();
    if (!s || !s->u) {
        sf_set_error("sfgpu_sph_get_u needs a simulation with cubic-spline SPH");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    if (u) SF_CUDA(cudaMemcpy(u, s->u, sizeof(float) * s->n, cudaMemcpyDeviceToHost));
    if (dudt) SF_CUDA(cudaMemcpy(dudt, s->dudt, sizeof(float) * s->n, cudaMemcpyDeviceToHost));
    return SFGPU_OK;
}

extern "C" int sfgpu_synchronize(sfgpu_sim* s) {
    sf_clear_error();
    if (!s) return SFGPU_FAILURE;
    SF_CUDA(cudaStreamSynchronize(s->stream));
    return SFGPU_OK;
}

__global__ static void k_set_step_host(uint32_t* d_step, const volatile uint32_t* h_step) { *d_step = *h_step; }
// the status word to page-locked memory, cleared for the next call
__global__ static void k_status_host(uint32_t* d_status, volatile uint32_t* h_status) {
    *h_status = *d_status;
    *d_status = 0u;
}

// Everything of one drop-in call, queued on the simulation's stream: the
// arrays a solve or a step reads (pos, vel, acc, mas, 0..9, and with SPH the
// smoothing lengths, 13) in, the step number from page-locked memory, the
// solve or the step, the whole slab and the status word out.
// early_pos: the slab is page-locked and the body is being captured, so the
// positions may be downloaded on the second stream while the forces run
static int host_step_body(sfgpu_sim* s, float* slab, int solve_only, bool early_pos) {
    const size_t n = s->n;
    SF_CUDA(cudaMemcpyAsync(s->slab, slab, sizeof(float) * 10 * n, cudaMemcpyHostToDevice, s->stream));
    if (s->dof > 13)
        SF_CUDA(cudaMemcpyAsync(s->slab + 13 * n, slab + 13 * n, sizeof(float) * n, cudaMemcpyHostToDevice,
                                s->stream));
    k_set_step_host<<<1, 1, 0, s->stream>>>(s->d_step, s->h_step_in);
    SF_CHECK_LAUNCH();
    if (refresh_fp64(s) != SFGPU_OK) return SFGPU_FAILURE;
    const bool split = early_pos && !solve_only;
    s->host_pos_out = split ? slab : nullptr;
    const int rc = solve_only ? solve_body(s, false) : step_body(s);
    s->host_pos_out = nullptr;
    if (rc != SFGPU_OK) return SFGPU_FAILURE;
    if (split) {
        SF_CUDA(cudaStreamWaitEvent(s->stream, s->ev_pos_done, 0));
        SF_CUDA(cudaMemcpyAsync(slab + 3 * n, s->slab + 3 * n, sizeof(float) * (s->dof - 3) * n,
                                cudaMemcpyDeviceToHost, s->stream));
    } else {
        SF_CUDA(cudaMemcpyAsync(slab, s->slab, sizeof(float) * s->dof * n, cudaMemcpyDeviceToHost, s->stream));
    }
    k_status_host<<<1, 1, 0, s->stream>>>(s->d_status, s->h_status);
    SF_CHECK_LAUNCH();
    return SFGPU_OK;
}

extern "C" int sfgpu_host_step(sfgpu_sim* s, float* slab, uint32_t step_number, int solve_only,
                               uint32_t* status) {
    sf_clear_error();
    if (!s || !slab) {
        sf_set_error("sfgpu_host_step: NULL argument");
        return SFGPU_FAILURE;
    }
    *s->h_step_in = step_number;  // the previous call has synchronised: nothing reads it now
    // a page-locked slab lets the copies live in one captured graph with the
    // step, replayed by a single launch per call
    bool use_graph = !(s->p.flags & SFGPU_FLAG_NOGRAPH) && !s->timer.enabled && s->host_graph_ok;
    if (use_graph && (s->host_graph_slab != slab || s->host_graph_solve != (solve_only ? 1 : 0))) {
        cudaPointerAttributes pa;
        const bool pinned = cudaPointerGetAttributes(&pa, slab) == cudaSuccess && pa.type == cudaMemoryTypeHost;
        cudaGetLastError();
        if (s->host_graph) {
            cudaGraphExecDestroy(s->host_graph);
            s->host_graph = nullptr;
        }
        if (pinned) {
            cudaGraph_t g = nullptr;
            SF_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            const int rc = host_step_body(s, slab, solve_only, true);
            const cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
            if (rc == SFGPU_OK && ce == cudaSuccess && cudaGraphInstantiate(&s->host_graph, g, 0) == cudaSuccess) {
                s->host_graph_slab = slab;
                s->host_graph_solve = solve_only ? 1 : 0;
            } else {
                s->host_graph = nullptr;
                s->host_graph_ok = false;
            }
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            sf_clear_error();
        }
        use_graph = s->host_graph != nullptr;
    }
    if (use_graph) {
        SF_CUDA(cudaGraphLaunch(s->host_graph, s->stream));
    } else if (host_step_body(s, slab, solve_only, false) != SFGPU_OK) {
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    if (status) *status = *s->h_status;
    return SFGPU_OK;
}

static int fetch_sums(sfgpu_sim* s) {
    SF_CUDA(cudaMemcpyAsync(s->h_sums, s->sums, sizeof(double) * 8, cudaMemcpyDeviceToHost, s->stream));
    SF_CUDA(cudaStreamSynchronize(s->stream));
    return SFGPU_OK;
}

extern "C" int sfgpu_energies(sfgpu_sim* s, double* T, double* V) {
    sf_clear_error();
    if (!s || fetch_sums(s) != SFGPU_OK) return SFGPU_FAILURE;
    if (T) *T = s->h_sums[0];
    if (V) *V = s->h_sums[1];
    return SFGPU_OK;
}

extern "C" int sfgpu_energies_corrected(sfgpu_sim* s, double* T, double* V, double* E) {
    sf_clear_error();
    if (!s || fetch_sums(s) != SFGPU_OK) return SFGPU_FAILURE;
    if (T) *T = s->h_sums[2];
    if (V) *V = s->h_sums[3];
    if (E) *E = s->h_sums[2] + s->h_sums[3];
    return SFGPU_OK;
}

extern "C" int sfgpu_momentum(sfgpu_sim* s, double P[3], double L[3]) {
    sf_clear_error();
    if (!s) {
        sf_set_error("sim is NULL");
        return SFGPU_FAILURE;
    }
    if (sf_stage_momentum(s) != SFGPU_OK) return SFGPU_FAILURE;
    SF_CUDA(cudaMemcpyAsync(s->h_sums + 8, s->sums + 8, sizeof(double) * 6, cudaMemcpyDeviceToHost, s->stream));
    SF_CUDA(cudaStreamSynchronize(s->stream));
    for (int c = 0; c < 3; c++) {
        if (P) P[c] = s->h_sums[8 + c];
        if (L) L[c] = s->h_sums[11 + c];
    }
    return SFGPU_OK;
}

extern "C" int sfgpu_status(sfgpu_sim* s, uint32_t* status) {
    sf_clear_error();
    if (!s) return SFGPU_FAILURE;
    SF_CUDA(cudaMemcpyAsync(s->h_status, s->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    SF_CUDA(cudaMemsetAsync(s->d_status, 0, sizeof(uint32_t), s->stream));
    SF_CUDA(cudaStreamSynchronize(s->stream));
    if (status) *status = *s->h_status;
    return SFGPU_OK;
}

extern "C" void* sfgpu_stream(sfgpu_sim* s) { return s ? (void*)s->stream : nullptr; }
extern "C" float* sfgpu_device_slab(sfgpu_sim* s) { return s ? s->slab : nullptr; }

extern "C" int sfgpu_stage_times(sfgpu_sim* s, const char** names, double* ms, uint32_t* launches, int cap) {
    sf_clear_error();
    if (!s) return SFGPU_FAILURE;
    s->timer.collect();
    const int m = std::min<int>(cap, (int)s->timer.names.size());
    for (int i = 0; i < m; i++) {
        if (names) names[i] = s->timer.names[i].c_str();
        if (ms) ms[i] = s->timer.ms[i];
        if (launches) launches[i] = s->timer.launches[i];
        s->timer.ms[i] = 0.0;
        s->timer.launches[i] = 0;
    }
    return m;
}

extern "C" int sfgpu_walk_stats(sfgpu_sim* s, uint32_t* interactions, uint32_t* opening_tests) {
    sf_clear_error();
    if (!s || !s->stat_int) {
        sf_set_error("walk statistics need a tree simulation created with SFGPU_FLAG_STATS");
        return SFGPU_FAILURE;
    }
    SF_CUDA(cudaStreamSynchronize(s->stream));
    if (interactions) SF_CUDA(cudaMemcpy(interactions, s->stat_int, sizeof(uint32_t) * s->n, cudaMemcpyDeviceToHost));
    if (opening_tests) SF_CUDA(cudaMemcpy(opening_tests, s->stat_open, sizeof(uint32_t) * s->n, cudaMemcpyDeviceToHost));
    return SFGPU_OK;
}

extern "C" int sfgpu_walk_totals(sfgpu_sim* s, uint64_t* interactions, uint64_t* opening_tests) {
    sf_clear_error();
    if (!s) return SFGPU_FAILURE;
    unsigned long long h[2] = {0, 0};
    SF_CUDA(cudaMemcpyAsync(h, s->walk_tot, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    SF_CUDA(cudaMemsetAsync(s->walk_tot, 0, sizeof(h), s->stream));
    SF_CUDA(cudaStreamSynchronize(s->stream));
    if (interactions) *interactions = h[0];
    if (opening_tests) *opening_tests = h[1];
    return SFGPU_OK;
}

extern "C" int sfgpu_tree_keys(sfgpu_sim* s, uint64_t* keys, uint32_t* index, uint32_t* n_inside, float bounds[6]) {
    sf_clear_error();
    if (!s) return SFGPU_FAILURE;
    if (bounds) {
        SF_CUDA(cudaStreamSynchronize(s->stream));
        SF_CUDA(cudaMemcpy(bounds, s->d_bounds, sizeof(float) * 6, cudaMemcpyDeviceToHost));
    }
    return sf_tree_keys(s, keys, index, n_inside);
}

extern "C" int sfgpu_tree_num_nodes(sfgpu_sim* s, uint32_t* num_nodes) {
    sf_clear_error();
    if (!s || !num_nodes) return SFGPU_FAILURE;
    return sf_tree_num_nodes(s, num_nodes);
}

extern "C" int sfgpu_tree_export(sfgpu_sim* s, uint32_t* parent, uint32_t* bodies, uint32_t* branch8, float* bounds6,
                                 float* params4) {
    sf_clear_error();
    if (!s) return SFGPU_FAILURE;
    return sf_tree_export(s, parent, bodies, branch8, bounds6, params4);
}

// ---------------------------------------------------------------------------
// stateless PP on caller arrays
// ---------------------------------------------------------------------------
struct ThreadScratch {
    float4* part = nullptr;
    size_t cap = 0;
};
static thread_local ThreadScratch g_pp_scratch;

extern "C" int sfgpu_gravity_pp(const sfgpu_params* p, uint32_t n, const float* pos, const float* mas, float* acc,
                                float* pot, void* stream) {
    sf_clear_error();
    if (validate(p) != SFGPU_OK) return SFGPU_FAILURE;
    if (p->form == SFGPU_FORM_COMPENSATED && p->math == SFGPU_MATH_EXACT) {
        sf_set_error("EXACT math applies to the PLAIN form only");
        return SFGPU_FAILURE;
    }
    return sf_pp_launch(*p, n, pos, mas, acc, pot, &g_pp_scratch.part, &g_pp_scratch.cap, (cudaStream_t)stream,
                        nullptr);
}
