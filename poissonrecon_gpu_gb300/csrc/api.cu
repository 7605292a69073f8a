// C ABI (include/prgpu.h) and stage orchestration.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_bf16.h>

#include "context.h"
#include "learned.h"
#include "prims.cuh"

namespace prgpu {

static thread_local char g_err[512] = {0};
std::atomic<unsigned long long> g_kernel_launches(0);
std::atomic<long long> g_fail_alloc_countdown(0);
static std::atomic<long long> g_spin_limit(DEFAULT_SPIN_LIMIT);
static std::atomic<int> g_wait_extra(0);
WaitLimits wait_limits() {
    WaitLimits w;
    w.spin_limit = g_spin_limit.load();
    w.extra = g_wait_extra.load();
    return w;
}
void set_last_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}
const char* last_error() { return g_err; }

void Ctx::free_nodes() {
    cudaStream_t s = stream;
    dfree(nodes.key, s); dfree(nodes.pidx, s); dfree(nodes.pnum, s); dfree(nodes.didx, s);
    dfree(nodes.dnum, s); dfree(nodes.parent, s); dfree(nodes.child0, s); dfree(nodes.depth, s);
    dfree(nodes.neigh, s);
    dfree(gn, s);
    dfree(gn_rows, s);
    nodes.M = 0;
}
void Ctx::free_all() {
    cudaStream_t s = stream;
    free_nodes();
    dfree(in_xyz, s); dfree(in_nrm, s); dfree(pts, s); dfree(nrm, s); dfree(sort_idx, s);
    dfree(point_node, s); dfree(basis, s); dfree(ddot_div, s); dfree(full_tables, s);
    dfree(cascade_tab, s);
    cascade_off.clear();
    dfree(vfield, s); dfree(divergence, s); dfree(x, s); dfree(point_value, s);
    dfree(point_weight, s); dfree(wnrm, s);
    dfree(d_cg_iters, s); dfree(d_cg_rr, s);
    dfree(d_has_tri, s); dfree(d_has_int, s);
    n_coarse = 0;
}

int Ctx::kbegin(const char* name, double bytes) {
    if (!profile) return -1;
    int slot = -1;
    for (size_t k = 0; k < ktimers.size(); ++k)
        if (ktimers[k].name == name) slot = (int)k;
    if (slot < 0) {
        ktimers.push_back(KernelTimer());
        ktimers.back().name = name;
        slot = (int)ktimers.size() - 1;
    }
    while (kevents.size() < kev_next + 2) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        kevents.push_back(e);
    }
    PendingTimer pt;
    pt.slot = slot;
    pt.a = kevents[kev_next++];
    pt.b = kevents[kev_next++];
    pt.bytes = bytes;
    CK(cudaEventRecord(pt.a, stream));
    kpending.push_back(pt);
    return (int)kpending.size() - 1;
}
void Ctx::kend(int h) {
    if (h < 0) return;
    CK(cudaEventRecord(kpending[h].b, stream));
}
void Ctx::kflush() {
    if (kpending.empty()) return;
    CK(cudaStreamSynchronize(stream));
    for (auto& p : kpending) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, p.a, p.b));
        KernelTimer& t = ktimers[p.slot];
        t.ms += ms;
        t.launches += 1;
        t.bytes += p.bytes;
    }
    kpending.clear();
    kev_next = 0;
}

int cg_csr_impl(int n, const int* rowptr, const int* col, const float* val, const float* rhs, float* x, float tol,
                int max_iter, int* iters, float* ms);

// timed stage runner: CUDA events on the context stream
template <class F>
static void timed(Ctx& c, float& acc, F&& f) {
    CK(cudaEventRecord(c.ev0, c.stream));
    f();
    CK(cudaEventRecord(c.ev1, c.stream));
    CK(cudaEventSynchronize(c.ev1));
    c.kflush();
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    acc = ms;
}

}  // namespace prgpu

using namespace prgpu;

namespace prgpu {
thread_local LiveAllocs* g_live = nullptr;
}

// One API call: collects the call's device allocations.  When the call fails, the
// context (if given) releases its buffers and must be given its points again (stage
// 0), then the call's remaining allocations -- temporaries of the stage that failed --
// are freed, so repeated failures do not accumulate device memory.
struct CallScope {
    LiveAllocs live;
    LiveAllocs* prev;
    Ctx* c;
    explicit CallScope(Ctx* ctx) : prev(g_live), c(ctx) { g_live = &live; }
    ~CallScope() { g_live = prev; }
    void fail() {
        if (c) {
            c->free_all();
            c->stage = 0;
            c->kpending.clear();   // timers of the failed stage may lack their end event
            c->kev_next = 0;
        }
        for (auto& a : live.v) cudaFreeAsync(a.first, a.second);
        live.v.clear();
    }
};

#define API_BEGIN_CTX(ctx) \
    CallScope scope_(ctx); \
    try {
#define API_BEGIN API_BEGIN_CTX(nullptr)
#define API_END                                                   \
    }                                                             \
    catch (const prgpu::Error& e) {                               \
        scope_.fail();                                            \
        return e.status;                                          \
    }                                                             \
    catch (...) {                                                 \
        scope_.fail();                                            \
        prgpu::set_last_error("unexpected host exception");       \
        return PRGPU_ERR_CUDA;                                    \
    }

static Ctx* as_ctx(void* p) { return (Ctx*)p; }

// nodes holding at least one point, per depth (the level of node i from the level bases)
__global__ void k_occupied(const int* __restrict__ pnum, const i64* __restrict__ base, int D,
                           unsigned long long* __restrict__ occ) {
    const i64 M = base[D + 1];
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (i64)gridDim.x * blockDim.x) {
        if (pnum[i] <= 0) continue;
        int d = 0;
        while (d < D && base[d + 1] <= i) ++d;
        atomicAdd(&occ[d], 1ull);
    }
}

extern "C" {

int prgpu_params_default(prgpu_params* p) {
    if (!p) return PRGPU_ERR_ARG;
    memset(p, 0, sizeof *p);
    p->depth = 8;
    p->solve_mode = PRGPU_SOLVE_REFERENCE;
    p->cg_tol = 1e-5;
    p->cg_max_iter = 10000;
    p->device = 0;
    return PRGPU_OK;
}

const char* prgpu_last_error(void) { return prgpu::last_error(); }

int prgpu_create(const prgpu_params* p, void** out) {
    if (!p || !out) return PRGPU_ERR_ARG;
    if (p->depth < 2 || p->depth > PRGPU_MAX_DEPTH) {
        set_last_error("depth %d outside the supported range 2..%d", p->depth, PRGPU_MAX_DEPTH);
        return PRGPU_ERR_LIMIT;
    }
    Ctx* c = new Ctx();
    API_BEGIN
    c->params = *p;
    c->D = p->depth;
    c->device = p->device;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    // keep freed pool memory for reuse across calls
    cudaMemPool_t pool;
    CK(cudaDeviceGetDefaultMemPool(&pool, c->device));
    uint64_t thr = ~0ull;
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    *out = c;
    return PRGPU_OK;
    }
    catch (...) {   // nothing is handed out: release what was created
        if (c->ev1) cudaEventDestroy(c->ev1);
        if (c->ev0) cudaEventDestroy(c->ev0);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        try {
            throw;
        } catch (const prgpu::Error& e) {
            return e.status;
        } catch (...) {
            set_last_error("unexpected host exception");
            return PRGPU_ERR_CUDA;
        }
    }
}

int prgpu_destroy(void* h) {
    Ctx* c = as_ctx(h);
    if (!c) return PRGPU_ERR_ARG;
    API_BEGIN
    for (Ctx* w : c->workers) prgpu_destroy(w);
    c->workers.clear();
    CK(cudaSetDevice(c->device));
    c->free_all();
    CK(cudaStreamSynchronize(c->stream));
    if (c->lp_params) cudaFree(c->lp_params);
    if (c->lp_w1b) cudaFree(c->lp_w1b);
    if (c->lp_w2b) cudaFree(c->lp_w2b);
    for (auto e : c->kevents) cudaEventDestroy(e);
    cudaEventDestroy(c->ev0);
    cudaEventDestroy(c->ev1);
    cudaStreamDestroy(c->stream);
    delete c;
    return PRGPU_OK;
    API_END
}

static int set_points_common(Ctx* c, const float* xyz, const float* nrm, int64_t n, cudaMemcpyKind kind) {
    if (!c || !xyz || !nrm || n <= 0) {
        set_last_error("prgpu_set_points: empty or null input");
        return PRGPU_ERR_ARG;
    }
    if (n > 0x7fffffffLL / 3) {
        set_last_error("%lld points exceed the supported count", (long long)n);
        return PRGPU_ERR_LIMIT;
    }
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    dfree(c->in_xyz, s);
    dfree(c->in_nrm, s);
    c->N = n;
    c->in_xyz = dalloc<float>(3 * n, s);
    c->in_nrm = dalloc<float>(3 * n, s);
    CK(cudaMemcpyAsync(c->in_xyz, xyz, (size_t)(3 * n) * sizeof(float), kind, s));
    CK(cudaMemcpyAsync(c->in_nrm, nrm, (size_t)(3 * n) * sizeof(float), kind, s));
    c->stage = 1;
    return PRGPU_OK;
    API_END
}

int prgpu_set_points(void* h, const float* xyz, const float* nrm, int64_t n) {
    return set_points_common(as_ctx(h), xyz, nrm, n, cudaMemcpyHostToDevice);
}
int prgpu_set_points_device(void* h, const float* xyz, const float* nrm, int64_t n) {
    return set_points_common(as_ctx(h), xyz, nrm, n, cudaMemcpyDeviceToDevice);
}

#define REQUIRE_STAGE(c, st)                                                  \
    do {                                                                      \
        if (!(c) || (c)->stage < (st)) {                                      \
            prgpu::set_last_error("%s called before its inputs exist", __func__); \
            return PRGPU_ERR_ARG;                                             \
        }                                                                     \
    } while (0)

int prgpu_build_octree(void* h) {
    Ctx* c = as_ctx(h);
    REQUIRE_STAGE(c, 1);
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    timed(*c, c->t.octree_ms, [&] { stage_octree(*c); });
    c->stage = 2;
    return PRGPU_OK;
    API_END
}

int prgpu_compute_rhs(void* h) {
    Ctx* c = as_ctx(h);
    REQUIRE_STAGE(c, 2);
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    timed(*c, c->t.basis_ms, [&] { stage_basis(*c); });
    timed(*c, c->t.splat_ms, [&] { stage_splat(*c); });
    timed(*c, c->t.divergence_ms, [&] { stage_divergence(*c); });
    c->stage = 3;
    return PRGPU_OK;
    API_END
}

int prgpu_solve(void* h) {
    Ctx* c = as_ctx(h);
    REQUIRE_STAGE(c, 3);
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    timed(*c, c->t.solve_ms, [&] { stage_solve(*c); });
    c->stage = 4;
    bool conv = true;
    for (int d = 0; d <= c->D; ++d)
        if (c->cg_iters[d] >= c->params.cg_max_iter) conv = false;
    return conv ? PRGPU_OK : PRGPU_ERR_NOT_CONVERGED;
    API_END
}

int prgpu_solve_depth(void* h, int32_t depth, int32_t mode) {
    Ctx* c = as_ctx(h);
    REQUIRE_STAGE(c, 3);
    if (depth < 0 || depth > c->D || (mode != PRGPU_SOLVE_REFERENCE && mode != PRGPU_SOLVE_RELATIVE)) {
        set_last_error("prgpu_solve_depth: depth %d (maxDepth %d), mode %d", depth, c->D, mode);
        return PRGPU_ERR_ARG;
    }
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    timed(*c, c->t.solve_ms, [&] {
        if (!c->params.cascadic) {
            stage_solve_depths(*c, depth, depth, mode);
            return;
        }
        if (!c->x || c->x_rows != c->nodes.M) {   // no solve yet: the coarser rows are 0
            dfree(c->x, c->stream);
            c->x = dalloc<float>(c->nodes.M, c->stream);
            c->x_rows = c->nodes.M;
            CK(cudaMemsetAsync(c->x, 0, c->nodes.M * sizeof(float), c->stream));
        }
        float* rhs = dalloc<float>(c->nodes.M, c->stream);
        cascade_rhs(*c, depth, rhs);
        stage_solve_depths(*c, depth, depth, mode, rhs);
        dfree(rhs, c->stream);
    });
    c->stage = std::max(c->stage, 4);
    return c->cg_iters[depth] >= c->params.cg_max_iter ? PRGPU_ERR_NOT_CONVERGED : PRGPU_OK;
    API_END
}

int prgpu_eval_points(void* h, float* iso_out) {
    Ctx* c = as_ctx(h);
    REQUIRE_STAGE(c, 4);
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    timed(*c, c->t.iso_ms, [&] { stage_points(*c); });
    if (iso_out) *iso_out = c->iso;
    c->stage = 5;
    return PRGPU_OK;
    API_END
}

int prgpu_extract_mesh(void* h) {
    Ctx* c = as_ctx(h);
    REQUIRE_STAGE(c, 5);
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    timed(*c, c->t.mesh_ms, [&] { stage_mesh(*c); });
    c->stage = 6;
    return PRGPU_OK;
    API_END
}

int prgpu_get_mesh(void* h, prgpu_mesh* out) {
    Ctx* c = as_ctx(h);
    REQUIRE_STAGE(c, 6);
    if (!out) return PRGPU_ERR_ARG;
    out->n_vertices = (int64_t)c->mesh_v.size() / 3;
    out->n_triangles = (int64_t)c->mesh_f.size() / 3;
    out->vertices = c->mesh_v.data();
    out->triangles = c->mesh_f.data();
    return PRGPU_OK;
}

int prgpu_reconstruct(void* h, const float* xyz, const float* nrm, int64_t n, prgpu_mesh* out) {
    int rc = prgpu_set_points(h, xyz, nrm, n);
    if (rc) return rc;
    if ((rc = prgpu_build_octree(h))) return rc;
    if ((rc = prgpu_compute_rhs(h))) return rc;
    int solve_rc = prgpu_solve(h);
    if (solve_rc && solve_rc != PRGPU_ERR_NOT_CONVERGED) return solve_rc;
    if ((rc = prgpu_eval_points(h, nullptr))) return rc;
    if ((rc = prgpu_extract_mesh(h))) return rc;
    if (out && (rc = prgpu_get_mesh(h, out))) return rc;
    return PRGPU_OK;
}

int prgpu_mesh_free(prgpu_mesh* m) {
    if (!m) return PRGPU_ERR_ARG;
    free((void*)m->vertices);
    free((void*)m->triangles);
    m->vertices = nullptr;
    m->triangles = nullptr;
    m->n_vertices = m->n_triangles = 0;
    return PRGPU_OK;
}

// a reconstructed mesh copied into memory the caller releases with prgpu_mesh_free
static int copy_mesh_out(const prgpu_mesh& m, prgpu_mesh* out) {
    float* vv = (float*)malloc(sizeof(float) * 3 * (size_t)std::max<int64_t>(m.n_vertices, 1));
    int32_t* ff = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(m.n_triangles, 1));
    if (!vv || !ff) {
        free(vv);
        free(ff);
        set_last_error("host allocation failed");
        return PRGPU_ERR_NOMEM;
    }
    memcpy(vv, m.vertices, sizeof(float) * 3 * (size_t)m.n_vertices);
    memcpy(ff, m.triangles, sizeof(int32_t) * 3 * (size_t)m.n_triangles);
    out->vertices = vv;
    out->triangles = ff;
    out->n_vertices = m.n_vertices;
    out->n_triangles = m.n_triangles;
    return PRGPU_OK;
}

// Clouds of at most BATCH_SHARED_POINTS points are reconstructed BATCH_WORKERS at a
// time, each on a context of its own (own stream and buffers, a host thread each), so
// that the launches and host round trips of small clouds overlap on the GPU; larger
// clouds follow one at a time on the calling context, which bounds the memory held.
// Every cloud's result is that of a separate reconstruction.
constexpr int BATCH_WORKERS = 4;
constexpr int64_t BATCH_SHARED_POINTS = 4000000;

int prgpu_reconstruct_batch(void* h, const float* xyz, const float* nrm, const int64_t* offsets,
                            const int32_t* depths, int32_t ncloud, prgpu_mesh* outs) {
    Ctx* c = as_ctx(h);
    if (!c || !xyz || !nrm || !offsets || !outs || ncloud < 0) {
        set_last_error("prgpu_reconstruct_batch: invalid argument");
        return PRGPU_ERR_ARG;
    }
    for (int k = 0; k < ncloud; ++k) {
        outs[k].vertices = nullptr;
        outs[k].triangles = nullptr;
        outs[k].n_vertices = outs[k].n_triangles = 0;
    }
    const int D0 = c->D;
    std::vector<int> shared, alone;
    for (int k = 0; k < ncloud; ++k) {
        const int64_t n = offsets[k + 1] - offsets[k];
        const int d = depths ? depths[k] : D0;
        if (n <= 0 || offsets[k] < 0 || d < 2 || d > 15) {
            set_last_error("prgpu_reconstruct_batch: cloud %d: %lld points at depth %d", k, (long long)n, d);
            return PRGPU_ERR_ARG;
        }
        (n <= BATCH_SHARED_POINTS ? shared : alone).push_back(k);
    }
    // the first failure (lowest cloud index) is reported
    std::mutex mu;
    int err_cloud = -1, err_rc = PRGPU_OK;
    std::string err_msg;
    auto fail = [&](int k, int rc) {
        std::lock_guard<std::mutex> lock(mu);
        if (err_cloud < 0 || k < err_cloud) {
            err_cloud = k;
            err_rc = rc;
            err_msg = last_error();
        }
    };
    auto run = [&](Ctx* w, int k) -> bool {
        w->D = depths ? depths[k] : D0;
        prgpu_mesh m;
        int rc = prgpu_reconstruct(w, xyz + 3 * offsets[k], nrm + 3 * offsets[k], offsets[k + 1] - offsets[k], &m);
        if (rc == PRGPU_OK) rc = copy_mesh_out(m, &outs[k]);
        if (rc != PRGPU_OK) fail(k, rc);
        return rc == PRGPU_OK;
    };
    if (!shared.empty()) {
        const int nw = (int)std::min<size_t>(BATCH_WORKERS, shared.size());
        while ((int)c->workers.size() < nw) {
            void* w = nullptr;
            const int rc = prgpu_create(&c->params, &w);
            if (rc != PRGPU_OK) {
                set_last_error("prgpu_reconstruct_batch: worker context: %s", std::string(last_error()).c_str());
                return rc;
            }
            c->workers.push_back(as_ctx(w));
        }
        std::atomic<size_t> next(0);
        std::atomic<bool> failed(false);
        std::vector<std::thread> th;
        for (int wi = 0; wi < nw; ++wi)
            th.emplace_back([&, wi]() {
                if (cudaSetDevice(c->device) != cudaSuccess) {
                    set_last_error("cudaSetDevice failed");
                    fail(shared[0], PRGPU_ERR_CUDA);
                    failed = true;
                    return;
                }
                for (size_t q = next++; q < shared.size() && !failed; q = next++)
                    if (!run(c->workers[wi], shared[q])) failed = true;
            });
        for (auto& t : th) t.join();
    }
    if (err_cloud < 0)
        for (int k : alone)
            if (!run(c, k)) break;
    c->D = D0;
    if (err_cloud >= 0) {
        for (int k = 0; k < ncloud; ++k) prgpu_mesh_free(&outs[k]);
        set_last_error("prgpu_reconstruct_batch: cloud %d: %s", err_cloud, err_msg.c_str());
        return err_rc;
    }
    return PRGPU_OK;
}

// ----------------------------- array access ---------------------------------
namespace {
__global__ void k_expand_children(const int* __restrict__ child0, i64 M, int* __restrict__ out) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (i64)gridDim.x * blockDim.x)
        for (int k = 0; k < 8; ++k) out[8 * i + k] = child0[i] == -1 ? -1 : child0[i] + k;
}
__global__ void k_neigh_aos(const int* __restrict__ neigh, i64 M, int* __restrict__ out) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (i64)gridDim.x * blockDim.x)
        for (int j = 0; j < 27; ++j) out[27 * i + j] = neigh[(i64)j * M + i];
}
}  // namespace

static int copy_out(Ctx* c, const void* dsrc, int64_t bytes, void* dst, int64_t max_bytes, int64_t* nbytes,
                    bool host_src = false) {
    if (nbytes) *nbytes = bytes;
    if (!dst) return PRGPU_OK;
    if (max_bytes < bytes) {
        set_last_error("destination holds %lld bytes, %lld needed", (long long)max_bytes, (long long)bytes);
        return PRGPU_ERR_ARG;
    }
    if (bytes == 0) return PRGPU_OK;
    if (host_src) { memcpy(dst, dsrc, (size_t)bytes); return PRGPU_OK; }
    CK(cudaMemcpyAsync(dst, dsrc, (size_t)bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PRGPU_OK;
}

int prgpu_get_node_arrays(void* h, prgpu_node_arrays* out) {
    Ctx* c = as_ctx(h);
    if (!c || !out) return PRGPU_ERR_ARG;
    REQUIRE_STAGE(c, 2);
    const int64_t M = c->nodes.M;
    out->n_nodes = M;
    out->max_depth = c->D;
    struct Field { const char* name; void* dst; int64_t bytes; };
    const Field fields[] = {{"base", out->base, (int64_t)(c->D + 2) * 8}, {"key", out->key, M * 8},
                            {"pidx", out->pidx, M * 4},     {"pnum", out->pnum, M * 4},
                            {"parent", out->parent, M * 4}, {"children", out->children, M * 32},
                            {"neighs", out->neighs, M * 108}, {"didx", out->didx, M * 4},
                            {"dnum", out->dnum, M * 4}};
    for (const Field& f : fields) {
        if (!f.dst) continue;
        int64_t got = 0;
        const int rc = prgpu_get_array(h, f.name, f.dst, f.bytes, &got);
        if (rc != PRGPU_OK) return rc;
    }
    return PRGPU_OK;
}

int prgpu_get_array(void* h, const char* name, void* dst, int64_t max_bytes, int64_t* nbytes) {
    Ctx* c = as_ctx(h);
    if (!c || !name) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(c->device));
    std::string n(name);
    const i64 M = c->nodes.M;
    cudaStream_t s = c->stream;
    if (c->stage >= 2) {
        if (n == "key") {
            // int64 copy of the u64 keys
            return copy_out(c, c->nodes.key, M * 8, dst, max_bytes, nbytes);
        }
        if (n == "pidx") return copy_out(c, c->nodes.pidx, M * 4, dst, max_bytes, nbytes);
        if (n == "pnum") return copy_out(c, c->nodes.pnum, M * 4, dst, max_bytes, nbytes);
        if (n == "didx") return copy_out(c, c->nodes.didx, M * 4, dst, max_bytes, nbytes);
        if (n == "dnum") return copy_out(c, c->nodes.dnum, M * 4, dst, max_bytes, nbytes);
        if (n == "parent") return copy_out(c, c->nodes.parent, M * 4, dst, max_bytes, nbytes);
        if (n == "point_node") return copy_out(c, c->point_node, c->N * 4, dst, max_bytes, nbytes);
        if (n == "points") return copy_out(c, c->pts, c->N * 12, dst, max_bytes, nbytes);
        if (n == "normals") return copy_out(c, c->nrm, c->N * 12, dst, max_bytes, nbytes);
        if (n == "sort_idx") return copy_out(c, c->sort_idx, c->N * 4, dst, max_bytes, nbytes);
        if (n == "base") return copy_out(c, c->base.data(), (int64_t)c->base.size() * 8, dst, max_bytes, nbytes, true);
        if (n == "count") return copy_out(c, c->count.data(), (int64_t)c->count.size() * 8, dst, max_bytes, nbytes, true);
        if (n == "center") return copy_out(c, c->center, 12, dst, max_bytes, nbytes, true);
        if (n == "scale") return copy_out(c, &c->scale, 4, dst, max_bytes, nbytes, true);
        if (n == "children" || n == "neighs") {
            const int w = (n == "children") ? 8 : 27;
            if (nbytes) *nbytes = M * w * 4;
            if (!dst) return PRGPU_OK;
            int* tmp = dalloc<int>(M * w, s);
            if (w == 8) k_expand_children<<<grid_for(M, 256), 256, 0, s>>>(c->nodes.child0, M, tmp);
            else k_neigh_aos<<<grid_for(M, 256), 256, 0, s>>>(c->nodes.neigh, M, tmp);
            CK_LAUNCH();
            int rc = copy_out(c, tmp, M * w * 4, dst, max_bytes, nbytes);
            dfree(tmp, s);
            return rc;
        }
    }
    if (c->stage >= 3) {
        if (n == "vfield") return copy_out(c, c->vfield, c->count[c->D] * 12, dst, max_bytes, nbytes);
        if (n == "divergence") return copy_out(c, c->divergence, M * 4, dst, max_bytes, nbytes);
        if (n == "stencil")
            return copy_out(c, c->stencil.data(), (int64_t)c->stencil.size() * 4, dst, max_bytes, nbytes, true);
        if (n == "ddot_rows")
            return copy_out(c, c->ddot_div, c->ddot_row_start.back() * 4, dst, max_bytes, nbytes);
        if (n == "dot" || n == "ddot" || n == "d2dot") {
            const i64 res = (1 << (c->D + 1)) - 1, R2 = res * res;
            if (nbytes) *nbytes = R2 * 8;
            if (!dst) return PRGPU_OK;
            if (!c->full_tables) stage_full_tables(*c);
            const int which = (n == "dot") ? 0 : (n == "ddot" ? 1 : 2);
            return copy_out(c, c->full_tables + which * R2, R2 * 8, dst, max_bytes, nbytes);
        }
    }
    if (c->stage >= 4) {
        if (n == "x") return copy_out(c, c->x, M * 4, dst, max_bytes, nbytes);
        if (n == "cg_iters")
            return copy_out(c, c->cg_iters.data(), (int64_t)c->cg_iters.size() * 4, dst, max_bytes, nbytes, true);
        if (n == "cg_rr") return copy_out(c, c->cg_rr.data(), (int64_t)c->cg_rr.size() * 4, dst, max_bytes, nbytes, true);
    }
    if (c->stage >= 5) {
        if (n == "point_value") return copy_out(c, c->point_value, c->N * 4, dst, max_bytes, nbytes);
        if (n == "point_weight") return copy_out(c, c->point_weight, c->point_weight ? c->N * 4 : 0, dst, max_bytes, nbytes);
        if (n == "iso") return copy_out(c, &c->iso, 4, dst, max_bytes, nbytes, true);
    }
    if (c->stage >= 6) {
        if (n == "has_tri") return copy_out(c, c->d_has_tri, c->n_coarse * 4, dst, max_bytes, nbytes);
        if (n == "has_int") return copy_out(c, c->d_has_int, c->n_coarse * 4, dst, max_bytes, nbytes);
        if (n == "batch_tri")
            return copy_out(c, c->batch_tri.data(), (int64_t)c->batch_tri.size() * 8, dst, max_bytes, nbytes, true);
        if (n == "subdivide_roots") return copy_out(c, &c->subdivide_roots, 8, dst, max_bytes, nbytes, true);
    }
    set_last_error("unknown array '%s' or its stage has not run", name);
    return PRGPU_ERR_ARG;
    API_END
}

int prgpu_set_array(void* h, const char* name, const void* src, int64_t bytes) {
    Ctx* c = as_ctx(h);
    if (!c || !name || !src) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(c->device));
    std::string n(name);
    const i64 M = c->nodes.M;
    float* dst = nullptr;
    i64 need = 0;
    if (n == "vfield" && c->stage >= 3) { dst = c->vfield; need = c->count[c->D] * 12; }
    else if (n == "divergence" && c->stage >= 3) { dst = c->divergence; need = M * 4; }
    else if (n == "x" && c->stage >= 4) { dst = c->x; need = M * 4; }
    else if (n == "iso" && c->stage >= 5) {
        if (bytes != 4) return PRGPU_ERR_ARG;
        memcpy(&c->iso, src, 4);
        return PRGPU_OK;
    }
    if (!dst || bytes != need) {
        set_last_error("cannot set '%s' (%lld bytes) at this stage", name, (long long)bytes);
        return PRGPU_ERR_ARG;
    }
    CK(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PRGPU_OK;
    API_END
}

int prgpu_choose_depth(const float* xyz, const float* nrm, int64_t n, int32_t max_depth, double samples_per_node,
                       int32_t device, int32_t* depth, int64_t* occupied) {
    if (!xyz || !nrm || n <= 0 || !depth || !(samples_per_node > 0.0)) {
        set_last_error("prgpu_choose_depth: points, a depth pointer and samples_per_node > 0 are required");
        return PRGPU_ERR_ARG;
    }
    prgpu_params p;
    prgpu_params_default(&p);
    p.depth = max_depth;
    p.device = device;
    void* h = nullptr;
    int rc = prgpu_create(&p, &h);
    if (rc) return rc;
    Ctx* c = as_ctx(h);
    std::vector<unsigned long long> occ(max_depth + 1, 0);
    rc = prgpu_set_points(h, xyz, nrm, n);
    if (!rc) rc = prgpu_build_octree(h);
    if (!rc) {
        API_BEGIN_CTX(c)
        cudaStream_t s = c->stream;
        i64* dbase = dalloc<i64>(max_depth + 2, s);
        unsigned long long* docc = dalloc<unsigned long long>(max_depth + 1, s);
        CK(cudaMemcpyAsync(dbase, c->base.data(), (max_depth + 2) * sizeof(i64), cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(docc, 0, (max_depth + 1) * sizeof(unsigned long long), s));
        k_occupied<<<grid_for(c->nodes.M, 256), 256, 0, s>>>(c->nodes.pnum, dbase, max_depth, docc);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(occ.data(), docc, (max_depth + 1) * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        dfree(dbase, s);
        dfree(docc, s);
        rc = PRGPU_OK;
        }
        catch (const prgpu::Error& e) {
            scope_.fail();
            rc = e.status;
        }
        catch (...) {
            scope_.fail();
            prgpu::set_last_error("unexpected host exception");
            rc = PRGPU_ERR_CUDA;
        }
    }
    prgpu_destroy(h);
    if (rc) return rc;
    int best = 2;
    for (int d = 2; d <= max_depth; ++d)
        if (occ[d] > 0 && (double)n / (double)occ[d] >= samples_per_node) best = d;
    *depth = best;
    if (occupied)
        for (int d = 0; d <= max_depth; ++d) occupied[d] = (int64_t)occ[d];
    return PRGPU_OK;
}

int prgpu_stats_json(void* h, char* buf, int64_t len) {
    Ctx* c = as_ctx(h);
    if (!c || !buf || len <= 0) return PRGPU_ERR_ARG;
    std::string js = "{";
    char tmp[1024];
    snprintf(tmp, sizeof tmp, "\"points\":%lld,\"depth\":%d,\"nodes\":%lld,", (long long)c->N, c->D,
             (long long)c->nodes.M);
    js += tmp;
    js += "\"count\":[";
    for (size_t d = 0; d < c->count.size(); ++d) {
        snprintf(tmp, sizeof tmp, "%s%lld", d ? "," : "", (long long)c->count[d]);
        js += tmp;
    }
    js += "],\"roots_per_depth\":[";
    for (size_t d = 0; d < c->roots_per_depth.size(); ++d) {
        snprintf(tmp, sizeof tmp, "%s%lld", d ? "," : "", (long long)c->roots_per_depth[d]);
        js += tmp;
    }
    snprintf(tmp, sizeof tmp,
             "],\"virtual_cells\":%lld,\"bricks\":%lld,\"live_bricks\":%lld,\"foreign_corners\":%lld,"
             "\"foreign_evaluated\":%lld,\"super_bricks\":%lld,\"super_decided\":%lld,\"kernel_launches\":%llu",
             (long long)c->virtual_cells, (long long)c->total_bricks, (long long)c->live_bricks,
             (long long)c->foreign_corners, (long long)c->foreign_slow, (long long)c->super_bricks,
             (long long)c->super_decided,
             (unsigned long long)g_kernel_launches.load());
    js += tmp;
    snprintf(tmp, sizeof tmp, ",\"solver_blocks\":%d", c->solver_blocks);
    js += tmp;
    js += ",\"cg_iters\":[";
    for (size_t d = 0; d < c->cg_iters.size(); ++d) {
        snprintf(tmp, sizeof tmp, "%s%d", d ? "," : "", c->cg_iters[d]);
        js += tmp;
    }
    js += "],\"cg_fallback\":[";
    for (size_t d = 0; d < c->cg_fallback.size(); ++d) {
        snprintf(tmp, sizeof tmp, "%s%d", d ? "," : "", c->cg_fallback[d]);
        js += tmp;
    }
    js += "],\"cg_rel_residual\":[";
    for (size_t d = 0; d < c->cg_true_rel.size(); ++d) {
        snprintf(tmp, sizeof tmp, "%s%.6g", d ? "," : "", c->cg_true_rel[d]);
        js += tmp;
    }
    js += "],\"cg_fp64_residual\":[";
    for (size_t d = 0; d < c->cg_fp64_rel.size(); ++d) {
        snprintf(tmp, sizeof tmp, "%s%.6g", d ? "," : "", c->cg_fp64_rel[d]);
        js += tmp;
    }
    js += "],\"cg_refinements\":[";
    for (size_t d = 0; d < c->cg_refines.size(); ++d) {
        snprintf(tmp, sizeof tmp, "%s%d", d ? "," : "", c->cg_refines[d]);
        js += tmp;
    }
    snprintf(tmp, sizeof tmp,
             "],\"ms\":{\"octree\":%.4f,\"basis\":%.4f,\"splat\":%.4f,\"divergence\":%.4f,\"solve\":%.4f,"
             "\"iso\":%.4f,\"mesh\":%.4f},",
             c->t.octree_ms, c->t.basis_ms, c->t.splat_ms, c->t.divergence_ms, c->t.solve_ms, c->t.iso_ms,
             c->t.mesh_ms);
    js += tmp;
    js += "\"kernels\":{";
    for (size_t k = 0; k < c->ktimers.size(); ++k) {
        const KernelTimer& t = c->ktimers[k];
        snprintf(tmp, sizeof tmp, "%s\"%s\":{\"ms\":%.5f,\"launches\":%lld,\"bytes\":%.6g}", k ? "," : "",
                 t.name.c_str(), t.ms, t.launches, t.bytes);
        js += tmp;
    }
    js += "},";
    snprintf(tmp, sizeof tmp, "\"iso\":%.9g,\"vertices\":%lld,\"triangles\":%lld,\"subdivide_roots\":%lld}",
             (double)c->iso, (long long)c->mesh_v.size() / 3, (long long)c->mesh_f.size() / 3,
             (long long)c->subdivide_roots);
    js += tmp;
    if ((int64_t)js.size() + 1 > len) return PRGPU_ERR_ARG;
    memcpy(buf, js.c_str(), js.size() + 1);
    return PRGPU_OK;
}

int prgpu_set_profiling(void* h, int32_t enable) {
    Ctx* c = as_ctx(h);
    if (!c) return PRGPU_ERR_ARG;
    c->profile = enable != 0;
    c->ktimers.clear();
    return PRGPU_OK;
}

int prgpu_get_stream(void* h, void** stream) {
    Ctx* c = as_ctx(h);
    if (!c || !stream) return PRGPU_ERR_ARG;
    *stream = (void*)c->stream;
    return PRGPU_OK;
}

int64_t prgpu_kernel_launches(void) { return (int64_t)prgpu::g_kernel_launches.load(); }

int prgpu_test_hook(int32_t what, int64_t arg, int64_t* out) {
    switch (what) {
    case PRGPU_HOOK_CLEAR:
        g_fail_alloc_countdown = 0;
        g_spin_limit = DEFAULT_SPIN_LIMIT;
        g_wait_extra = 0;
        return PRGPU_OK;
    case PRGPU_HOOK_FAIL_ALLOC:
        if (arg < 1) return PRGPU_ERR_ARG;
        g_fail_alloc_countdown = arg;
        return PRGPU_OK;
    case PRGPU_HOOK_BARRIER_WAIT:
        if (arg < 1) return PRGPU_ERR_ARG;
        g_spin_limit = arg;
        g_wait_extra = 1;
        return PRGPU_OK;
    case PRGPU_HOOK_POOL_USED: {
        if (!out) return PRGPU_ERR_ARG;
        API_BEGIN
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceSynchronize());
        cudaMemPool_t pool;
        CK(cudaDeviceGetDefaultMemPool(&pool, dev));
        uint64_t used = 0;
        CK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used));
        *out = (int64_t)used;
        return PRGPU_OK;
        API_END
    }
    default:
        set_last_error("prgpu_test_hook: unknown hook %d", what);
        return PRGPU_ERR_ARG;
    }
}

// ----------------------------- learned preconditioner ------------------------
static Trainer* as_tr(void* p) { return (Trainer*)p; }

int prgpu_load_preconditioner(void* h, const char* path) {
    Ctx* c = as_ctx(h);
    if (!c || !path) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(c->device));
    std::vector<float> hp, hm, hv;
    i64 step = 0, epoch = 0;
    uint64_t seed = 0;
    read_checkpoint(path, hp, hm, hv, step, seed, epoch);
    if (!c->lp_params) {
        CK(cudaMalloc(&c->lp_params, P_COUNT * sizeof(float)));
        CK(cudaMalloc(&c->lp_w1b, 4096 * sizeof(__nv_bfloat16)));
        CK(cudaMalloc(&c->lp_w2b, 4096 * sizeof(__nv_bfloat16)));
    }
    std::vector<__nv_bfloat16> b1(4096), b2(4096);
    for (int k = 0; k < 4096; ++k) {
        b1[k] = __float2bfloat16_rn(hp[P_W1 + k]);
        b2[k] = __float2bfloat16_rn(hp[P_W2 + k]);
    }
    CK(cudaMemcpyAsync(c->lp_params, hp.data(), P_COUNT * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->lp_w1b, b1.data(), 4096 * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->lp_w2b, b2.data(), 4096 * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_create(int32_t device, uint64_t seed, void** out) {
    if (!out) return PRGPU_ERR_ARG;
    API_BEGIN
    *out = new Trainer(device, seed);
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_destroy(void* t) {
    if (!t) return PRGPU_ERR_ARG;
    delete as_tr(t);
    return PRGPU_OK;
}

int prgpu_trainer_record(void* t, void* h, int32_t rows_per_depth, int64_t* added) {
    Trainer* T = as_tr(t);
    Ctx* c = as_ctx(h);
    if (!T || !c || rows_per_depth < 1) return PRGPU_ERR_ARG;
    REQUIRE_STAGE(c, 3);
    if (c->device != T->device) {
        set_last_error("trainer on device %d, context on device %d", T->device, c->device);
        return PRGPU_ERR_ARG;
    }
    API_BEGIN_CTX(c)
    CK(cudaSetDevice(c->device));
    const i64 n = T->record(*c, rows_per_depth);
    if (added) *added = n;
    c->stage = std::max(c->stage, 4);
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_train(void* t, int32_t steps, int32_t batch, float lr, double* loss) {
    Trainer* T = as_tr(t);
    if (!T || steps < 0 || batch < 1 || !(lr > 0.f)) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(T->device));
    const double l = T->train(steps, batch, lr);
    if (loss) *loss = l;
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_save(void* t, const char* path) {
    if (!t || !path) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(as_tr(t)->device));
    as_tr(t)->save(path);
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_load(void* t, const char* path) {
    if (!t || !path) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(as_tr(t)->device));
    as_tr(t)->load(path);
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_info(void* t, int64_t* samples, int64_t* step) {
    if (!t) return PRGPU_ERR_ARG;
    if (samples) *samples = as_tr(t)->nsamples;
    if (step) *step = as_tr(t)->step;
    return PRGPU_OK;
}

int prgpu_trainer_get_params(void* t, float* params) {
    if (!t || !params) return PRGPU_ERR_ARG;
    API_BEGIN
    Trainer* T = as_tr(t);
    CK(cudaSetDevice(T->device));
    CK(cudaMemcpyAsync(params, T->p, P_COUNT * sizeof(float), cudaMemcpyDeviceToHost, T->stream));
    CK(cudaStreamSynchronize(T->stream));
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_set_params(void* t, const float* params) {
    if (!t || !params) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(as_tr(t)->device));
    as_tr(t)->set_params(params, nullptr, nullptr);
    return PRGPU_OK;
    API_END
}

int prgpu_trainer_samples(void* t, int64_t first, int64_t n, uint16_t* features, float* targets) {
    Trainer* T = as_tr(t);
    if (!T || first < 0 || n < 0 || first + n > T->nsamples) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(T->device));
    if (features && n)
        CK(cudaMemcpyAsync(features, T->feat + first * 64, (size_t)n * 128, cudaMemcpyDeviceToHost, T->stream));
    if (targets && n)
        CK(cudaMemcpyAsync(targets, T->target + first, (size_t)n * 4, cudaMemcpyDeviceToHost, T->stream));
    CK(cudaStreamSynchronize(T->stream));
    return PRGPU_OK;
    API_END
}

int prgpu_mlp_forward(void* t, const uint16_t* features, int64_t n, float* y) {
    Trainer* T = as_tr(t);
    if (!T || !features || !y || n < 1) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(T->device));
    cudaStream_t s = T->stream;
    __nv_bfloat16* df = dalloc<__nv_bfloat16>(n * 64, s);
    float* dy = dalloc<float>(n, s);
    CK(cudaMemcpyAsync(df, features, (size_t)n * 128, cudaMemcpyHostToDevice, s));
    T->forward(df, n, dy);
    CK(cudaMemcpyAsync(y, dy, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    dfree(df, s);
    dfree(dy, s);
    return PRGPU_OK;
    API_END
}

int prgpu_mlp_gradients(void* t, const uint16_t* features, const float* targets, int64_t n, float* grad, double* loss) {
    Trainer* T = as_tr(t);
    if (!T || !features || !targets || !grad || n < 1) return PRGPU_ERR_ARG;
    API_BEGIN
    CK(cudaSetDevice(T->device));
    cudaStream_t s = T->stream;
    __nv_bfloat16* df = dalloc<__nv_bfloat16>(n * 64, s);
    float* dt = dalloc<float>(n, s);
    CK(cudaMemcpyAsync(df, features, (size_t)n * 128, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dt, targets, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    const double l = T->gradients(df, dt, n, grad);
    if (loss) *loss = l;
    dfree(df, s);
    dfree(dt, s);
    CK(cudaStreamSynchronize(s));
    return PRGPU_OK;
    API_END
}

int prgpu_cg_csr(int32_t n, int32_t nz, const int32_t* rowptr, const int32_t* col, const float* val, const float* rhs,
                 float* x, float tol, int32_t max_iter, int32_t* iters, float* kernel_ms) {
    (void)nz;
    if (n <= 0 || !rowptr || !col || !val || !rhs || !x || max_iter < 0) return PRGPU_ERR_ARG;
    API_BEGIN
    return cg_csr_impl(n, rowptr, col, val, rhs, x, tol, max_iter, iters, kernel_ms);
    API_END
}

}  // extern "C"
