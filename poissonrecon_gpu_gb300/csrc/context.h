// Reconstruction context shared by the stage translation units.
#pragma once
#include <string>
#include <vector>

#include "common.cuh"

namespace prgpu {

// Node arrays in HBM, structure of arrays, global index = base[d] + slot.
struct NodeArrays {
    i64 M = 0;
    u64* key = nullptr;      // full-depth key
    int* pidx = nullptr;     // first sorted point of the node
    int* pnum = nullptr;     // number of points
    int* didx = nullptr;     // first finest-depth slot below the node
    int* dnum = nullptr;     // number of finest-depth slots below the node
    int* parent = nullptr;   // -1 for the root
    int* child0 = nullptr;   // first of 8 contiguous children, -1 if none
    int8_t* depth = nullptr;
    int* neigh = nullptr;    // 27 x M, neighbour j of node i at neigh[j*M + i]
};

// per-kernel device time with CUDA events on the context stream, and the
// kernel's algorithmic (compulsory) byte count per launch
struct KernelTimer {
    std::string name;
    double ms = 0;
    long long launches = 0;
    double bytes = 0;
};
struct PendingTimer {
    int slot;
    cudaEvent_t a, b;
    double bytes;
};

struct StageTimes {
    float octree_ms = 0, basis_ms = 0, splat_ms = 0, divergence_ms = 0, solve_ms = 0, iso_ms = 0, mesh_ms = 0;
};

// page-locked host array that grows and keeps its capacity (mesh output)
template <class T>
struct PinnedBuf {
    T* ptr = nullptr;
    i64 n = 0, cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() {
        if (ptr) cudaFreeHost(ptr);
    }
    void resize(i64 m) {
        if (m > cap) {
            if (ptr) cudaFreeHost(ptr);
            ptr = nullptr;
            cap = 0;
            n = 0;
            const i64 want = std::max<i64>(m, cap + cap / 4);
            CK(cudaMallocHost((void**)&ptr, (size_t)want * sizeof(T)));
            cap = want;
        }
        n = m;
    }
    void clear() { n = 0; }
    i64 size() const { return n; }
    T* data() { return ptr; }
    const T* data() const { return ptr; }
    T& operator[](i64 k) { return ptr[k]; }
};

struct Ctx {
    prgpu_params params;
    std::vector<Ctx*> workers;          // contexts of prgpu_reconstruct_batch's host threads
    int device = 0;
    cudaStream_t stream = nullptr;
    int sms = 152;                      // multiprocessors of the device
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int D = 8;
    int res = 0;

    // input
    i64 N = 0;
    float* in_xyz = nullptr;   // 3N raw
    float* in_nrm = nullptr;
    // normalised, sorted
    float* pts = nullptr;      // 3N
    float* nrm = nullptr;      // 3N (length 2^(D+1))
    uint32_t* sort_idx = nullptr;
    float center[3] = {0, 0, 0};
    float scale = 1.f;

    std::vector<i64> base, count;
    NodeArrays nodes;
    int* point_node = nullptr;

    // basis
    CPoly* basis = nullptr;          // res functions (degree 3 storage)
    CPoly basis_maxdepth;            // splat kernel, degree 2
    float* ddot_div = nullptr;       // compact inner-product rows used by the divergence
    std::vector<i64> ddot_row_start; // per depth
    std::vector<float> stencil;      // 27 per depth
    double* full_tables = nullptr;   // dot, ddot, d2dot (res*res each), on demand
    double2* cascade_tab = nullptr;  // cross-depth 1-D (dot, d2dot) for params.cascadic
    std::vector<i64> cascade_off;    // (D+1)^2: start of the (depth, coarser depth) table

    // rhs / solve
    float* vfield = nullptr;         // 3 x count[D]
    float* point_weight = nullptr;   // N: density weights (params.density_weights), mean 1
    float* wnrm = nullptr;           // 3N: the normals times the density weights
    float* divergence = nullptr;     // M
    float* x = nullptr;              // M
    i64 x_rows = 0;                  // rows x was allocated for
    std::vector<int> cg_iters;
    std::vector<float> cg_rr;
    std::vector<int> cg_fallback;    // learned solve: iteration at which plain CG took a depth over (-1: never)
    std::vector<double> cg_true_rel; // final relative residual of the CG recurrence per depth (FP64 reductions)
    std::vector<double> cg_fp64_rel; // params.refine: |b - Ax| / |b| recomputed in FP64 (-1: not computed)
    std::vector<int> cg_refines;     // params.refine: restarts on the recomputed residual
    int solver_blocks = 0;           // co-resident blocks of the last persistent solve

    // learned preconditioner weights (prgpu_load_preconditioner), owned by the context
    float* lp_params = nullptr;      // fp32 parameter vector
    void* lp_w1b = nullptr;          // bf16 [64][64]
    void* lp_w2b = nullptr;
    int* d_cg_iters = nullptr;
    float* d_cg_rr = nullptr;

    // iso
    float* point_value = nullptr;
    float iso = 0.f;

    // mesh (host, input coordinates)
    PinnedBuf<float> mesh_v;
    PinnedBuf<int32_t> mesh_f;
    int* d_has_tri = nullptr;           // per node at depth < D (device)
    int* d_has_int = nullptr;
    i64 n_coarse = 0;
    i64 subdivide_roots = 0;
    std::vector<i64> batch_tri;
    std::vector<i64> roots_per_depth;   // subdivided leaves by depth
    i64 virtual_cells = 0;
    int* gn = nullptr;                  // sibling-group table (ensure_group_table), freed with the nodes
    int* gn_rows = nullptr;             // the same table row by row, GN_ROW ints per group (ensure_group_rows)
    i64 total_bricks = 0, live_bricks = 0;   // subdivided leaves: bricks, and those not culled
    i64 foreign_corners = 0;                 // brick corners owned by another leaf of the batch
    i64 foreign_slow = 0;                    // of those, evaluated because the owner's brick was culled
    i64 super_bricks = 0, super_decided = 0; // 4^3-brick groups bounded first, and those proven (profiling)

    StageTimes t;
    bool profile = false;
    std::vector<KernelTimer> ktimers;
    std::vector<PendingTimer> kpending;
    std::vector<cudaEvent_t> kevents;   // pool
    size_t kev_next = 0;
    int kbegin(const char* name, double bytes);   // returns a handle for kend, -1 when not profiling
    void kend(int handle);
    void kflush();                                // after a stream sync
    int stage = 0;   // 0 none, 1 points, 2 octree, 3 rhs, 4 solved, 5 iso, 6 mesh
    i64 kernel_launches = 0;

    void free_nodes();
    void free_all();
};

// stage entry points (each throws prgpu::Error on failure)
void stage_octree(Ctx& c);
void stage_basis(Ctx& c);
void stage_full_tables(Ctx& c);
void ensure_cascade_tables(Ctx& c);
void stage_splat(Ctx& c);
void stage_divergence(Ctx& c);
void stage_solve(Ctx& c);
void stage_solve_depths(Ctx& c, int d0, int d1, int mode, const float* rhs = nullptr);
void stage_solve_learned(Ctx& c);   // flexcg.cu
// co-resident blocks of the persistent solvers split between depths d0..d1 in proportion
// to their rows (one block for a depth of at most 4*256 rows); fills deps and block_depth
struct CgDepth;
void partition_depths(const Ctx& c, int d0, int d1, int G, std::vector<CgDepth>& deps, std::vector<int>& block_depth);
void cascade_rhs(Ctx& c, int d, float* rhs);   // depth d's rows of an M-row device buffer
void ensure_group_table(Ctx& c);
void ensure_group_rows(Ctx& c);
void stage_points(Ctx& c);
void stage_mesh(Ctx& c);

// host-side basis setup (reference host arithmetic, unfused)
struct HostBasis {
    CPoly base;       // F/F(0), degree 2, 4 pieces
    CPoly dbase;      // derivative, degree 1
    int npieces;
};
HostBasis host_base_function();
void host_stencils(int D, std::vector<float>& stencil);

}  // namespace prgpu
