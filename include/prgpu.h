/*
 * prgpu.h -- C ABI of the GB300 Poisson surface reconstruction library
 * (libprgpu.so, sm_103a).
 *
 * The reference (DavidXu-JJ/PoissonRecon_GPU) has no library interface: it is a
 * single executable whose stages are host functions inside main.cu.  Each entry
 * point below replaces one of those stages; the comment on each names the
 * reference code it stands in for.  Conventions:
 *   - every function returns a prgpu_status (0 = success) and never throws;
 *     when a stage fails (CUDA error, allocation, limit, timeout), the context
 *     releases its device buffers and needs its points again; nothing the
 *     failed call allocated stays behind;
 *   - a context owns one CUDA stream and all device buffers of one
 *     reconstruction; it is not thread safe, distinct contexts are independent;
 *   - host pointers are caller owned; arrays returned through prgpu_mesh are
 *     library owned and stay valid until the next call on the same context or
 *     prgpu_destroy().
 */
#ifndef PRGPU_H
#define PRGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PRGPU_OK = 0,
    PRGPU_ERR_ARG = 1,           /* invalid argument or call order */
    PRGPU_ERR_CUDA = 2,          /* CUDA runtime error (see prgpu_last_error) */
    PRGPU_ERR_NOMEM = 3,         /* device allocation failed */
    PRGPU_ERR_LIMIT = 4,         /* input beyond a supported size */
    PRGPU_ERR_NOT_CONVERGED = 5, /* solver hit its iteration cap (results still written) */
    PRGPU_ERR_TIMEOUT = 6,       /* a device-side wait gave up (kernel returned early) */
    PRGPU_ERR_IO = 7             /* file could not be read or written */
} prgpu_status;

typedef enum {
    PRGPU_SOLVE_REFERENCE = 0,   /* CG per depth from x0=0 until float(r.r) <= tol^2 or max_iter (CG_CUDA.cuh:256-324) */
    PRGPU_SOLVE_RELATIVE = 1     /* CG per depth until ||r|| <= tol*||b||, FP64 reductions */
} prgpu_solve_mode;

typedef struct {
    int32_t depth;        /* maxDepth, root = depth 0 (main.cu:69); 1..15 */
    int32_t solve_mode;   /* prgpu_solve_mode */
    double cg_tol;        /* 1e-5 absolute (reference) or relative tolerance */
    int32_t cg_max_iter;  /* 10000 in the reference (CG_CUDA.cuh:263) */
    int32_t device;       /* CUDA device ordinal */
    int32_t weld;         /* 0: a vertex per lattice edge and subdivision batch, as the reference
                             (its batches share no vertices, main.cu:3799-4564); 1: one vertex per
                             lattice edge across batches (no cracks at batch boundaries; the
                             triangles are the same, a vertex on a batch boundary takes the
                             position computed by one of its batches) */
    int32_t density_weights; /* 0: every sample weighs 1, as the reference; 1: each sample's normal
                                and its share of the iso-value are weighted by the inverse of the
                                sampling density around it, estimated at depth maxDepth-2 (Kazhdan's
                                adaptive weighting of non-uniform samples; not in the reference) */
    int32_t cascadic;     /* 0: every depth solves L_d x_d = b_d on its own, as the reference
                             (main.cu:1237-1329); 1: the depths are solved coarse to fine and depth
                             d's right-hand side first loses the coarser depths' solution,
                             b_d - sum_{d'<d} L_{d,d'} x_{d'}, with the exact cross-depth
                             inner products over the 27 neighbours of each ancestor (Kazhdan's
                             coarse-to-fine formulation; not in the reference) */
    int32_t learned;      /* 0: plain CG, as the reference (CG_CUDA.cuh:256-324); 1: flexible CG
                             preconditioned by the per-node network loaded with
                             prgpu_load_preconditioner, with the same stopping rule, and plain CG
                             taking over a depth whenever a learned step fails to reduce its
                             residual (not in the reference) */
    int32_t refine;       /* PRGPU_SOLVE_RELATIVE only.  0: stop on the CG recurrence's residual,
                             as the reference does (CG_CUDA.cuh:284); 1: then recompute the true
                             residual b - Ax with FP64 accumulation on the GPU and, while it is
                             above tol*||b||, restart CG from the current x on it (at most two
                             refinements); the true relative residual per depth is reported
                             (the reference checks max|Ax-b| on the host afterwards,
                             CG_CUDA.cuh:476-490) */
    int32_t stable_basis; /* 0: basis values as the reference computes them in single precision:
                             the B-spline shifted to the point, then evaluated
                             (ConfirmedPPolynomial.cuh:37-91), whose coefficients grow as 4^depth,
                             so their rounding error does too (about 1e-3 of the vector field at
                             maxDepth 8, 2e-2 at 10); 1: the closed form of the same B-spline at an
                             offset formed with one rounding (not in the reference) */
    int32_t reserved[2];
} prgpu_params;

typedef struct {
    int64_t n_vertices;
    int64_t n_triangles;
    const float* vertices;     /* 3*n_vertices, in input coordinates */
    const int32_t* triangles;  /* 3*n_triangles vertex indices */
} prgpu_mesh;

/* Defaults: depth 8, reference CG schedule (tol 1e-5, 10000 iterations), device 0. */
int prgpu_params_default(prgpu_params* p);

/* Context lifetime.  Replaces the process-global state of main.cu:3247-3270. */
int prgpu_create(const prgpu_params* p, void** ctx);
int prgpu_destroy(void* ctx);

/* Oriented points, 3 floats per point each, host memory.  The reference reads
 * them from a PointStream (main.cu:516-571; PointStream.inl). */
int prgpu_set_points(void* ctx, const float* xyz, const float* nrm, int64_t n);
/* Same, from device memory already resident on the context's device. */
int prgpu_set_points_device(void* ctx, const float* d_xyz, const float* d_nrm, int64_t n);

/* Normalisation, Morton keys, radix sort, node arrays and 27-neighbour tables.
 * Replaces pipelineBuildNodeArray (main.cu:511-841). */
int prgpu_build_octree(void* ctx);

/* Basis tables, vector-field splat and divergence for every depth.
 * Replaces main.cu:3306-3462 (FunctionData tables, computeVectorField,
 * computeEncodedFinerNodesDivergence and the coarse divergence loop). */
int prgpu_compute_rhs(void* ctx);

/* Per-depth Laplacian solve (matrix-free 27-point stencil).
 * Replaces LaplacianIteration (main.cu:1223-1332) and solverCG_DeviceToDevice. */
int prgpu_solve(void* ctx);

/* One depth's system L_d x_d = b_d (0 <= depth <= maxDepth) with the given
 * prgpu_solve_mode; the other depths' rows of x keep their values (0 before any
 * solve).  The body of LaplacianIteration's per-depth loop (main.cu:1237-1329).
 * With params.cascadic the right-hand side is b_d less the coarser depths'
 * current rows of x (as prgpu_solve uses it). */
int prgpu_solve_depth(void* ctx, int32_t depth, int32_t mode);

/* Implicit function at the input points and the iso-value.
 * Replaces calculatePointsImplicitFunctionValue + reduce (main.cu:1334-1381,3480-3499). */
int prgpu_eval_points(void* ctx, float* iso_out);

/* Marching cubes on the finest nodes and on subdivided coarse leaves.
 * Replaces main.cu:3504-4561. */
int prgpu_extract_mesh(void* ctx);

/* Copies the mesh to library-owned host memory (input coordinates). */
int prgpu_get_mesh(void* ctx, prgpu_mesh* out);

/* All stages in order; equivalent to the body of main() (main.cu:3247-4573)
 * without file I/O. */
int prgpu_reconstruct(void* ctx, const float* xyz, const float* nrm, int64_t n, prgpu_mesh* out);

/* Several point clouds: cloud k is points [offsets[k], offsets[k+1]) of xyz/nrm,
 * reconstructed at maxDepth depths[k] (the context's depth when depths is NULL).
 * Clouds of at most 4M points run four at a time on worker contexts the context
 * keeps (own stream, buffers and host thread each, released by prgpu_destroy),
 * larger ones one at a time; every mesh is that of a separate reconstruction.
 * outs[k] receives a copy of the mesh in memory the caller releases with
 * prgpu_mesh_free.  The reference has no counterpart (one cloud per process run,
 * main.cu:3247-4573); it is the batched form of prgpu_reconstruct.  On error, the
 * meshes already produced are released and the error names the cloud. */
int prgpu_reconstruct_batch(void* ctx, const float* xyz, const float* nrm, const int64_t* offsets,
                            const int32_t* depths, int32_t ncloud, prgpu_mesh* outs);

/* Releases a mesh returned by prgpu_reconstruct_batch and zeroes it. */
int prgpu_mesh_free(prgpu_mesh* mesh);

/* The octree as the reference's OctNode fields (OctNode.cuh:8-41), structure of
 * arrays in caller-allocated host memory: n_nodes and max_depth are filled in,
 * and every non-NULL array is copied (base: max_depth + 2 entries, the first node
 * of each depth and the total; children: 8 and neighs: 27 per node; the others
 * one per node).  Call once with NULL arrays to learn n_nodes.  Replaces the
 * NodeArray output of pipelineBuildNodeArray (main.cu:511-513). */
typedef struct {
    int64_t n_nodes;
    int32_t max_depth;
    int64_t* base;
    uint64_t* key;
    int32_t* pidx;
    int32_t* pnum;
    int32_t* parent;
    int32_t* children;
    int32_t* neighs;
    int32_t* didx;
    int32_t* dnum;
} prgpu_node_arrays;
int prgpu_get_node_arrays(void* ctx, prgpu_node_arrays* out);

/* Copy an internal array to host memory.  Names: "key","pidx","pnum","parent",
 * "children","neighs","didx","dnum","base","count","points","normals",
 * "point_node","vfield","divergence","x","point_value","stencil","cg_iters",
 * "cg_rr","has_tri","has_int","dot","ddot","d2dot","center","scale","iso".
 * Node arrays follow the reference OctNode field meaning (OctNode.cuh:8-41);
 * "children" and "neighs" are 8 and 27 int32 per node.  *bytes receives the
 * size; with dst == NULL only the size is returned. */
int prgpu_get_array(void* ctx, const char* name, void* dst, int64_t max_bytes, int64_t* bytes);
/* Replace an internal float array ("vfield","divergence","x","iso") before the
 * next stage runs (stage-by-stage parity tests). */
int prgpu_set_array(void* ctx, const char* name, const void* src, int64_t bytes);

/* Per-stage device times, counts and solver statistics as one JSON object. */
int prgpu_stats_json(void* ctx, char* buf, int64_t len);

/* Per-kernel timing: when enabled, the main kernels are bracketed by CUDA
 * events on the context stream and their times, launch counts and algorithmic
 * byte counts appear under "kernels" in prgpu_stats_json.  Enabling resets them. */
int prgpu_set_profiling(void* ctx, int32_t enable);

/* The context's CUDA stream (a cudaStream_t), for callers that order their own
 * work or timing events after the library's. */
int prgpu_get_stream(void* ctx, void** stream);

/* Number of kernels this process has launched through the library. */
int64_t prgpu_kernel_launches(void);

/* Human-readable text of the last error on this thread. */
const char* prgpu_last_error(void);

/* Failure-path hooks for tests.  The reference has no counterpart: its failures
 * end the process (exit() in PointStream.inl:33, CG_CUDA.cuh:359-373).  The
 * hooks are process-wide and off by default.  'what':
 *   PRGPU_HOOK_CLEAR          all hooks off;
 *   PRGPU_HOOK_FAIL_ALLOC     the arg-th device allocation from now on fails (once) as if
 *                             the device were out of memory (arg >= 1);
 *   PRGPU_HOOK_BARRIER_WAIT   the solvers' grid barriers expect one block more than the
 *                             launch has -- an arrival that never comes -- and give up
 *                             after arg polls of about 32 ns, so a solve returns
 *                             PRGPU_ERR_TIMEOUT without hanging (arg >= 1);
 *   PRGPU_HOOK_POOL_USED      *out = bytes the current device's memory pool has handed out
 *                             and not taken back (after a device synchronisation).
 * out may be NULL except for PRGPU_HOOK_POOL_USED. */
enum {
    PRGPU_HOOK_CLEAR = 0,
    PRGPU_HOOK_FAIL_ALLOC = 1,
    PRGPU_HOOK_BARRIER_WAIT = 2,
    PRGPU_HOOK_POOL_USED = 3
};
int prgpu_test_hook(int32_t what, int64_t arg, int64_t* out);

/* Conjugate gradients on a CSR matrix in device memory, x0 = 0, stopping when
 * float(r.r) <= tol^2 or after max_iter iterations; FP32 vectors, FP64 dots.
 * Replaces solverCG_DeviceToDevice(N, nz, I, J, val, rhs, x) (CG_CUDA.cuh:344-509).
 * I has N+1 row offsets.  iters / kernel_ms may be NULL. */
int prgpu_cg_csr(int32_t n, int32_t nz, const int32_t* d_rowptr, const int32_t* d_col,
                 const float* d_val, const float* d_rhs, float* d_x, float tol, int32_t max_iter,
                 int32_t* iters, float* kernel_ms);

/* The same solver for callers that cannot allocate device memory at solve time
 * (a framework's caching allocator owns the device memory, cudaFree's implicit
 * synchronisation is not affordable, or the host forbids allocation after
 * start-up).  No counterpart in the reference.  It allocates nothing: the
 * scratch vectors and solver state live in one static device array of the
 * library (about 3 MiB per GPU that loads the library, held until exit), so n
 * is limited to 262144 rows (PRGPU_ERR_LIMIT beyond).  All calls share that
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller.  Runs on 'stream' (a cudaStream_t, NULL = legacy default stream) and
 * returns after the solve has finished, so it cannot be captured into a CUDA
 * graph: on a capturing stream it returns PRGPU_ERR_ARG. */
int prgpu_cg_csr_noalloc(int32_t n, int32_t nz, const int32_t* d_rowptr, const int32_t* d_col,
                         const float* d_val, const float* d_rhs, float* d_x, float tol, int32_t max_iter,
                         void* stream, int32_t* iters);

/* ---- learned preconditioner --------------------------------------------------
 * None of these has a counterpart in the reference, which solves every depth with
 * plain CG (CG_CUDA.cuh:256-324).  The network: per node, 64 features (the 27
 * neighbours' residuals scaled by their largest magnitude, the 27 normalised
 * stencil coefficients of the neighbours present, depth/16, zero padding) ->
 * 64 -> 64 -> 1 with ReLU, BF16 weights and FP32 accumulation on the tensor cores;
 * parameters as 8385 floats: W1[64][64] (out, in), b1[64], W2[64][64], b2[64],
 * w3[64], b3.  Features are passed as BF16 bit patterns, 64 per row.
 * Checkpoint file: "PRGPULPC", u32 version 1, u32 64, u32 64, u32 8385, i64 step,
 * u64 seed, i64 epoch, then the parameters and Adam's two moment vectors (f32,
 * little endian). */

/* Loads a checkpoint's weights into the context (used when params.learned = 1). */
int prgpu_load_preconditioner(void* ctx, const char* checkpoint_path);

/* A trainer: parameters (initialised from the seed), Adam state and training
 * samples on one device. */
int prgpu_trainer_create(int32_t device, uint64_t seed, void** trainer);
int prgpu_trainer_destroy(void* trainer);
/* Residual/error pairs of plain CG on ctx's system (after prgpu_compute_rhs):
 * the solution to relative 1e-7, then the iterates after 1, 2, 3, 5, 8, 12 and 20
 * iterations; rows_per_depth random rows of every depth >= 1 per iterate.  The
 * context's x is left at the solution.  *added may be NULL. */
int prgpu_trainer_record(void* trainer, void* ctx, int32_t rows_per_depth, int64_t* added);
/* Adam steps on shuffled minibatches of the recorded samples (mean squared
 * error); *loss (may be NULL) receives the last minibatch's loss. */
int prgpu_trainer_train(void* trainer, int32_t steps, int32_t batch, float lr, double* loss);
int prgpu_trainer_save(void* trainer, const char* path);
/* Resumes from a checkpoint: parameters, Adam state, step count and seed. */
int prgpu_trainer_load(void* trainer, const char* path);
int prgpu_trainer_info(void* trainer, int64_t* samples, int64_t* step);
int prgpu_trainer_get_params(void* trainer, float* params);
int prgpu_trainer_set_params(void* trainer, const float* params);
/* Copies recorded samples [first, first+n) to host memory (features: 64 BF16 bit
 * patterns per row; targets: one float per row). */
int prgpu_trainer_samples(void* trainer, int64_t first, int64_t n, uint16_t* features, float* targets);
/* The network on host feature rows: forward outputs y[n]; or the gradient of the
 * mean squared error against targets (grad: 8385 floats) and the loss. */
int prgpu_mlp_forward(void* trainer, const uint16_t* features, int64_t n, float* y);
int prgpu_mlp_gradients(void* trainer, const uint16_t* features, const float* targets, int64_t n, float* grad,
                        double* loss);

/* Density-based depth (not in the reference, whose maxDepth is a compile-time constant,
 * main.cu:69): the octree of the cloud is built at max_depth on the device, occupied[d]
 * (nodes of depth d holding at least one point, max_depth+1 entries, may be NULL) counted, and
 * *depth set to the largest d in 2..max_depth whose mean points per occupied node
 * n / occupied[d] is at least samples_per_node (2 when none is).  Kazhdan's samples-per-node
 * rule applied to the whole cloud: sparse clouds get a coarser octree. */
int prgpu_choose_depth(const float* xyz, const float* nrm, int64_t n, int32_t max_depth, double samples_per_node,
                       int32_t device, int32_t* depth, int64_t* occupied);

/* PLY I/O (PointStream.inl:160-239 input; PlyWriteTriangles plyfile.cu:2769-2836 output).
 * prgpu_read_points returns library-owned arrays valid until the next call. */
int prgpu_read_points(const char* path, int64_t* n, const float** xyz, const float** nrm);
int prgpu_write_mesh_ply(const char* path, const prgpu_mesh* mesh, int32_t binary);

#ifdef __cplusplus
}
#endif
#endif /* PRGPU_H */
