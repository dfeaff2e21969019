/*
 * smearfem_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the
 * smearFEM.jl hot path: Q1/Q2 element stiffness with 2x2(x2) Gauss
 * quadrature, global sparse assembly, Dirichlet elimination and the solve of
 * K u = f.
 *
 * The entry points are what a Julia `ccall` binding (or Python ctypes, or C)
 * needs to replace the reference's calling surface:
 *
 *   gaussian_quadrature(a,b,nGaussPoints)         src/fem.jl:21-31
 *   basis_function(xi,eta,zeta,FunctionClass)     src/fem.jl:48-114
 *   assemble_system(ne,NodeList,IEN,ndim,
 *                   FunctionClass,nDof,ID,Young,nu) src/fem.jl:135-256
 *   setboundaryCond / C'*K_bar*C / inv(Matrix(K_free)) / q_d + C*q_f
 *                                                  examples/vector3D.jl:133-173,315-322
 *
 * Conventions
 *  - Arrays use the reference's (Julia) layout: column-major, 1-based indices.
 *      NodeList : double [ndim x nNodes]   (xyz of a node contiguous)
 *      IEN      : int64  [ldIEN x nen]     (element index fastest)
 *      ID       : int64  [nNodes x nDof]
 *    The matrix is returned in SparseMatrixCSC form (colptr, rowval, nzval;
 *    1-based, rows sorted per column, explicit zeros kept).
 *  - `mem_space` says where every pointer argument of that call lives:
 *    SFEM_MEM_HOST (any host memory; copies are staged by the library) or
 *    SFEM_MEM_DEVICE (device memory of the context's GPU).
 *  - Every function returns an sfem_status.  sfem_last_error() gives a
 *    human-readable reason for the last failure on a context.
 *  - Ownership: handles are created and destroyed by the library.  Output
 *    arrays are allocated by the caller; sizes come from sfem_matrix_info.
 *  - A context owns one CUDA stream and is not thread-safe.  Calls are
 *    synchronous: when they return, outputs are complete.
 *  - There is no CPU fallback: if no GPU is usable, sfem_ctx_create fails.
 */
#ifndef SMEARFEM_GPU_H
#define SMEARFEM_GPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define SFEM_API __attribute__((visibility("default")))
#else
#define SFEM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SFEM_OK = 0,
    SFEM_BAD_ARG = 1,            /* invalid argument (sizes, classes, NULLs)          */
    SFEM_BAD_INDEX = 2,          /* IEN/ID entry out of range (Julia: BoundsError)    */
    SFEM_SINGULAR_JACOBIAN = 3,  /* det J == 0 at a Gauss point (Julia: inv throws)   */
    SFEM_OOM = 4,                /* device allocation failed                          */
    SFEM_NOT_CONVERGED = 5,      /* maxit reached before rtol                         */
    SFEM_CUDA_ERROR = 6,         /* CUDA runtime error                                */
    SFEM_SINGULAR = 7,           /* K_free singular: zero pivot / CG breakdown        */
    SFEM_UNSUPPORTED = 8,        /* element class the reference cannot assemble       */
    SFEM_TIMEOUT = 9             /* a wait ended before the request finished          */
} sfem_status;

enum { SFEM_MEM_HOST = 0, SFEM_MEM_DEVICE = 1 };
enum { SFEM_Q1 = 1, SFEM_Q2 = 2 };                      /* FunctionClass              */
enum { SFEM_PLANE_STRESS = 0, SFEM_PLANE_STRAIN = 1 };  /* 2D elasticity law          */
enum { SFEM_FP64 = 0, SFEM_MIXED = 1 };                 /* solver precision           */
enum { SFEM_PC_JACOBI = 0, SFEM_PC_BLOCK_JACOBI = 1,  /* preconditioner             */
       SFEM_PC_MULTIGRID = 2 };  /* batch and server, mixed precision: geometric multigrid on
                                    structured (meshgrid) Q1 meshes, block Jacobi otherwise */
enum { SFEM_FP32_UPPER = 0, SFEM_FP32_FULL = 1 };       /* mixed-precision K storage  */

typedef struct sfem_ctx sfem_ctx;
typedef struct sfem_mesh sfem_mesh;
typedef struct sfem_matrix sfem_matrix;

/* ---- context ------------------------------------------------------------ */

/* Create a context on CUDA device `device` (no reference counterpart: the
 * reference runs in one Julia thread on the CPU). */
SFEM_API int sfem_ctx_create(int device, sfem_ctx **out);
SFEM_API int sfem_ctx_destroy(sfem_ctx *ctx);
SFEM_API const char *sfem_last_error(const sfem_ctx *ctx);
/* Wait for all work on the context's stream. */
SFEM_API int sfem_ctx_synchronize(sfem_ctx *ctx);
/* Library version string. */
SFEM_API const char *sfem_version(void);
/* The context's CUDA stream (a cudaStream_t), so callers can order their own
 * work and CUDA events against the library's (no reference counterpart). */
SFEM_API void *sfem_ctx_stream(sfem_ctx *ctx);
/* Kernels the context has launched so far (graph-launched kernels included). */
SFEM_API int64_t sfem_ctx_kernel_launches(const sfem_ctx *ctx);

/* ---- host helpers (pure host code, identical expressions) --------------- */

/* gaussian_quadrature(a,b,nGaussPoints), src/fem.jl:21-31.
 * xi, w: caller arrays of length nGaussPoints (2 or 3). */
SFEM_API int sfem_gaussian_quadrature(double a, double b, int nGaussPoints, double *xi, double *w);

/* basis_function(xi,eta,zeta,FunctionClass), src/fem.jl:48-114.
 * ndim 1..3 (Q1) or 2 (Q2).  N: nen values; dN: nen x ndim column-major
 * (column k = dN/dxi_k), exactly the reference's hcat layout. */
SFEM_API int sfem_basis_function(int ndim, int function_class, double xi, double eta, double zeta,
                        double *N, double *dN);

/* ---- mesh and sparsity pattern ------------------------------------------ */

/* Upload and validate a mesh: the inputs of assemble_system
 * (src/fem.jl:135, with ne^ndim elements processed, src/fem.jl:179).
 *   ne        elements per direction; the first ne^ndim rows of IEN are used
 *   nen       columns of IEN: 2^ndim for Q1, 9 for Q2
 *   nDof      1 (scalar Laplace) or ndim (elasticity); ID may be NULL if 1
 * IEN entries must lie in 1..nNodes and ID entries of referenced nodes must
 * be >= 1 and distinct (SFEM_BAD_INDEX / SFEM_BAD_ARG otherwise). */
SFEM_API int sfem_mesh_create(sfem_ctx *ctx, int ndim, int function_class, int nDof, int64_t ne,
                     const double *NodeList, int64_t nNodes, const int64_t *IEN,
                     int64_t ldIEN, int nen, const int64_t *ID, int mem_space,
                     sfem_mesh **out);
SFEM_API int sfem_mesh_destroy(sfem_mesh *mesh);

/* Build the sparsity pattern of K on the device: the structure that
 * sparse(E,J,V) produces at src/fem.jl:253 (union of element DOF-pair
 * blocks, explicit zeros kept).  n_out = size(K,1) = maximum row index,
 * nnz_out = nnz(K).  Idempotent; assembly builds it on demand. */
SFEM_API int sfem_pattern_build(sfem_ctx *ctx, sfem_mesh *mesh, int64_t *n_out, int64_t *nnz_out);

/* ---- assembly ----------------------------------------------------------- */

/* Numeric assembly of K on a mesh (src/fem.jl:179-252): per element the
 * Jacobian, |det J|-weighted Gauss sum of B'DB (or grad N_i . grad N_j),
 * summed into the pattern in ascending element order without atomics.
 * Young/nu: length 1 (the reference's scalars) or ne^ndim (per element).
 * plane selects the 2D law (the reference's is plane stress). */
SFEM_API int sfem_assemble(sfem_ctx *ctx, sfem_mesh *mesh, int plane, const double *Young,
                  int64_t nYoung, const double *nu, int64_t nNu, int mem_space,
                  sfem_matrix **out);

/* One call doing mesh upload + pattern + assembly: assemble_system(ne,
 * NodeList, IEN, ndim, FunctionClass, nDof, ID, Young, nu), src/fem.jl:135.
 * The returned matrix keeps the mesh it was built on alive. */
SFEM_API int sfem_assemble_system(sfem_ctx *ctx, int64_t ne, const double *NodeList, int64_t nNodes,
                         const int64_t *IEN, int64_t ldIEN, int nen, int ndim,
                         int function_class, int nDof, const int64_t *ID, const double *Young,
                         int64_t nYoung, const double *nu, int64_t nNu, int plane,
                         int mem_space, sfem_matrix **out, int64_t *n_out, int64_t *nnz_out);

/* Re-assemble an existing matrix K for new Young/nu without allocating any
 * device memory.  This entry point has no counterpart in the reference.
 *
 * It is meant for callers that cannot call cudaMalloc/cudaFree when they
 * refresh K: processes whose device memory is owned by another allocator
 * under a hard budget, latency-bound loops (load increments, material
 * updates) in which cudaFree's device-wide synchronisation would stall other
 * streams, and deployments that forbid dynamic allocation after start-up.
 * Build the mesh, pattern and K once with the allocating calls above; this
 * call then only launches kernels and copies into memory that already
 * exists.  The result equals sfem_assemble with the same Young/nu.
 *
 *  - Scratch: a fixed 64 MiB device array (8,388,608 doubles) inside the
 *    library, held on every GPU that loads it until the process exits.  It
 *    must fit the element blocks (pairs*nDof^2 doubles per element: 324 for
 *    a 3D elasticity hex, 40 for a 2D elasticity quad, 36 for a 3D Laplace
 *    hex) plus the Young/nu values; larger meshes get SFEM_BAD_ARG.  That is
 *    at most 25,890 hex elasticity elements with per-element Young.
 *  - Each call looks up the array's device address (cudaGetSymbolAddress)
 *    with the context's device current.  The first lookup on a device may
 *    load the library's device code there, so make the first call before
 *    any stream capture; later lookups allocate nothing, and a context
 *    created after cudaDeviceReset gets the array's new address.
 *  - Every call, from any context, shares the one array: calls that overlap
 *    on the GPU (other streams, other host threads) race.  Calls on one
 *    context are ordered by its stream and do not.
 *  - Young/nu: length 1 or ne^ndim, in `mem_space` (host or device).  The
 *    FP32 copy of K used by SFEM_MIXED solves is refreshed too.
 *  - On a non-zero return from the argument checks or the element kernel
 *    (det J = 0, a bad index), K keeps its previous values; after any later
 *    failure (a CUDA error in the gather or the FP32 refresh) K's values are
 *    undefined and K should be re-assembled. */
SFEM_API int sfem_reassemble_noalloc(sfem_ctx *ctx, sfem_matrix *K, const double *Young,
                                     int64_t nYoung, const double *nu, int64_t nNu,
                                     int mem_space);

/* n = size(K,1) = size(K,2); nnz = length(nzval). */
SFEM_API int sfem_matrix_info(const sfem_matrix *K, int64_t *n, int64_t *nnz);

/* Copy K out in SparseMatrixCSC form (the return value of assemble_system,
 * src/fem.jl:253-255).  colptr: n+1, rowval: nnz, nzval: nnz; any may be
 * NULL to skip it.  1-based indices. */
SFEM_API int sfem_matrix_export_csc(sfem_ctx *ctx, const sfem_matrix *K, int64_t *colptr,
                           int64_t *rowval, double *nzval, int mem_space);
SFEM_API int sfem_matrix_destroy(sfem_matrix *K);

/* ---- Dirichlet elimination and solve ------------------------------------ */

typedef struct {
    int precision;        /* SFEM_FP64 (default) or SFEM_MIXED                    */
    int precond;          /* SFEM_PC_JACOBI (default) or SFEM_PC_BLOCK_JACOBI;
                             SFEM_PC_MULTIGRID in batches and servers          */
    double rtol;          /* stop at ||f_f - K_ff u_f|| <= rtol ||f_f - K_fd u_d|| */
    int maxit;            /* iteration cap (SFEM_NOT_CONVERGED beyond it)          */
    int check_every;      /* iterations per device-side chunk between host checks */
    double reliable_delta;/* mixed: refresh the FP64 residual when the FP32
                             residual has dropped by this factor (0.1; with
                             SFEM_PC_MULTIGRID, 0.01 refreshes half as often
                             at the same error)                                 */
    int profile;          /* 1: time the SpMV launches with CUDA events           */
    int fp32_storage;     /* SFEM_MIXED: SFEM_FP32_UPPER (default) stores the
                             upper-triangle blocks of K once (K is symmetric);
                             SFEM_FP32_FULL keeps every block                    */
} sfem_solve_opts;

typedef struct {
    int status;           /* sfem_status of the solve                              */
    int iterations;       /* CG iterations (inner iterations for SFEM_MIXED)       */
    int reliable_updates; /* FP64 residual refreshes (SFEM_MIXED)                  */
    double relres;        /* final relative residual (FP64 true residual)          */
    double ms_total;      /* wall time of the solve call                           */
    double ms_spmv;       /* summed CUDA-event time of the SpMV launches (profile) */
    int spmv_launches;    /* SpMV launches timed                                   */
    int kernel_launches;  /* kernels launched by the solve                         */
    int64_t n_free;       /* free DOFs                                             */
} sfem_solve_stats;

SFEM_API void sfem_solve_opts_default(sfem_solve_opts *opts);

/* Solve K u = f with u prescribed on `fixed_dofs` (1-based global DOF ids,
 * values `fixed_vals`): the elimination of examples/vector3D.jl:314-322,
 *   K_free = C'KC;  q_f = K_free \ C'(f - K q_d);  u = q_d + C q_f,
 * with the reference's dense inverse replaced by preconditioned CG on the
 * GPU.  f may be NULL (the reference's case, f = 0).  u_out has n entries. */
SFEM_API int sfem_solve_dirichlet(sfem_ctx *ctx, sfem_matrix *K, const int64_t *fixed_dofs,
                         int64_t nfix, const double *fixed_vals, const double *f,
                         double *u_out, int mem_space, const sfem_solve_opts *opts,
                         sfem_solve_stats *stats);

/* ---- batches of independent meshes ---------------------------------------- */

/* Many independent meshes of one element class, assembled and solved together
 * by one persistent kernel (no reference counterpart: the reference solves one
 * mesh per call, examples/vector3D.jl:305-322).  Each mesh gets its own
 * Jacobian/assembly, Dirichlet elimination and CG; results do not depend on
 * what else is in the batch. */
typedef struct sfem_batch sfem_batch;

typedef struct {
    int status;      /* sfem_status of this mesh's solve                    */
    int iterations;  /* CG iterations                                       */
    int refreshes;   /* FP64 residual refreshes (SFEM_MIXED)                */
    int group_ctas;  /* CTAs that worked on the mesh (1, or the cluster)    */
    double relres;   /* relative residual at exit (FP64 true residual for
                        SFEM_MIXED, recursive residual for SFEM_FP64)        */
    double ms;       /* GPU time from the mesh's start to its result        */
} sfem_batch_stats;

/* Upload nmesh meshes.  Mesh m owns nodes [node_offsets[m], node_offsets[m+1])
 * of NodeList (ndim x total nodes) and elements [elem_offsets[m],
 * elem_offsets[m+1]) of IEN (total elements x nen, column-major); IEN and ID
 * entries are 1-based and local to their mesh.  ID (total nodes x nDof,
 * column-major) may be NULL for the interleaved numbering ID[k,l] =
 * nDof*(k-1)+l (examples/vector3D.jl:73-75); its entries must lie in
 * 1..nDof*(mesh nodes).  Builds the sparsity pattern of every mesh. */
SFEM_API int sfem_batch_create(sfem_ctx *ctx, int ndim, int function_class, int nDof, int64_t nmesh,
                               const int64_t *node_offsets, const int64_t *elem_offsets,
                               const double *NodeList, const int64_t *IEN, const int64_t *ID,
                               int mem_space, sfem_batch **out);

/* total_dofs = nDof * total nodes: the length of u in sfem_batch_solve. */
SFEM_API int sfem_batch_info(const sfem_batch *batch, int64_t *total_dofs, int64_t *total_nodes,
                             int64_t *total_elements);

/* Launch shape of the persistent kernel: threads per CTA (256 or 512), CTAs
 * per SM (capped by occupancy) and the thread-block cluster size (1, 2, 4, 8
 * or 16) that works together on every mesh with at least cluster_min_nodes
 * nodes; smaller meshes get one CTA each.  sfem_batch_autotune picks them. */
SFEM_API int sfem_batch_set_launch(sfem_batch *batch, int threads, int ctas_per_sm, int cluster,
                                   int64_t cluster_min_nodes);

/* Assemble and solve every mesh in one persistent kernel launch.
 *   Young/nu: length 1 (all), nmesh (per mesh) or total elements.
 *   fix_offsets (nmesh+1): mesh m's prescribed DOFs are entries
 *   [fix_offsets[m], fix_offsets[m+1]) of fixed_dofs (1-based, local to the
 *   mesh) and fixed_vals.
 *   u_out (total_dofs): mesh m's displacement starts at nDof*node_offsets[m],
 *   in its ID numbering.
 *   opts: precision, precond, rtol, maxit, reliable_delta are used.
 *   stats: nmesh entries (may be NULL).  The call returns SFEM_OK when the
 *   launch ran; per-mesh outcomes are in stats.
 * The device work of a call is one CUDA graph launch: uploads from device or
 * pinned host memory, the persistent kernel, and the copy of u to device or
 * pinned host memory (pageable host arrays are copied before and after it).
 * The graph is captured at the first call and re-launched while the
 * options, launch shape, argument lengths and those pointers stay the same. */
SFEM_API int sfem_batch_solve(sfem_ctx *ctx, sfem_batch *batch, int plane, const double *Young,
                              int64_t nYoung, const double *nu, int64_t nNu,
                              const int64_t *fix_offsets, const int64_t *fixed_dofs,
                              const double *fixed_vals, double *u_out, int mem_space,
                              const sfem_solve_opts *opts, sfem_batch_stats *stats);
/* Project autotuner for the persistent kernel's launch shape: runs the solve
 * (same arguments as sfem_batch_solve) on a sample of about `sample` meshes
 * taken evenly from the batch's size order, for a set of candidate shapes
 * (threads per CTA, CTAs per SM, cluster size, cluster threshold), times each
 * with CUDA events and keeps the fastest for later sfem_batch_solve calls.
 * best_ms: time of the best candidate on the sample. */
SFEM_API int sfem_batch_autotune(sfem_ctx *ctx, sfem_batch *batch, int plane, const double *Young,
                                 int64_t nYoung, const double *nu, int64_t nNu,
                                 const int64_t *fix_offsets, const int64_t *fixed_dofs,
                                 const double *fixed_vals, int mem_space,
                                 const sfem_solve_opts *opts, int64_t sample, double *best_ms);
/* The launch shape in use, and the grid of the last launch. */
SFEM_API int sfem_batch_get_launch(const sfem_batch *batch, int *threads, int *ctas_per_sm,
                                   int *cluster, int64_t *cluster_min_nodes, int *last_grid);
SFEM_API int sfem_batch_destroy(sfem_batch *batch);

/* ---- multigrid: which meshes get a hierarchy -------------------------------- */

/* Host-only query (no device, no context).  ne_out: elements per direction
 * when the mesh is the structured grid the reference's meshgrid makes
 * (examples/vector3D.jl:66-101: (ne+1)^ndim nodes, ne^ndim Q1 elements, its
 * node numbering and connectivity), else 0.  levels_out / bytes_out: the
 * SFEM_PC_MULTIGRID hierarchy of such a mesh (levels, the fine one included;
 * device bytes on top of the CG's), 0 when it gets none (other meshes, Q2,
 * ne < 3).  IEN: nEl x nen, column-major, 1-based, host memory. */
SFEM_API int sfem_multigrid_info(int ndim, int function_class, int nDof, int64_t nNodes,
                                 const int64_t *IEN, int64_t nEl, int *ne_out, int *levels_out,
                                 int64_t *bytes_out);

/* ---- on-device mesh generation --------------------------------------------- */

/* The reference's structured grid generator (examples/vector3D.jl:10-130) on
 * the GPU.  Outputs in the reference's Julia layouts, 1-based, column-major,
 * any may be NULL: NodeList ndim x (ne+1)^ndim; IEN ne^ndim x 2^ndim; ID
 * (ne+1)^ndim x ndim with ID[m,l] = ndim(m-1)+l; IEN_top / IEN_btm
 * ne^(ndim-1) x 2^(ndim-1) (left zero where the reference leaves them:
 * IEN_top when ne = 1).  Coordinates are linspace-rounded, boundary planes
 * exact.  z0/z1 are ignored in 2D. */
SFEM_API int sfem_meshgrid(sfem_ctx *ctx, double x0, double x1, double y0, double y1, double z0, double z1,
                           int64_t ne, int ndim, double *NodeList, int64_t *IEN, int64_t *ID, int64_t *IEN_top,
                           int64_t *IEN_btm, int mem_space);
/* inflate_sphere (src/PostProcess.jl:30-44), in place like the reference:
 * each node's (x, y) moves radially about the centre of [x0,x1]x[y0,y1] so
 * that a square ring of half-width s lands on the circle of radius s. */
SFEM_API int sfem_inflate_sphere(sfem_ctx *ctx, double *NodeList, int ndim, int64_t nNodes, double x0, double x1,
                                 double y0, double y1, int mem_space);

/* ---- VTK output ------------------------------------------------------------ */

/* write_vtk (src/PostProcess.jl:258-279): one VTK XML UnstructuredGrid file
 * (.vtu, appended raw data) with the mesh and one point field of ncomp
 * components (field: ncomp x nNodes column-major, NULL for none).  Cells by
 * nen: 8 hexahedron, 4 quad, 2 line; 2D points get z = 0.  With host arrays
 * (SFEM_MEM_HOST) no GPU is needed and ctx may be NULL. */
SFEM_API int sfem_vtk_write(sfem_ctx *ctx, const char *path, const double *NodeList, int ndim, int64_t nNodes,
                            const int64_t *IEN, int64_t nEl, int nen, const char *field_name, const double *field,
                            int ncomp, int mem_space);
/* write_scene (src/PostProcess.jl:281-304): step i (1-based) of fields
 * (nsteps blocks of ncomp x nNodes) to <basename>timestep_<i>.vtu as point
 * field "u", and <basename>displacement.pvd listing them at times 0, 1, ...
 * Device fields are copied through two pinned buffers, each step's copy
 * overlapping the previous step's write. */
SFEM_API int sfem_vtk_write_scene(sfem_ctx *ctx, const char *basename, const double *NodeList, int ndim,
                                  int64_t nNodes, const int64_t *IEN, int64_t nEl, int nen, const double *fields,
                                  int ncomp, int64_t nsteps, int mem_space);

/* ---- load increments ------------------------------------------------------ */

/* The driver's load-increment loop (examples/vector3D.jl:310-338): one K,
 * one set of prescribed DOFs, nsteps sets of prescribed values -- step s
 * reads fixed_vals[s*nfix .. s*nfix+nfix) and writes u_out[s*n .. s*n+n),
 * n = the matrix size; stats (optional) has nsteps entries.  No single
 * reference counterpart (the reference re-inverts K_free at every step).
 * warm_start != 0 starts step s from the affine combination of up to three
 * earlier solutions whose prescribed values best match step s's: the
 * solution is affine in the prescribed values, so on the reference's
 * linear load path (q_d = -d on the top face) every step after the second
 * starts at the answer and needs no CG iteration. */
SFEM_API int sfem_solve_increments(sfem_ctx *ctx, sfem_matrix *K, const int64_t *fixed_dofs, int64_t nfix,
                                   const double *fixed_vals, int64_t nsteps, const double *f, double *u_out,
                                   int mem_space, const sfem_solve_opts *opts, int warm_start,
                                   sfem_solve_stats *stats);

/* ---- surface penalty ------------------------------------------------------ */

/* K <- K + beta * b in place, where b is the surface penalty ("slip") matrix
 * of apply_boundary_conditions (examples/vector3D.jl:175-264) and the sum is
 * the driver's K_bar = K + beta*b (examples/vector3D.jl:306-308).  3D Q1
 * elasticity only (the reference's 2D branch cannot run).  NodeList: the
 * 3 x nNodes coordinates the faces are integrated on (the reference passes
 * the inflated cylinder, not K's cube); IEN_faces: nFaces x 4, column-major,
 * 1-based -- the reference's order is [IEN_btm; IEN_top].  Every face node
 * pair must already be coupled in K (true for faces of K's elements).  The
 * FP32 copies used by the mixed solver are refreshed. */
SFEM_API int sfem_penalty_add(sfem_ctx *ctx, sfem_matrix *K, const double *NodeList, const int64_t *IEN_faces,
                              int64_t nFaces, int nenFace, double beta, int mem_space);

/* ---- serving: a device-resident request loop ------------------------------ */

/* A server runs one persistent kernel that takes assemble-and-solve requests
 * from a device queue while they keep arriving (continuous batching).  Each
 * request names its own element class (any that sfem_mesh_create accepts)
 * and plane law; requests of every class share the one kernel.  No reference
 * counterpart: the reference solves one mesh per call.  Requests wait on the
 * host until their device footprint fits the HBM budget; the sparsity
 * pattern is built once per topology key and kept on the GPU.  Each
 * request's result is independent of what else is in flight. */
typedef struct sfem_server sfem_server;

typedef struct {
    int cluster;               /* CTAs working together on one request: 1,2,4,8  */
    int threads;               /* threads per CTA: 256 or 512                    */
    double sm_fraction;        /* share of the GPU's CTA slots the kernel uses;
                                  the rest runs the pattern builds of new keys   */
    double hbm_budget_fraction;/* of free HBM at creation, for request buffers   */
    int64_t hbm_budget_bytes;  /* > 0: explicit budget instead of the fraction   */
    int max_inflight;          /* requests on the GPU at once (ring capacity)    */
    double idle_exit_ms;       /* the kernel leaves after this long without work;
                                  the server relaunches it on the next request   */
    sfem_solve_opts solve;     /* precision, precond, rtol, maxit, reliable_delta */
    int warm_start;            /* != 0: a request with a topology key starts from
                                  the last solution served on that key (kept on
                                  the GPU); results then depend, within the
                                  tolerance, on what was served before          */
} sfem_server_config;

typedef struct {
    int status;                /* sfem_status of the request                     */
    int iterations, refreshes;
    double relres;
    double queue_ms;           /* submit -> published to the GPU                 */
    double gpu_ms;             /* GPU time of the request                        */
    double total_ms;           /* submit -> result on the host                   */
    int64_t ndof;
    double t_claim_ms, t_end_ms; /* GPU clock (%globaltimer, ms) when a group took
                                  the request and when it finished it          */
    int smid;                  /* SM of the first CTA of that group              */
} sfem_server_result;

typedef struct {
    int64_t completed, pending, inflight, peak_inflight, kernel_launches;
    int64_t bytes_in_use, peak_bytes, budget_bytes, topologies;
    int grid, cluster, last_error;
} sfem_server_totals;

SFEM_API void sfem_server_config_default(sfem_server_config *cfg);
SFEM_API int sfem_server_create(int device, const sfem_server_config *cfg, sfem_server **out);
/* Queue one request: element class and arrays as for sfem_mesh_create and
 * sfem_solve_dirichlet (host memory, copied before the call returns; nen
 * follows from the class).  topology_key != 0 shares the pattern with earlier
 * requests of the same key, which must have the same class and sizes (IEN/ID
 * may then be NULL); 0 builds it for this request only.  Young: 1 or nEl
 * values; nu: 1 value. */
SFEM_API int sfem_server_submit(sfem_server *srv, int ndim, int function_class, int nDof, int plane,
                                int64_t topology_key, const double *NodeList, int64_t nNodes,
                                const int64_t *IEN, int64_t nEl, const int64_t *ID, const double *Young,
                                int64_t nYoung, const double *nu, int64_t nNu, const int64_t *fixed_dofs,
                                int64_t nfix, const double *fixed_vals, int64_t *request_id);
SFEM_API int sfem_server_wait(sfem_server *srv, int64_t request_id, double timeout_ms, double *u_out,
                              int64_t u_len, sfem_server_result *result);
SFEM_API int sfem_server_info(sfem_server *srv, sfem_server_totals *totals);
/* Requests still waiting on the host are dropped (SFEM_TIMEOUT); those on the
 * GPU finish first. */
SFEM_API int sfem_server_destroy(sfem_server *srv);

#ifdef __cplusplus
}
#endif
#endif /* SMEARFEM_GPU_H */
