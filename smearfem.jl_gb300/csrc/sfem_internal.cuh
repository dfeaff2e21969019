// Internal declarations shared by the CUDA translation units of
// libsmearfem_gpu.so.  Nothing here is part of the C ABI.
//
// Device data layout (all in HBM, one mesh):
//   X        double [nN][ndim]                node coordinates (Julia's NodeList order)
//   ien      int32  [nen][nEl]                0-based node ids, element index fastest
//   id       int32  [b][nN]                   0-based global DOF of (node, component)
//   n2e      node -> incident elements, CSR (n2e_ptr int64 [nN+1], n2e int32),
//            each list sorted ascending (the reference's duplicate-sum order)
//   pattern  node-block rows in sliced-ELL form (SELL-32): 32 consecutive
//            nodes form a slice; slice s owns slabs sliceptr[s] ..
//            sliceptr[s+1]-1; slab k of a slice holds the k-th (ascending)
//            neighbour of each of its 32 rows:
//              col [slab*32 + lane]                      int32 neighbour node
//              val [(slab*b*b + i*b + j)*32 + lane]      b x b block, row-major
//            Rows shorter than their slice are padded with (own node, 0).
//   rowptr   int64 [nN+1]  CSR offsets of the node-block rows (export order)
//   g2i      int32 [n]     global DOF (0-based) -> internal index node*b + comp
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <nvtx3/nvToolsExt.h>

#include <string>

#include "smearfem_gpu.h"

#define SFEM_VERSION "smearfem-gb300 0.1.0 (sm_103a)"

struct DevErr {
    int code;          // first error wins (atomicCAS from 0)
    int aux;
    long long index;   // offending element / node / DOF
    unsigned long long neg_det;   // Gauss points with det J < 0 (diagnostic)
};

struct sfem_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    DevErr *d_err = nullptr;
    DevErr *h_err = nullptr;    // pinned
    void *h_small = nullptr;    // pinned scratch for small read-backs (4 KB)
    std::string last_error;
    long long launches = 0;     // kernels launched through the library
    int num_sms = 1;            // streaming multiprocessors of the device
};

struct sfem_mesh {
    sfem_ctx *ctx = nullptr;
    int refcnt = 1;
    int ndim = 0, nen = 0, fclass = 0, b = 1;
    int64_t ne = 0, nEl = 0, nN = 0;
    double *X = nullptr;
    int *ien = nullptr;
    int *id = nullptr;
    // pattern
    bool has_pattern = false;
    int64_t n_global = 0, nnzb = 0, nslices = 0, nslabs = 0;
    int64_t *n2e_ptr = nullptr;
    int *n2e = nullptr;
    int *rowlen = nullptr;
    int64_t *rowptr = nullptr;
    int64_t *sliceptr = nullptr;
    int *col = nullptr;
    int *g2i = nullptr;
    unsigned long long neg_det = 0;
    int mg_ne = -1;  // elements per direction of a structured (meshgrid) mesh, 0 if not, -1 unknown
};

struct sfem_matrix {
    sfem_mesh *mesh = nullptr;
    int plane = 0;
    double *val = nullptr;     // FP64 blocks, SELL layout
    float *val32 = nullptr;    // FP32 copy (mixed precision), built on demand
    int64_t n = 0, nnz = 0;
    // upper-triangle FP32 copy for the mixed solver (sfem_sym.cu), built on demand
    int sym_state = 0;         // 0 not built, 1 ready, -1 not usable (full FP32 copy instead)
    int64_t nslabsU = 0, nslabsL = 0;
    int64_t *sptrU = nullptr, *sptrL = nullptr;
    int *colU = nullptr;
    int2 *lo = nullptr;
    float *valU = nullptr;
};

// ---- host-side error helpers (sfem_ctx.cu) -------------------------------
int sfem_set_error(sfem_ctx *ctx, int code, const char *fmt, ...);
int sfem_cuda_status(sfem_ctx *ctx, cudaError_t e, const char *what);
// Synchronise the stream, read the device error word, reset it.
int sfem_check_device(sfem_ctx *ctx, const char *where);
int sfem_dalloc(sfem_ctx *ctx, void **p, size_t bytes, const char *what);
void sfem_dfree(sfem_ctx *ctx, void *p);
// SFEM_BAD_ARG unless p is NULL or lives in the declared memory space.
int sfem_check_ptr(sfem_ctx *ctx, const void *p, int mem_space);
int sfem_copy_in(sfem_ctx *ctx, void *dst, const void *src, size_t bytes, int mem_space);
int sfem_copy_out(sfem_ctx *ctx, void *dst, const void *src, size_t bytes, int mem_space);
// Exclusive scan of n int32 (or int64) values into out[0..n], out[n] = total.
int sfem_scan_i32(sfem_ctx *ctx, const int *in, int64_t *out, int64_t n);
int sfem_scan_i64(sfem_ctx *ctx, const int64_t *in, int64_t *out, int64_t n);
void sfem_mesh_release(sfem_mesh *m);
// sfem_mesh_create with an explicit element count (batches concatenate meshes).
int sfem_mesh_create_nel(sfem_ctx *ctx, int ndim, int function_class, int nDof, int64_t nEl,
                         const double *NodeList, int64_t nNodes, const int64_t *IEN, int64_t ldIEN, int nen,
                         const int64_t *ID, int mem_space, sfem_mesh **out);

#define SFEM_TRY(...)                     \
    do {                                  \
        int _st = (__VA_ARGS__);          \
        if (_st != SFEM_OK) return _st;   \
    } while (0)

#define SFEM_CUDA(ctx, expr) SFEM_TRY(sfem_cuda_status((ctx), (expr), #expr))

#define SFEM_LAUNCHED(ctx) ((ctx)->launches++)

// Scoped NVTX range around a library phase (pattern, assembly, Dirichlet
// set-up, hierarchy, PCG, batch and serving work): visible to Nsight tools,
// free when none is attached.
struct SfemRange {
    explicit SfemRange(const char *name) { nvtxRangePushA(name); }
    ~SfemRange() { nvtxRangePop(); }
    SfemRange(const SfemRange &) = delete;
    SfemRange &operator=(const SfemRange &) = delete;
};

// ---- device helpers -------------------------------------------------------
__device__ __forceinline__ void sfem_dev_error(DevErr *e, int code, long long index) {
    if (atomicCAS(&e->code, 0, code) == 0) e->index = index;
}

__host__ __device__ __forceinline__ int64_t sfem_cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// number of node pairs a <= b in an element with nen nodes, and their index
__host__ __device__ __forceinline__ int sfem_npairs(int nen) { return nen * (nen + 1) / 2; }
__host__ __device__ __forceinline__ int sfem_pair(int a, int b, int nen) {
    return a * nen - a * (a - 1) / 2 + (b - a);
}

// Element stiffness buffer produced by the element kernel and consumed by the
// slot gather: for pair p = (a <= b), block entry (i, j) of element e lives at
//   kbuf[((size_t)p * B * B + i * B + j) * nEl + e]
int sfem_element_stiffness(sfem_ctx *ctx, const sfem_mesh *m, int plane, const double *dYoung,
                           int64_t nYoung, const double *dnu, int64_t nNu, double *kbuf);
int sfem_gather_blocks(sfem_ctx *ctx, const sfem_mesh *m, const double *kbuf, double *val,
                       float *val32);
// Upper-triangle FP32 copy of K (sfem_sym.cu).
int sfem_sym_build(sfem_ctx *ctx, sfem_matrix *K);
int sfem_sym_refresh_values(sfem_ctx *ctx, sfem_matrix *K);
void sfem_sym_free(sfem_ctx *ctx, sfem_matrix *K);

// Lane-contiguous FP32 block layout (the per-mesh pipeline's K copy and the
// upper-triangle storage of the mixed solver).  Each lane's block entries of
// a slab are contiguous -- chunks of four, then the rest -- so a lane reads
// its block with one (B = 2) or three (B = 3) vector loads while the warp
// still reads whole contiguous segments: B = 1 one float per lane; B = 2 a
// float4; B = 3 a float4, a float4 and a float (1152 bytes per slab, no
// padding).  Fewer load instructions per product than the entry-major
// layout.  STREAM: read with the evict-first hint (values used once).
template <int B>
__device__ __forceinline__ int64_t v32_at(int64_t slab, int lane, int e) {
    if constexpr (B == 1) {
        return slab * 32 + lane;
    } else if constexpr (B == 2) {
        return (slab * 32 + lane) * 4 + e;
    } else {
        const int64_t base = slab * 288;
        return e < 4 ? base + lane * 4 + e : (e < 8 ? base + 128 + lane * 4 + (e - 4) : base + 256 + lane);
    }
}

template <typename V>
__device__ __forceinline__ V sfem_ld(const V *p, bool stream) {
    return stream ? __ldcs(p) : __ldg(p);
}

template <int B, bool STREAM>
__device__ __forceinline__ void load_v32(const float *__restrict__ v, int64_t slab, int lane, float *out) {
    if constexpr (B == 1) {
        out[0] = sfem_ld(v + slab * 32 + lane, STREAM);
    } else if constexpr (B == 2) {
        const float4 t = sfem_ld(reinterpret_cast<const float4 *>(v + (slab * 32 + lane) * 4), STREAM);
        out[0] = t.x;
        out[1] = t.y;
        out[2] = t.z;
        out[3] = t.w;
    } else {
        const float *b = v + slab * 288;
        const float4 t0 = sfem_ld(reinterpret_cast<const float4 *>(b + lane * 4), STREAM);
        const float4 t1 = sfem_ld(reinterpret_cast<const float4 *>(b + 128 + lane * 4), STREAM);
        out[0] = t0.x;
        out[1] = t0.y;
        out[2] = t0.z;
        out[3] = t0.w;
        out[4] = t1.x;
        out[5] = t1.y;
        out[6] = t1.z;
        out[7] = t1.w;
        out[8] = sfem_ld(b + 256 + lane, STREAM);
    }
}

// One row's share of the assembly gather (k_gather, and the multigrid
// instantiations of the per-mesh pipeline).  The row's elements, their
// nodes and the row node's local position are read once, so each of the
// row's slots costs one compare per element node instead of re-reading and
// re-matching every element.  `fast` is false when the row lies in more than
// MAXE elements or one of them repeats a node; callers then take their
// general loop.  Blocks are added in ascending element order, the same order
// (and so the same sums) as that general loop.
template <int NEN>
struct GatherRow {
    static constexpr int MAXE = NEN == 9 ? 4 : NEN;  // elements around a node of a conforming Q1 / Q2 grid
    int n;
    bool fast;
    int e[MAXE], a[MAXE], nodes[MAXE][NEN];

    __device__ __forceinline__ void load(const int *__restrict__ n2e, int64_t q0, int64_t q1,
                                         const int *__restrict__ ien, int64_t nEl, int r) {
        n = (int)(q1 - q0);
        fast = n <= MAXE;
#pragma unroll
        for (int m = 0; m < MAXE; ++m) {
            const bool use = fast && m < n;
            e[m] = use ? n2e[q0 + m] : 0;
            a[m] = -1;
#pragma unroll
            for (int b = 0; b < NEN; ++b) {
                nodes[m][b] = use ? __ldg(&ien[(int64_t)b * nEl + e[m]]) : -1;
                if (nodes[m][b] == r) a[m] = b;
            }
            bool distinct = true;
#pragma unroll
            for (int b = 0; b < NEN; ++b)
#pragma unroll
                for (int c = b + 1; c < NEN; ++c) distinct = distinct && nodes[m][b] != nodes[m][c];
            if (use && (a[m] < 0 || !distinct)) fast = false;
        }
    }

    // acc += the element blocks of slot (row, c); kbuf: [pair][B][B][nEl]
    template <int B>
    __device__ __forceinline__ void add(int c, const double *__restrict__ kbuf, int64_t nEl, double *acc) const {
#pragma unroll
        for (int m = 0; m < MAXE; ++m) {
            int hit = -1;
#pragma unroll
            for (int bq = 0; bq < NEN; ++bq) hit = nodes[m][bq] == c ? bq : hit;
            if (m < n && hit >= 0) {
                const int am = a[m];
                const bool up = am <= hit;
                const int64_t base = (int64_t)sfem_pair(up ? am : hit, up ? hit : am, NEN) * B * B;
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j)
                        acc[i * B + j] += __ldg(&kbuf[(base + (up ? i * B + j : j * B + i)) * nEl + e[m]]);
            }
        }
    }
};
