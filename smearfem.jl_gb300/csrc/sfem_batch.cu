// Batches of independent meshes, assembled and solved by ONE persistent kernel.
//
// Layout.  The meshes of a batch become one block-diagonal "combined" mesh:
// mesh b's nodes are renumbered into [pad_base[b], pad_base[b] + nN_b) with
// every range padded to a multiple of 32, so each 32-row slice of the
// sliced-ELL pattern belongs to exactly one mesh.  The pattern of the
// combined mesh is built once (sfem_batch_create) with the single-mesh
// kernels; its rows never couple two meshes.
//
// Solve.  k_batch runs with a grid sized to fill the GPU once.  Each CTA
// takes meshes from an atomic work queue, largest first, and for each one:
//   1. element stiffness of the mesh's elements (FP64, as k_element),
//   2. deterministic gather into the mesh's K blocks (as k_gather), FP64 and
//      an FP32 copy for the mixed solver,
//   3. Dirichlet set-up: mask, lift q_d, right-hand side -K q_d,
//   4. nodal block-Jacobi inverse,
//   5. preconditioned CG: FP64, or FP32 recurrences refreshed from an FP64
//      residual whenever the FP32 residual drops by `reliable_delta`,
//   6. u = q_d + x in the mesh's own DOF numbering.
// All reductions are CTA-wide in a fixed order and no CTA ever waits on
// another, so a mesh's result does not depend on which CTA solves it or on
// what else is in the batch: it is bitwise the same alone and in any mix.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "sfem_meshsolve.cuh"

struct sfem_batch {
    sfem_ctx *ctx = nullptr;
    sfem_mesh *mesh = nullptr;  // combined mesh (owns the pattern)
    int ndim = 0, nen = 0, b = 1, fclass = 1;
    int64_t nmesh = 0, total_nodes = 0, total_elems = 0, total_dofs = 0;
    std::vector<int64_t> h_node_off, h_elem_off, h_pad_base;
    BatchMesh *meshes = nullptr;  // device
    int *order = nullptr;         // device: meshes by decreasing size
    unsigned *queue = nullptr;    // device work counter
    // solve buffers (allocated at the first solve, reused)
    bool buffers = false;
    double *kbuf = nullptr, *val64 = nullptr, *ud = nullptr, *b64 = nullptr, *x64 = nullptr, *q64 = nullptr;
    float *val32 = nullptr;
    void *vecT = nullptr;         // 6 work vectors of the CG type + preconditioner
    unsigned char *fixed = nullptr, *gfixed = nullptr;
    double *E = nullptr, *nu = nullptr, *fvals = nullptr, *u = nullptr;
    int64_t *fdofs = nullptr, *fix_off_dev = nullptr;
    int64_t cap_E = 0, cap_nu = 0, cap_fixd = 0, cap_fixv = 0;
    int threads = 512, ctas_per_sm = 1;  // launch shape (autotuned)
    int cluster = 4;                     // CTAs per cluster working on one large mesh
    int64_t big_nodes = 16384;           // meshes with at least this many nodes use a cluster
    int last_grid = 0, last_cluster = 0;
    std::vector<int64_t> h_nodes;        // nodes per mesh
    // multigrid (built at the first multigrid solve): structured meshes get a hierarchy
    bool mg_checked = false, mg_any = false;
    std::vector<int> h_mg_ne;            // elements per direction of each structured mesh, else 0
    char *mg_buf = nullptr;              // every hierarchy's arrays
    MgMesh *mg_rec = nullptr;            // device: one record per mesh (nlev 0: no hierarchy)
    // per-solve state: the host copy of the per-mesh table (its fixed-DOF
    // ranges change per solve), pinned staging for it and for the statistics,
    // and the CUDA graph of the last solve with the key it was captured for
    std::vector<BatchMesh> h_meshes;
    BatchMesh *h_tab = nullptr;
    sfem_batch_stats *d_stats = nullptr, *h_stats = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> gkey;
};

namespace {

using namespace sfem_dev;

// 2D classes fit two 512-thread CTAs per SM (64 registers; the multigrid
// variants spill some around the hierarchy's calls, and still run faster
// than at one CTA per SM); 3D elasticity needs the full register file of one.
template <int NDIM, int NEN, int NGP, int B, bool MIXED, bool MG>
__global__ void __launch_bounds__(512, (NDIM == 2 ? 2 : 1)) k_batch(const __grid_constant__ ElemTableB tab, const __grid_constant__ BatchArgs a) {
    __shared__ double red[128];  // two halves, alternating (block_sum2)
    __shared__ double xch[4];
    __shared__ int s_flag, s_mesh;
    constexpr int WF = (NDIM == 2 && NEN == 4 && B == 2) ? 9 : 0;  // pipelined 9-slab slices of 2D Q1 elasticity
    constexpr int UF = (NDIM == 3 && B == 3) ? 9 : 4;                 // 3D elasticity: 9 slabs in flight
    const int tid = threadIdx.x;
    cgrp::cluster_group cl = cgrp::this_cluster();
    // 1. large meshes: the whole cluster works on one mesh
    for (;;) {
        if (cl.block_rank() == 0 && tid == 0) s_mesh = (int)atomicAdd(a.queue, 1u);
        cl.sync();
        const int64_t q = *cl.map_shared_rank(&s_mesh, 0);
        cl.sync();
        if (q >= a.nbig) break;
        process_mesh<ClusterGroup, NDIM, NEN, NGP, B, MIXED, UF, WF, 1, false, MG>(ClusterGroup(), tab, a,
                                                                                       a.order[q], red, xch, &s_flag);
        cl.sync();
    }
    // 2. small meshes: every CTA on its own
    for (;;) {
        if (tid == 0) s_mesh = (int)atomicAdd(a.queue + 1, 1u);
        __syncthreads();
        const int64_t q = (int64_t)a.nbig + s_mesh;
        __syncthreads();
        if (q >= a.nmesh) break;
        process_mesh<SoloGroup, NDIM, NEN, NGP, B, MIXED, UF, WF, 1, false, MG>(SoloGroup(), tab, a,
                                                                                    a.order[q], red, xch, &s_flag);
        __syncthreads();
    }
    cl.sync();  // peers may still read this CTA's shared memory until every CTA is done
}

__global__ void k_batch_nodes(const double *__restrict__ Xin, const int64_t *__restrict__ IDin, int64_t total_nodes,
                              const int64_t *__restrict__ node_off, const int64_t *__restrict__ pad_base,
                              int64_t nmesh, int ndim, int b, double *__restrict__ Xc, int64_t *__restrict__ IDc,
                              int64_t total_pad, DevErr *err) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_pad) return;
    int64_t lo = 0, hi = nmesh - 1;  // mesh with pad_base[m] <= t < pad_base[m+1]
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (pad_base[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const int64_t m = lo, local = t - pad_base[m], nn = node_off[m + 1] - node_off[m];
    if (local < nn) {
        const int64_t src = node_off[m] + local;
        for (int i = 0; i < ndim; ++i) Xc[t * ndim + i] = Xin[src * ndim + i];
        for (int d = 0; d < b; ++d) {
            int64_t v = IDin ? IDin[(int64_t)d * total_nodes + src] : (int64_t)b * local + d + 1;
            if (v < 1 || v > (int64_t)b * nn) {
                sfem_dev_error(err, SFEM_BAD_INDEX, src);
                v = 1;
            }
            IDc[(int64_t)d * total_pad + t] = (int64_t)b * node_off[m] + v;
        }
    } else {
        for (int i = 0; i < ndim; ++i) Xc[t * ndim + i] = 0.0;
        for (int d = 0; d < b; ++d) IDc[(int64_t)d * total_pad + t] = 0;  // never referenced
    }
}

__global__ void k_batch_elems(const int64_t *__restrict__ IENin, int64_t total_el, int nen,
                              const int64_t *__restrict__ elem_off, const int64_t *__restrict__ node_off,
                              const int64_t *__restrict__ pad_base, int64_t nmesh, int64_t *__restrict__ IENc,
                              DevErr *err) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_el * nen) return;
    const int64_t e = t % total_el;
    int64_t lo = 0, hi = nmesh - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (elem_off[mid] <= e) lo = mid;
        else hi = mid - 1;
    }
    const int64_t nn = node_off[lo + 1] - node_off[lo];
    int64_t v = IENin[t];
    if (v < 1 || v > nn) {
        sfem_dev_error(err, SFEM_BAD_INDEX, e);
        v = 1;
    }
    IENc[t] = pad_base[lo] + v;  // 1-based combined node id
}

// Structured-grid check of every mesh of a batch: ok[m] is cleared when an
// element of mesh m differs from the meshgrid connectivity of cand[m]
// elements per direction (combined 0-based node ids, element index fastest).
__global__ void k_mg_check(const int *__restrict__ ien, int64_t nEl, int nen, int ndim,
                           const BatchMesh *__restrict__ meshes, int64_t nmesh, const int *__restrict__ cand,
                           int *__restrict__ ok) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nEl) return;
    int64_t lo = 0, hi = nmesh - 1;  // last mesh with elem0 <= e
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (meshes[mid].elem0 <= e) lo = mid;
        else hi = mid - 1;
    }
    const BatchMesh M = meshes[lo];
    const int ne = cand[lo];
    if (ne == 0 || e >= M.elem1) return;
    for (int c = 0; c < nen; ++c)
        if ((int64_t)ien[(int64_t)c * nEl + e] != M.node0 + mg_grid_node(ndim, ne, e - M.elem0, c) - 1) ok[lo] = 0;
}

template <int NDIM, int NEN, int NGP, int B, bool MIXED, bool MG = false>
int launch_batch(sfem_ctx *ctx, sfem_batch *bt, const BatchArgs &args) {
    constexpr int GS = NEN * NDIM + 1;
    const int threads = bt->threads;
    const int ngroups = (threads / 32) / NGP;
    const size_t smem = sizeof(double) * (size_t)ngroups * (NGP * 32 * GS + NGP * 32);
    auto kern = k_batch<NDIM, NEN, NGP, B, MIXED, MG>;
    SFEM_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const ElemTableB tab = make_table_b(NDIM, bt->fclass);
    SFEM_CUDA(ctx, cudaMemsetAsync(bt->queue, 0, 2 * sizeof(unsigned), ctx->stream));
    int csize = bt->cluster;
    int nclusters = 0;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr[1];
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    if (csize > 1) {
        if (csize > 8) SFEM_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = csize;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cfg.gridDim = dim3(csize * ctx->num_sms, 1, 1);
        if (cudaOccupancyMaxActiveClusters(&nclusters, (void *)kern, &cfg) != cudaSuccess || nclusters < 1) {
            cudaGetLastError();
            csize = 1;  // clusters of this shape do not fit: every CTA works alone
        }
    }
    if (csize <= 1) {
        int per_sm = 0;
        SFEM_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
        if (per_sm < 1) return sfem_set_error(ctx, SFEM_UNSUPPORTED, "batch kernel does not fit with %d threads", threads);
        nclusters = std::min(per_sm, bt->ctas_per_sm) * ctx->num_sms;
        cfg.attrs = nullptr;
        cfg.numAttrs = 0;
        csize = 1;
    }
    const int64_t want = std::max<int64_t>(1, std::min<int64_t>((int64_t)nclusters * csize, bt->nmesh * csize));
    cfg.gridDim = dim3((unsigned)(want / csize * csize), 1, 1);
    bt->last_grid = (int)cfg.gridDim.x;
    bt->last_cluster = csize;
    SFEM_CUDA(ctx, cudaLaunchKernelEx(&cfg, kern, tab, args));
    SFEM_LAUNCHED(ctx);
    return sfem_cuda_status(ctx, cudaGetLastError(), "batch kernel launch");
}

template <bool MIXED>
int dispatch_batch(sfem_ctx *ctx, sfem_batch *bt, const BatchArgs &args) {
    if constexpr (MIXED) {
        if (args.mg && bt->fclass == SFEM_Q1) {  // the multigrid variants (Q1 classes, mixed precision)
            if (bt->ndim == 2)
                return bt->b == 1 ? launch_batch<2, 4, 4, 1, true, true>(ctx, bt, args)
                                  : launch_batch<2, 4, 4, 2, true, true>(ctx, bt, args);
            return bt->b == 1 ? launch_batch<3, 8, 8, 1, true, true>(ctx, bt, args)
                              : launch_batch<3, 8, 8, 3, true, true>(ctx, bt, args);
        }
    }
    if (bt->fclass == SFEM_Q2) return launch_batch<2, 9, 4, 1, MIXED>(ctx, bt, args);
    if (bt->ndim == 2)
        return bt->b == 1 ? launch_batch<2, 4, 4, 1, MIXED>(ctx, bt, args) : launch_batch<2, 4, 4, 2, MIXED>(ctx, bt, args);
    return bt->b == 1 ? launch_batch<3, 8, 8, 1, MIXED>(ctx, bt, args) : launch_batch<3, 8, 8, 3, MIXED>(ctx, bt, args);
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" int sfem_batch_create(sfem_ctx *ctx, int ndim, int function_class, int nDof, int64_t nmesh,
                                 const int64_t *node_offsets, const int64_t *elem_offsets, const double *NodeList,
                                 const int64_t *IEN, const int64_t *ID, int mem_space, sfem_batch **out) {
    if (!ctx || !out || !node_offsets || !elem_offsets || nmesh < 1) return SFEM_BAD_ARG;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    if (ndim != 2 && ndim != 3) return sfem_set_error(ctx, ndim == 1 ? SFEM_UNSUPPORTED : SFEM_BAD_ARG, "ndim must be 2 or 3");
    if (nDof != 1 && nDof != ndim) return sfem_set_error(ctx, SFEM_UNSUPPORTED, "nDof must be 1 or ndim");
    if (function_class == SFEM_Q2 && (ndim != 2 || nDof != 1))
        return sfem_set_error(ctx, SFEM_UNSUPPORTED, "Q2 batches are 2D scalar only");
    const int nen = function_class == SFEM_Q2 ? 9 : (1 << ndim);
    sfem_batch *bt = new sfem_batch();
    bt->ctx = ctx;
    bt->ndim = ndim;
    bt->nen = nen;
    bt->b = nDof;
    bt->fclass = function_class;
    bt->nmesh = nmesh;
    bt->h_node_off.resize(nmesh + 1);
    bt->h_elem_off.resize(nmesh + 1);
    bt->h_pad_base.resize(nmesh + 1);
    int st = SFEM_OK;
    int64_t *d_no = nullptr, *d_eo = nullptr, *d_pb = nullptr, *IDin = nullptr, *IENin = nullptr, *IDc = nullptr,
            *IENc = nullptr;
    double *Xin = nullptr, *Xc = nullptr;
    do {
        if ((st = sfem_check_ptr(ctx, node_offsets, mem_space)) || (st = sfem_check_ptr(ctx, elem_offsets, mem_space)))
            break;
        SFEM_CUDA(ctx, cudaMemcpy(bt->h_node_off.data(), node_offsets, sizeof(int64_t) * (nmesh + 1), cudaMemcpyDefault));
        SFEM_CUDA(ctx, cudaMemcpy(bt->h_elem_off.data(), elem_offsets, sizeof(int64_t) * (nmesh + 1), cudaMemcpyDefault));
        const auto &no = bt->h_node_off, &eo = bt->h_elem_off;
        if (no[0] != 0 || eo[0] != 0) {
            st = sfem_set_error(ctx, SFEM_BAD_ARG, "offsets must start at 0");
            break;
        }
        bt->h_pad_base[0] = 0;
        for (int64_t m = 0; m < nmesh; ++m) {
            if (no[m + 1] <= no[m] || eo[m + 1] < eo[m]) {
                st = sfem_set_error(ctx, SFEM_BAD_ARG, "mesh %lld has no nodes or negative elements", (long long)m);
                break;
            }
            bt->h_pad_base[m + 1] = bt->h_pad_base[m] + sfem_cdiv(no[m + 1] - no[m], 32) * 32;
        }
        if (st) break;
        bt->total_nodes = no[nmesh];
        bt->total_elems = eo[nmesh];
        bt->total_dofs = nDof * bt->total_nodes;
        const int64_t total_pad = bt->h_pad_base[nmesh];
        if (total_pad * nDof > INT_MAX / 2 || bt->total_elems * nen > INT_MAX) {
            st = sfem_set_error(ctx, SFEM_BAD_ARG, "batch too large");
            break;
        }
        const int64_t tn = bt->total_nodes, te = bt->total_elems;
        if ((st = sfem_dalloc(ctx, (void **)&d_no, sizeof(int64_t) * (nmesh + 1), "offsets"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&d_eo, sizeof(int64_t) * (nmesh + 1), "offsets"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&d_pb, sizeof(int64_t) * (nmesh + 1), "offsets"))) break;
        if ((st = sfem_copy_in(ctx, d_no, no.data(), sizeof(int64_t) * (nmesh + 1), SFEM_MEM_HOST))) break;
        if ((st = sfem_copy_in(ctx, d_eo, eo.data(), sizeof(int64_t) * (nmesh + 1), SFEM_MEM_HOST))) break;
        if ((st = sfem_copy_in(ctx, d_pb, bt->h_pad_base.data(), sizeof(int64_t) * (nmesh + 1), SFEM_MEM_HOST))) break;
        if ((st = sfem_dalloc(ctx, (void **)&Xin, sizeof(double) * ndim * tn, "NodeList"))) break;
        if ((st = sfem_copy_in(ctx, Xin, NodeList, sizeof(double) * ndim * tn, mem_space))) break;
        if (ID) {
            if ((st = sfem_dalloc(ctx, (void **)&IDin, sizeof(int64_t) * nDof * tn, "ID"))) break;
            if ((st = sfem_copy_in(ctx, IDin, ID, sizeof(int64_t) * nDof * tn, mem_space))) break;
        }
        if ((st = sfem_dalloc(ctx, (void **)&IENin, sizeof(int64_t) * (te * nen + 1), "IEN"))) break;
        if ((st = sfem_copy_in(ctx, IENin, IEN, sizeof(int64_t) * te * nen, mem_space))) break;
        if ((st = sfem_dalloc(ctx, (void **)&Xc, sizeof(double) * ndim * total_pad, "combined nodes"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&IDc, sizeof(int64_t) * nDof * total_pad, "combined ID"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&IENc, sizeof(int64_t) * (te * nen + 1), "combined IEN"))) break;
        k_batch_nodes<<<(unsigned)sfem_cdiv(total_pad, 256), 256, 0, ctx->stream>>>(
            Xin, IDin, tn, d_no, d_pb, nmesh, ndim, nDof, Xc, IDc, total_pad, ctx->d_err);
        SFEM_LAUNCHED(ctx);
        if (te > 0) {
            k_batch_elems<<<(unsigned)sfem_cdiv(te * nen, 256), 256, 0, ctx->stream>>>(IENin, te, nen, d_eo, d_no, d_pb,
                                                                                     nmesh, IENc, ctx->d_err);
            SFEM_LAUNCHED(ctx);
        }
        if ((st = sfem_check_device(ctx, "batch inputs"))) break;
        if ((st = sfem_mesh_create_nel(ctx, ndim, function_class, nDof, te, Xc, total_pad, IENc, te, nen, IDc,
                                       SFEM_MEM_DEVICE, &bt->mesh)))
            break;
        if ((st = sfem_pattern_build(ctx, bt->mesh, nullptr, nullptr))) break;
        // per-mesh descriptors and the largest-first order
        std::vector<BatchMesh> hm(nmesh);
        std::vector<int> order(nmesh);
        for (int64_t m = 0; m < nmesh; ++m) {
            BatchMesh &M = hm[m];
            M.node0 = bt->h_pad_base[m];
            M.nnode = no[m + 1] - no[m];
            M.slice0 = bt->h_pad_base[m] / 32;
            M.slice1 = bt->h_pad_base[m + 1] / 32;
            M.elem0 = eo[m];
            M.elem1 = eo[m + 1];
            M.dof0 = nDof * no[m];
            M.ndof = nDof * M.nnode;
            M.fix0 = M.fix1 = 0;
            order[m] = (int)m;
        }
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return hm[x].nnode > hm[y].nnode; });
        bt->h_nodes.resize(nmesh);
        for (int64_t mm = 0; mm < nmesh; ++mm) bt->h_nodes[mm] = hm[order[mm]].nnode;  // in queue order
        if ((st = sfem_dalloc(ctx, (void **)&bt->meshes, sizeof(BatchMesh) * nmesh, "batch meshes"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&bt->order, sizeof(int) * nmesh, "batch order"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&bt->queue, 2 * sizeof(unsigned), "batch queue"))) break;
        if ((st = sfem_copy_in(ctx, bt->meshes, hm.data(), sizeof(BatchMesh) * nmesh, SFEM_MEM_HOST))) break;
        bt->h_meshes = hm;
        if ((st = sfem_cuda_status(ctx, cudaMallocHost((void **)&bt->h_tab, sizeof(BatchMesh) * nmesh),
                                   "pinned batch table")))
            break;
        if ((st = sfem_cuda_status(ctx, cudaMallocHost((void **)&bt->h_stats, sizeof(sfem_batch_stats) * nmesh),
                                   "pinned batch statistics")))
            break;
        if ((st = sfem_dalloc(ctx, (void **)&bt->d_stats, sizeof(sfem_batch_stats) * nmesh, "batch stats"))) break;
        if ((st = sfem_copy_in(ctx, bt->order, order.data(), sizeof(int) * nmesh, SFEM_MEM_HOST))) break;
        st = sfem_check_device(ctx, "batch create");
    } while (0);
    void *tmp[] = {d_no, d_eo, d_pb, IDin, IENin, IDc, IENc, Xin, Xc};
    for (void *p : tmp) sfem_dfree(ctx, p);
    cudaStreamSynchronize(ctx->stream);
    if (st != SFEM_OK) {
        sfem_batch_destroy(bt);
        return st;
    }
    *out = bt;
    return SFEM_OK;
}

extern "C" int sfem_batch_info(const sfem_batch *bt, int64_t *total_dofs, int64_t *total_nodes,
                               int64_t *total_elements) {
    if (!bt) return SFEM_BAD_ARG;
    if (total_dofs) *total_dofs = bt->total_dofs;
    if (total_nodes) *total_nodes = bt->total_nodes;
    if (total_elements) *total_elements = bt->total_elems;
    return SFEM_OK;
}

extern "C" int sfem_batch_set_launch(sfem_batch *bt, int threads, int ctas_per_sm, int cluster,
                                     int64_t cluster_min_nodes) {
    if (!bt || (threads != 256 && threads != 512) || ctas_per_sm < 1 || ctas_per_sm > 8)
        return SFEM_BAD_ARG;
    if (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16) return SFEM_BAD_ARG;
    if (cluster_min_nodes < 1) return SFEM_BAD_ARG;
    const int ngp = bt->ndim == 2 ? 4 : 8;
    if ((threads / 32) < ngp) return SFEM_BAD_ARG;
    bt->threads = threads;
    bt->ctas_per_sm = ctas_per_sm;
    bt->cluster = cluster;
    bt->big_nodes = cluster_min_nodes;
    return SFEM_OK;
}

static int batch_buffers(sfem_ctx *ctx, sfem_batch *bt) {
    if (bt->buffers) return SFEM_OK;
    sfem_mesh *m = bt->mesh;
    const int b = bt->b;
    const int64_t nd = m->nN * b, nv = m->nslabs * 32 * b * b;
    const int64_t nk = (int64_t)sfem_npairs(m->nen) * b * b * m->nEl;
    const size_t tsz = sizeof(double);  // vecT sized for the FP64 variant (FP32 fits too)
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->kbuf, sizeof(double) * (nk + 1), "batch element stiffness"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->val64, sizeof(double) * (nv + 1), "batch K"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->val32, sizeof(float) * (nv + 1), "batch K fp32"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->ud, sizeof(double) * nd, "batch q_d"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->b64, sizeof(double) * nd, "batch rhs"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->x64, sizeof(double) * nd, "batch x"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->q64, sizeof(double) * nd, "batch q64"));
    SFEM_TRY(sfem_dalloc(ctx, &bt->vecT, tsz * (6 * nd + m->nN * b * b), "batch CG vectors"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->fixed, nd, "batch mask"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->gfixed, bt->total_dofs + 1, "batch global mask"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->u, sizeof(double) * (bt->total_dofs + 1), "batch u"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->fix_off_dev, sizeof(int64_t) * (bt->nmesh + 1), "batch fix offsets"));
    bt->buffers = true;
    return SFEM_OK;
}

// Multigrid hierarchies of the batch's structured meshes (once per batch):
// the connectivity check on the device, then one buffer for every
// hierarchy.  The fine level's vectors and smoother are indexed by combined
// node like the CG's, so their pointers are shifted by the mesh's first node.
static int batch_mg(sfem_ctx *ctx, sfem_batch *bt) {
    if (bt->mg_checked) return SFEM_OK;
    const int64_t nm = bt->nmesh;
    const int b = bt->b;
    std::vector<int> cand(nm, 0), ok(nm, 1);
    bool anyc = false;
    for (int64_t m = 0; m < nm; ++m) {
        if (bt->fclass != SFEM_Q1) break;
        const int ne = mg_grid_ne(bt->ndim, bt->h_node_off[m + 1] - bt->h_node_off[m],
                                  bt->h_elem_off[m + 1] - bt->h_elem_off[m]);
        cand[m] = mg_levels(ne) >= 2 ? ne : 0;
        anyc = anyc || cand[m] > 0;
    }
    if (anyc) {
        int *dc = nullptr, *dok = nullptr;
        int st = sfem_dalloc(ctx, (void **)&dc, sizeof(int) * nm, "multigrid check");
        if (st == SFEM_OK) st = sfem_dalloc(ctx, (void **)&dok, sizeof(int) * nm, "multigrid check");
        if (st == SFEM_OK) st = sfem_copy_in(ctx, dc, cand.data(), sizeof(int) * nm, SFEM_MEM_HOST);
        if (st == SFEM_OK) st = sfem_copy_in(ctx, dok, ok.data(), sizeof(int) * nm, SFEM_MEM_HOST);
        if (st == SFEM_OK && bt->mesh->nEl > 0) {
            k_mg_check<<<(unsigned)sfem_cdiv(bt->mesh->nEl, 256), 256, 0, ctx->stream>>>(
                bt->mesh->ien, bt->mesh->nEl, bt->nen, bt->ndim, bt->meshes, nm, dc, dok);
            SFEM_LAUNCHED(ctx);
        }
        if (st == SFEM_OK) st = sfem_copy_out(ctx, ok.data(), dok, sizeof(int) * nm, SFEM_MEM_HOST);
        sfem_dfree(ctx, dc);
        sfem_dfree(ctx, dok);
        SFEM_TRY(st);
    }
    bt->h_mg_ne.assign(nm, 0);
    std::vector<int64_t> off(nm + 1, 0);
    for (int64_t m = 0; m < nm; ++m) {
        int64_t bytes = 0;
        if (cand[m] > 0 && ok[m]) {
            bt->h_mg_ne[m] = cand[m];
            bytes = (mg_layout(bt->ndim, b, cand[m], (bt->h_pad_base[m + 1] - bt->h_pad_base[m]) * b, nullptr,
                               nullptr) + 255) / 256 * 256;
            bt->mg_any = true;
        }
        off[m + 1] = off[m] + bytes;
    }
    std::vector<MgMesh> rec(nm);
    memset(rec.data(), 0, sizeof(MgMesh) * nm);
    if (bt->mg_any) {
        SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->mg_buf, (size_t)off[nm], "batch multigrid"));
        for (int64_t m = 0; m < nm; ++m) {
            if (!bt->h_mg_ne[m]) continue;
            const int64_t padded = bt->h_pad_base[m + 1] - bt->h_pad_base[m], node0 = bt->h_pad_base[m];
            mg_layout(bt->ndim, b, bt->h_mg_ne[m], padded * b, bt->mg_buf + off[m], &rec[m]);
            MgLevel &f = rec[m].lev[0];
            f.x = (float *)((uintptr_t)f.x - sizeof(float) * node0 * b);
            f.t = (float *)((uintptr_t)f.t - sizeof(float) * node0 * b);
            f.minv = (float *)((uintptr_t)f.minv - sizeof(float) * node0 * b * b);
        }
    }
    SFEM_TRY(sfem_dalloc(ctx, (void **)&bt->mg_rec, sizeof(MgMesh) * nm, "batch multigrid records"));
    SFEM_TRY(sfem_copy_in(ctx, bt->mg_rec, rec.data(), sizeof(MgMesh) * nm, SFEM_MEM_HOST));
    bt->mg_checked = true;
    return SFEM_OK;
}

static int grow(sfem_ctx *ctx, void **p, int64_t *cap, int64_t need, size_t elem, const char *what) {
    if (need <= *cap && *p) return SFEM_OK;
    sfem_dfree(ctx, *p);
    *p = nullptr;
    SFEM_TRY(sfem_dalloc(ctx, p, elem * (need > 0 ? need : 1), what));
    *cap = need;
    return SFEM_OK;
}

// A copy between a caller's pointer and the batch's buffers.  Copies from
// or to device memory or pinned host memory run inside the solve's graph;
// pageable host memory is copied outside it (a graph cannot copy from it).
struct GCopy {
    void *dst;
    const void *src;
    size_t bytes;
};

static bool graph_copyable(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeHost;
}

// Check the material and boundary data, size the batch's buffers, and set
// up the copies into them: pageable sources are copied now (ordered before
// the solve on the stream), the others are returned in `in` for the graph.
// The per-mesh table gets each mesh's fixed-DOF range from the host copy.
static int batch_upload(sfem_ctx *ctx, sfem_batch *bt, int plane, const double *Young, int64_t *nYoung,
                        const double *nu, int64_t *nNu, const int64_t *fix_offsets, const int64_t *fixed_dofs,
                        const double *fixed_vals, int mem_space, std::vector<GCopy> *in) {
    if (plane != SFEM_PLANE_STRESS && plane != SFEM_PLANE_STRAIN) return sfem_set_error(ctx, SFEM_BAD_ARG, "bad plane");
    const int64_t nm = bt->nmesh;
    if (bt->b > 1) {
        if (!Young || !nu) return sfem_set_error(ctx, SFEM_BAD_ARG, "Young and nu are required for elasticity");
        auto okn = [&](int64_t n) { return n == 1 || n == nm || n == bt->total_elems; };
        if (!okn(*nYoung) || !okn(*nNu))
            return sfem_set_error(ctx, SFEM_BAD_ARG, "Young/nu: length 1, nmesh or total elements");
    } else {
        *nYoung = *nNu = 1;
    }
    SFEM_TRY(sfem_check_ptr(ctx, fix_offsets, mem_space));
    std::vector<int64_t> fo(nm + 1);
    if (mem_space == SFEM_MEM_HOST) memcpy(fo.data(), fix_offsets, sizeof(int64_t) * (nm + 1));
    else SFEM_CUDA(ctx, cudaMemcpy(fo.data(), fix_offsets, sizeof(int64_t) * (nm + 1), cudaMemcpyDeviceToHost));
    if (fo[0] != 0) return sfem_set_error(ctx, SFEM_BAD_ARG, "fix_offsets must start at 0");
    for (int64_t m = 0; m < nm; ++m)
        if (fo[m + 1] < fo[m]) return sfem_set_error(ctx, SFEM_BAD_ARG, "fix_offsets must not decrease");
    const int64_t nfix = fo[nm];
    SFEM_TRY(batch_buffers(ctx, bt));
    SFEM_TRY(grow(ctx, (void **)&bt->E, &bt->cap_E, *nYoung, sizeof(double), "batch Young"));
    SFEM_TRY(grow(ctx, (void **)&bt->nu, &bt->cap_nu, *nNu, sizeof(double), "batch nu"));
    SFEM_TRY(grow(ctx, (void **)&bt->fdofs, &bt->cap_fixd, nfix, sizeof(int64_t), "batch fixed dofs"));
    SFEM_TRY(grow(ctx, (void **)&bt->fvals, &bt->cap_fixv, nfix, sizeof(double), "batch fixed values"));
    auto add = [&](void *dst, const void *src, size_t bytes) -> int {
        if (bytes == 0) return SFEM_OK;
        SFEM_TRY(sfem_check_ptr(ctx, src, mem_space));
        if (graph_copyable(src)) {
            in->push_back({dst, src, bytes});
            return SFEM_OK;
        }
        return sfem_cuda_status(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream), "upload");
    };
    if (bt->b > 1) {
        SFEM_TRY(add(bt->E, Young, sizeof(double) * *nYoung));
        SFEM_TRY(add(bt->nu, nu, sizeof(double) * *nNu));
    }
    SFEM_TRY(add(bt->fdofs, fixed_dofs, sizeof(int64_t) * nfix));
    SFEM_TRY(add(bt->fvals, fixed_vals, sizeof(double) * nfix));
    // the previous solve has finished (solves end with a stream synchronise),
    // so the pinned table can be rewritten
    for (int64_t m = 0; m < nm; ++m) {
        bt->h_meshes[m].fix0 = fo[m];
        bt->h_meshes[m].fix1 = fo[m + 1];
    }
    memcpy(bt->h_tab, bt->h_meshes.data(), sizeof(BatchMesh) * nm);
    in->push_back({bt->meshes, bt->h_tab, sizeof(BatchMesh) * nm});
    return SFEM_OK;
}

static int run_copies(sfem_ctx *ctx, const std::vector<GCopy> &cs) {
    for (const GCopy &c : cs)
        SFEM_CUDA(ctx, cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDefault, ctx->stream));
    return SFEM_OK;
}

// Launch the persistent kernel over the meshes order[0..n) (decreasing size;
// `nodes` holds their node counts in the same order).
static int batch_run(sfem_ctx *ctx, sfem_batch *bt, const sfem_solve_opts &o, int plane, int64_t nYoung,
                     int64_t nNu, const int *order, int64_t n, const int64_t *nodes, sfem_batch_stats *dstats) {
    sfem_mesh *m = bt->mesh;
    BatchArgs a;
    memset(&a, 0, sizeof(a));
    a.meshes = bt->meshes;
    a.order = order;
    a.nmesh = n;
    a.nbig = 0;
    if (bt->cluster > 1)
        while (a.nbig < n && nodes[a.nbig] >= bt->big_nodes) ++a.nbig;
    a.queue = bt->queue;
    a.X = m->X;
    a.ien = m->ien;
    a.nEl = m->nEl;
    a.n2e_ptr = m->n2e_ptr;
    a.n2e = m->n2e;
    a.rowlen = m->rowlen;
    a.sliceptr = m->sliceptr;
    a.col = m->col;
    a.g2i = m->g2i;
    a.id = m->id;
    a.nN = m->nN;
    a.n_global = m->n_global;
    a.E = bt->E;
    a.nE = nYoung;
    a.nu = bt->nu;
    a.nNu = nNu;
    a.plane = plane;
    a.fix_dofs = bt->fdofs;
    a.fix_vals = bt->fvals;
    a.kbuf = bt->kbuf;
    a.val64 = bt->val64;
    a.val32 = bt->val32;
    a.fixed = bt->fixed;
    a.gfixed = bt->gfixed;
    a.ud = bt->ud;
    a.b64 = bt->b64;
    a.x64 = bt->x64;
    a.q64 = bt->q64;
    a.vecT = bt->vecT;
    a.nd = m->nN * bt->b;
    a.u_out = bt->u;
    a.rtol = o.rtol;
    a.delta2 = o.reliable_delta * o.reliable_delta;
    a.maxit = o.maxit > 0 ? o.maxit : 1000000;
    a.block_jacobi = o.precond != SFEM_PC_JACOBI ? 1 : 0;
    if (o.precond == SFEM_PC_MULTIGRID && o.precision == SFEM_MIXED) {
        SFEM_TRY(batch_mg(ctx, bt));
        if (bt->mg_any) a.mg = bt->mg_rec;
    }
    a.stats = dstats;
    a.err = ctx->d_err;
    a.nmesh_all = bt->nmesh;
    return o.precision == SFEM_MIXED ? dispatch_batch<true>(ctx, bt, a) : dispatch_batch<false>(ctx, bt, a);
}

static int batch_opts(sfem_ctx *ctx, const sfem_solve_opts *opts, sfem_solve_opts *o) {
    sfem_solve_opts_default(o);
    if (opts) *o = *opts;
    if (!(o->rtol >= 0.0) || o->maxit < 0 || (o->precision != SFEM_FP64 && o->precision != SFEM_MIXED) ||
        o->precond < SFEM_PC_JACOBI || o->precond > SFEM_PC_MULTIGRID ||
        !(o->reliable_delta > 0.0 && o->reliable_delta < 1.0))
        return sfem_set_error(ctx, SFEM_BAD_ARG, "bad solve options");
    return SFEM_OK;
}

template <typename V>
static void key_put(std::vector<unsigned char> &k, const V &v) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(&v);
    k.insert(k.end(), p, p + sizeof(V));
}

// One solve = one CUDA graph launch: the uploads from device or pinned
// memory, the clearing of u and of the work queue, the persistent kernel, and
// the copies of u (to device or pinned memory) and of the statistics.  The
// graph is captured at the first solve and launched again as long as
// nothing it holds changes (options, launch shape, buffer addresses, the
// caller's device or pinned pointers); otherwise it is captured anew.
extern "C" int sfem_batch_solve(sfem_ctx *ctx, sfem_batch *bt, int plane, const double *Young, int64_t nYoung,
                                const double *nu, int64_t nNu, const int64_t *fix_offsets, const int64_t *fixed_dofs,
                                const double *fixed_vals, double *u_out, int mem_space, const sfem_solve_opts *opts,
                                sfem_batch_stats *stats) {
    SfemRange range_("sfem batch solve");
    if (!ctx || !bt || !u_out || !fix_offsets) return SFEM_BAD_ARG;
    cudaSetDevice(ctx->device);
    sfem_solve_opts o;
    SFEM_TRY(batch_opts(ctx, opts, &o));
    std::vector<GCopy> in;
    SFEM_TRY(batch_upload(ctx, bt, plane, Young, &nYoung, nu, &nNu, fix_offsets, fixed_dofs, fixed_vals, mem_space,
                          &in));
    SFEM_TRY(sfem_check_ptr(ctx, u_out, mem_space));
    if (o.precond == SFEM_PC_MULTIGRID && o.precision == SFEM_MIXED) SFEM_TRY(batch_mg(ctx, bt));  // allocates once
    const int64_t nm = bt->nmesh;
    const size_t ubytes = sizeof(double) * bt->total_dofs;
    const bool u_in_graph = graph_copyable(u_out);
    std::vector<unsigned char> key;
    key_put(key, o.precision);
    key_put(key, o.precond);
    key_put(key, o.rtol);
    key_put(key, o.maxit);
    key_put(key, o.reliable_delta);
    key_put(key, plane);
    key_put(key, nYoung);
    key_put(key, nNu);
    key_put(key, bt->threads);
    key_put(key, bt->ctas_per_sm);
    key_put(key, bt->cluster);
    key_put(key, bt->big_nodes);
    key_put(key, (const void *)bt->E);
    key_put(key, (const void *)bt->nu);
    key_put(key, (const void *)bt->fdofs);
    key_put(key, (const void *)bt->fvals);
    key_put(key, (const void *)bt->mg_rec);
    key_put(key, bt->mg_any);
    for (const GCopy &c : in) key_put(key, c);
    key_put(key, u_in_graph ? (const void *)u_out : nullptr);
    if (!bt->gexec || key != bt->gkey) {
        if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
        bt->gexec = nullptr;
        bt->gkey.clear();
        const long long launches = ctx->launches;
        SFEM_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int st = run_copies(ctx, in);
        if (st == SFEM_OK)
            st = sfem_cuda_status(ctx, cudaMemsetAsync(bt->u, 0, sizeof(double) * (bt->total_dofs + 1), ctx->stream),
                                  "memset");
        if (st == SFEM_OK) st = batch_run(ctx, bt, o, plane, nYoung, nNu, bt->order, nm, bt->h_nodes.data(), bt->d_stats);
        if (st == SFEM_OK && u_in_graph)
            st = sfem_cuda_status(ctx, cudaMemcpyAsync(u_out, bt->u, ubytes, cudaMemcpyDefault, ctx->stream), "copy-out");
        if (st == SFEM_OK)
            st = sfem_cuda_status(ctx, cudaMemcpyAsync(bt->h_stats, bt->d_stats, sizeof(sfem_batch_stats) * nm,
                                                       cudaMemcpyDeviceToHost, ctx->stream),
                                  "stats copy");
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
        ctx->launches = launches;  // counted per graph launch below
        if (st == SFEM_OK && ec != cudaSuccess) st = sfem_cuda_status(ctx, ec, "batch graph capture");
        if (st == SFEM_OK) st = sfem_cuda_status(ctx, cudaGraphInstantiate(&bt->gexec, g, 0), "batch graph instantiate");
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (st != SFEM_OK) {
            bt->gexec = nullptr;
            cudaStreamSynchronize(ctx->stream);
            return st;
        }
        bt->gkey = key;
    }
    int st = sfem_cuda_status(ctx, cudaGraphLaunch(bt->gexec, ctx->stream), "batch graph launch");
    if (st == SFEM_OK) ctx->launches += 1;
    if (st == SFEM_OK && !u_in_graph) st = sfem_copy_out(ctx, u_out, bt->u, ubytes, mem_space);
    if (st == SFEM_OK) st = sfem_check_device(ctx, "batch solve");
    if (st == SFEM_OK && stats)
        st = sfem_cuda_status(ctx, cudaMemcpy(stats, bt->h_stats, sizeof(sfem_batch_stats) * nm, cudaMemcpyDefault),
                              "stats copy");
    cudaStreamSynchronize(ctx->stream);
    return st;
}

// Autotuner: time candidate launch shapes on a sample of the batch (every
// k-th mesh in size order, so the sample keeps the batch's size mix) and
// keep the fastest.
extern "C" int sfem_batch_autotune(sfem_ctx *ctx, sfem_batch *bt, int plane, const double *Young, int64_t nYoung,
                                   const double *nu, int64_t nNu, const int64_t *fix_offsets,
                                   const int64_t *fixed_dofs, const double *fixed_vals, int mem_space,
                                   const sfem_solve_opts *opts, int64_t sample, double *best_ms) {
    if (!ctx || !bt || !fix_offsets) return SFEM_BAD_ARG;
    cudaSetDevice(ctx->device);
    sfem_solve_opts o;
    SFEM_TRY(batch_opts(ctx, opts, &o));
    std::vector<GCopy> in;
    SFEM_TRY(batch_upload(ctx, bt, plane, Young, &nYoung, nu, &nNu, fix_offsets, fixed_dofs, fixed_vals, mem_space,
                          &in));
    SFEM_TRY(run_copies(ctx, in));
    const int64_t nm = bt->nmesh;
    const int64_t stride = std::max<int64_t>(1, sample > 0 ? nm / sample : 1);
    std::vector<int> horder(nm);
    SFEM_CUDA(ctx, cudaMemcpy(horder.data(), bt->order, sizeof(int) * nm, cudaMemcpyDeviceToHost));
    std::vector<int> sub;
    std::vector<int64_t> subnodes;
    for (int64_t q = 0; q < nm; q += stride) {
        sub.push_back(horder[q]);
        subnodes.push_back(bt->h_nodes[q]);
    }
    const int64_t ns = (int64_t)sub.size();
    int *dsub = nullptr;
    sfem_batch_stats *dstats = nullptr;
    SFEM_TRY(sfem_dalloc(ctx, (void **)&dsub, sizeof(int) * ns, "autotune order"));
    SFEM_TRY(sfem_dalloc(ctx, (void **)&dstats, sizeof(sfem_batch_stats) * nm, "autotune stats"));
    SFEM_TRY(sfem_copy_in(ctx, dsub, sub.data(), sizeof(int) * ns, SFEM_MEM_HOST));
    struct Cand { int threads, ctas, cluster; int64_t min_nodes; };
    // Candidates span "every CTA on its own mesh" to clusters of 4 or 8 CTAs
    // on the larger meshes (measured on GB300: 16-CTA clusters leave too few
    // meshes in flight and lose).
    const int64_t big = bt->ndim == 2 ? 16384 : 32768;
    const Cand cands[] = {{512, 1, 1, big},     {512, 2, 1, big},     {512, 1, 4, big},
                          {512, 1, 4, big / 4}, {512, 1, 8, big / 4}, {512, 1, 8, big},
                          {256, 2, 4, big}};
    const int nc = (int)(sizeof(cands) / sizeof(cands[0]));
    cudaEvent_t e0, e1;
    SFEM_CUDA(ctx, cudaEventCreate(&e0));
    SFEM_CUDA(ctx, cudaEventCreate(&e1));
    double best = 1e300;
    Cand pick = {bt->threads, bt->ctas_per_sm, bt->cluster, bt->big_nodes};
    int st = SFEM_OK;
    for (int c = 0; c < nc && st == SFEM_OK; ++c) {
        if (sfem_batch_set_launch(bt, cands[c].threads, cands[c].ctas, cands[c].cluster, cands[c].min_nodes) != SFEM_OK)
            continue;
        cudaEventRecord(e0, ctx->stream);
        st = batch_run(ctx, bt, o, plane, nYoung, nNu, dsub, ns, subnodes.data(), dstats);
        cudaEventRecord(e1, ctx->stream);
        if (st != SFEM_OK) break;
        SFEM_CUDA(ctx, cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            pick = cands[c];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sfem_dfree(ctx, dsub);
    sfem_dfree(ctx, dstats);
    sfem_batch_set_launch(bt, pick.threads, pick.ctas, pick.cluster, pick.min_nodes);
    if (st == SFEM_OK) st = sfem_check_device(ctx, "batch autotune");
    if (best_ms) *best_ms = best;
    return st;
}

extern "C" int sfem_batch_get_launch(const sfem_batch *bt, int *threads, int *ctas_per_sm, int *cluster,
                                     int64_t *cluster_min_nodes, int *last_grid) {
    if (!bt) return SFEM_BAD_ARG;
    if (threads) *threads = bt->threads;
    if (ctas_per_sm) *ctas_per_sm = bt->ctas_per_sm;
    if (cluster) *cluster = bt->cluster;
    if (cluster_min_nodes) *cluster_min_nodes = bt->big_nodes;
    if (last_grid) *last_grid = bt->last_grid;
    return SFEM_OK;
}

extern "C" int sfem_multigrid_info(int ndim, int function_class, int nDof, int64_t nNodes, const int64_t *IEN,
                                   int64_t nEl, int *ne_out, int *levels_out, int64_t *bytes_out) {
    if (ndim != 2 && ndim != 3) return SFEM_BAD_ARG;
    if ((nDof != 1 && nDof != ndim) || nNodes < 1 || nEl < 1 || !IEN) return SFEM_BAD_ARG;
    const int nen = function_class == SFEM_Q2 ? 9 : (1 << ndim);
    const int ne = mg_structured_ne(ndim, function_class, nen, nNodes, nEl, IEN, nEl);
    const int L = mg_levels(ne);
    if (ne_out) *ne_out = ne;
    if (levels_out) *levels_out = L;
    if (bytes_out) *bytes_out = L >= 2 ? mg_layout(ndim, nDof, ne, (nNodes + 31) / 32 * 32 * nDof, nullptr, nullptr) : 0;
    return SFEM_OK;
}

extern "C" int sfem_batch_destroy(sfem_batch *bt) {
    if (!bt) return SFEM_OK;
    sfem_ctx *ctx = bt->ctx;
    cudaSetDevice(ctx->device);
    void *bufs[] = {bt->meshes, bt->order, bt->queue, bt->kbuf, bt->val64, bt->val32, bt->ud, bt->b64, bt->x64,
                    bt->q64, bt->vecT, bt->fixed, bt->gfixed, bt->E, bt->nu, bt->fvals, bt->u, bt->fdofs,
                    bt->fix_off_dev, bt->mg_buf, bt->mg_rec};
    for (void *p : bufs) sfem_dfree(ctx, p);
    sfem_dfree(ctx, bt->d_stats);
    if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
    if (bt->mesh) sfem_mesh_release(bt->mesh);
    cudaStreamSynchronize(ctx->stream);
    if (bt->h_tab) cudaFreeHost(bt->h_tab);
    if (bt->h_stats) cudaFreeHost(bt->h_stats);
    delete bt;
    return SFEM_OK;
}
