// Mesh upload/validation, device pattern build and SparseMatrixCSC export.
//
// The reference gets K's structure from sparse(E,J,V) over the COO triplets
// of every element DOF-pair (src/fem.jl:203-205, 242-244, 253): the union of
// the element blocks, duplicates merged, explicit zeros kept.  With nDof > 1
// every node pair of an element contributes a full nDof x nDof block, so the
// structure is exactly "node pattern (x) dense nDof x nDof block".  Here the
// node pattern is built on the device, without sorting the COO:
//   1. node -> element incidence lists (counting + atomic placement, then a
//      per-node sort so every list is in ascending element order),
//   2. per node, its distinct neighbour nodes in ascending order, enumerated
//      by repeated minimum selection over the incident elements' nodes,
//   3. the rows are laid out as sliced ELL (32 rows per slice) for the SpMV,
//      plus CSR offsets used for the CSC export.
#include <limits.h>

#include <algorithm>
#include <math.h>
#include <string.h>

#include "sfem_internal.cuh"

namespace {

__global__ void k_convert_ien(const int64_t *__restrict__ src, int64_t nEl, int nen, int64_t nN,
                              int *__restrict__ ien, DevErr *err) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nEl * nen) return;
    int64_t v = src[t];
    if (v < 1 || v > nN) {
        sfem_dev_error(err, SFEM_BAD_INDEX, t % nEl);
        v = 1;
    }
    ien[t] = (int)(v - 1);
}

__global__ void k_convert_id(const int64_t *__restrict__ src, int64_t count, int *__restrict__ id,
                             DevErr *err) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    int64_t v = src[t];
    if (v > (int64_t)INT_MAX) {
        sfem_dev_error(err, SFEM_BAD_INDEX, t);
        v = 0;
    }
    id[t] = v >= 1 ? (int)(v - 1) : -1;
}

__global__ void k_n2e_count(const int *__restrict__ ien, int64_t nEl, int nen, int *__restrict__ cnt) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nEl * nen) return;
    atomicAdd(&cnt[ien[t]], 1);
}

__global__ void k_n2e_fill(const int *__restrict__ ien, int64_t nEl, int nen,
                           unsigned long long *__restrict__ cursor, int *__restrict__ n2e) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nEl * nen) return;
    int node = ien[t];
    unsigned long long p = atomicAdd(&cursor[node], 1ull);
    n2e[p] = (int)(t % nEl);
}

// Insertion sort of each node's incident-element list (lists are short).
__global__ void k_n2e_sort(const int64_t *__restrict__ ptr, int *__restrict__ n2e, int64_t nN) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nN) return;
    int64_t s = ptr[r], e = ptr[r + 1];
    for (int64_t i = s + 1; i < e; ++i) {
        int v = n2e[i];
        int64_t j = i - 1;
        while (j >= s && n2e[j] > v) {
            n2e[j + 1] = n2e[j];
            --j;
        }
        n2e[j + 1] = v;
    }
}

// Referenced nodes: validate their ID entries and find the matrix size.
// *maxg receives (largest referenced DOF index) + 1; a warp-level max goes
// first so the single-address atomic sees one request per warp.
__global__ void k_dof_extent(const int64_t *__restrict__ ptr, const int *__restrict__ id, int64_t nN,
                             int b, unsigned int *__restrict__ maxg, DevErr *err) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int v = 0;
    if (r < nN && ptr[r + 1] != ptr[r]) {  // nodes no element uses do not count
        if (b == 1) {
            v = (unsigned int)r + 1u;
        } else {
            for (int d = 0; d < b; ++d) {
                const int g = id[(int64_t)d * nN + r];
                if (g < 0) {
                    sfem_dev_error(err, SFEM_BAD_INDEX, r);
                    continue;
                }
                v = max(v, (unsigned int)g + 1u);
            }
        }
    }
    v = __reduce_max_sync(0xffffffffu, v);  // blocks are whole warps; no thread has returned
    if ((threadIdx.x & 31) == 0 && v) atomicMax(maxg, v);
}

__global__ void k_g2i(const int64_t *__restrict__ ptr, const int *__restrict__ id, int64_t nN, int b,
                      int64_t ng, int *__restrict__ g2i, DevErr *err) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nN) return;
    if (ptr[r + 1] == ptr[r]) return;
    for (int d = 0; d < b; ++d) {
        int g = b == 1 ? (int)r : id[(int64_t)d * nN + r];
        if (g < 0 || g >= ng) continue;
        int old = atomicCAS(&g2i[g], -1, (int)(r * b + d));
        if (old != -1) {
            err->aux = 1;
            sfem_dev_error(err, SFEM_BAD_ARG, g);  // two (node, component) pairs share a DOF id
        }
    }
}

// Distinct neighbours of node r in ascending order by repeated minimum
// selection over the nodes of its incident elements.  Writes them to
// out[k*stride] when out != nullptr; returns their count.
__device__ int row_neighbours(int r, const int64_t *__restrict__ n2e_ptr, const int *__restrict__ n2e,
                              const int *__restrict__ ien, int64_t nEl, int nen, int *out, int64_t stride) {
    const int64_t s = n2e_ptr[r], t = n2e_ptr[r + 1];
    int prev = -1, k = 0;
    while (true) {
        int best = INT_MAX;
        for (int64_t q = s; q < t; ++q) {
            const int e = n2e[q];
            for (int a = 0; a < nen; ++a) {
                int c = __ldg(&ien[(int64_t)a * nEl + e]);
                if (c > prev && c < best) best = c;
            }
        }
        if (best == INT_MAX) break;
        if (out) out[(int64_t)k * stride] = best;
        prev = best;
        ++k;
    }
    return k;
}

// The same selection with the node lists of up to MAXE incident elements
// held in registers (loaded once, all loads in flight together); rows with
// more incident elements take row_neighbours.
template <int NEN, int MAXE>
__device__ int row_neighbours_reg(int r, const int64_t *__restrict__ n2e_ptr, const int *__restrict__ n2e,
                                  const int *__restrict__ ien, int64_t nEl, int *out, int64_t stride) {
    const int64_t s = n2e_ptr[r], t = n2e_ptr[r + 1];
    if (t - s > MAXE) return row_neighbours(r, n2e_ptr, n2e, ien, nEl, NEN, out, stride);
    const int n = (int)(t - s);
    int nodes[MAXE * NEN];
#pragma unroll
    for (int m = 0; m < MAXE; ++m) {
        const int e = m < n ? n2e[s + m] : 0;
#pragma unroll
        for (int a = 0; a < NEN; ++a) nodes[m * NEN + a] = m < n ? __ldg(&ien[(int64_t)a * nEl + e]) : INT_MAX;
    }
    int prev = -1, k = 0;
    while (true) {
        int best = INT_MAX;
#pragma unroll
        for (int i = 0; i < MAXE * NEN; ++i) best = (nodes[i] > prev && nodes[i] < best) ? nodes[i] : best;
        if (best == INT_MAX) break;
        if (out) out[(int64_t)k * stride] = best;
        prev = best;
        ++k;
    }
    return k;
}

// NEN > 0: the register form for NEN nodes per element; NEN = 0: any nen.
template <int NEN, int MAXE>
__device__ __forceinline__ int row_neighbours_any(int r, const int64_t *__restrict__ n2e_ptr,
                                                  const int *__restrict__ n2e, const int *__restrict__ ien,
                                                  int64_t nEl, int nen, int *out, int64_t stride) {
    if constexpr (NEN > 0) return row_neighbours_reg<NEN, MAXE>(r, n2e_ptr, n2e, ien, nEl, out, stride);
    else return row_neighbours(r, n2e_ptr, n2e, ien, nEl, nen, out, stride);
}

template <int NEN, int MAXE>
__global__ void k_rowlen(const int64_t *__restrict__ n2e_ptr, const int *__restrict__ n2e,
                         const int *__restrict__ ien, int64_t nEl, int nen, int64_t nN,
                         int *__restrict__ rowlen) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nN) return;
    rowlen[r] = row_neighbours_any<NEN, MAXE>((int)r, n2e_ptr, n2e, ien, nEl, nen, nullptr, 0);
}

__global__ void k_slice_width(const int *__restrict__ rowlen, int64_t nN, int64_t nslices,
                              int64_t *__restrict__ width) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t s = t >> 5;
    int lane = threadIdx.x & 31;
    if (s >= nslices) return;  // whole warps exit together (slices are warp-aligned)
    int64_t r = s * 32 + lane;
    int w = r < nN ? rowlen[r] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w = max(w, __shfl_xor_sync(0xffffffffu, w, o));
    if (lane == 0) width[s] = w;
}

template <int NEN, int MAXE>
__global__ void k_rowfill(const int64_t *__restrict__ n2e_ptr, const int *__restrict__ n2e,
                          const int *__restrict__ ien, int64_t nEl, int nen, int64_t nN,
                          const int *__restrict__ rowlen, const int64_t *__restrict__ sliceptr,
                          int *__restrict__ col) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t s = r >> 5;
    int lane = (int)(r & 31);
    int64_t nsl = sfem_cdiv(nN, 32);
    if (s >= nsl) return;
    int64_t slab0 = sliceptr[s], width = sliceptr[s + 1] - slab0;
    int *base = col + slab0 * 32 + lane;
    int len = 0;
    if (r < nN) len = row_neighbours_any<NEN, MAXE>((int)r, n2e_ptr, n2e, ien, nEl, nen, base, 32);
    int self = r < nN ? (int)r : 0;
    for (int64_t k = len; k < width; ++k) base[k * 32] = self;  // padding: (own node, value 0)
}

// CSC export.  Thread per (node c, component dj): column g = ID[c, dj].
// K is stored with bitwise-symmetric blocks (block(r,c) == block(c,r)^T),
// so column (c,dj) is read from row c: K[(r,di),(c,dj)] = block(c,r)[dj][di].
__global__ void k_csc_count(const int *__restrict__ rowlen, const int *__restrict__ id, int64_t nN, int b,
                            int64_t *__restrict__ colcnt) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nN * b) return;
    int64_t c = t / b;
    int dj = (int)(t % b);
    int len = rowlen[c];
    if (len == 0) return;
    int g = b == 1 ? (int)c : id[(int64_t)dj * nN + c];
    colcnt[g] = (int64_t)len * b;
}

__global__ void k_csc_fill(const int *__restrict__ rowlen, const int *__restrict__ id, int64_t nN, int b,
                           const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                           const double *__restrict__ val, const int64_t *__restrict__ colptr0,
                           int64_t *__restrict__ rowval, double *__restrict__ nzval) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nN * b) return;
    int64_t c = t / b;
    int dj = (int)(t % b);
    int len = rowlen[c];
    if (len == 0) return;
    int g = b == 1 ? (int)c : id[(int64_t)dj * nN + c];
    int64_t s = c >> 5;
    int lane = (int)(c & 31);
    int64_t slab0 = sliceptr[s];
    int64_t o = colptr0[g];
    const int64_t o0 = o;
    for (int k = 0; k < len; ++k) {
        int64_t slab = slab0 + k;
        int r = col[slab * 32 + lane];
        for (int di = 0; di < b; ++di) {
            int64_t grow = b == 1 ? r : id[(int64_t)di * nN + r];
            double v = nzval ? val[(slab * b * b + dj * b + di) * 32 + lane] : 0.0;
            // insertion keeps the column sorted even for a non-monotone ID
            int64_t j = o - 1;
            while (j >= o0 && rowval[j] > grow + 1) {
                rowval[j + 1] = rowval[j];
                if (nzval) nzval[j + 1] = nzval[j];
                --j;
            }
            rowval[j + 1] = grow + 1;
            if (nzval) nzval[j + 1] = v;
            ++o;
        }
    }
}

__global__ void k_colptr_1based(const int64_t *__restrict__ in, int64_t n, int64_t *__restrict__ out) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t <= n) out[t] = in[t] + 1;
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)sfem_cdiv(n > 0 ? n : 1, t); }

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" int sfem_mesh_create(sfem_ctx *ctx, int ndim, int function_class, int nDof, int64_t ne,
                                const double *NodeList, int64_t nNodes, const int64_t *IEN,
                                int64_t ldIEN, int nen, const int64_t *ID, int mem_space,
                                sfem_mesh **out) {
    if (!ctx || !out) return SFEM_BAD_ARG;
    if (ne < 0) return sfem_set_error(ctx, SFEM_BAD_ARG, "bad ne");
    double nel_d = pow((double)ne, (double)ndim);
    if (ndim >= 2 && ndim <= 3 && nel_d * nen > (double)INT_MAX)
        return sfem_set_error(ctx, SFEM_BAD_ARG, "mesh too large (nEl*nen >= 2^31)");
    int64_t nEl = 1;
    for (int d = 0; d < ndim && ndim <= 3; ++d) nEl *= ne;  // src/fem.jl:179: elements 1:ne^ndim
    int st = sfem_mesh_create_nel(ctx, ndim, function_class, nDof, nEl, NodeList, nNodes, IEN, ldIEN, nen, ID,
                                  mem_space, out);
    if (st == SFEM_OK) (*out)->ne = ne;
    return st;
}

int sfem_mesh_create_nel(sfem_ctx *ctx, int ndim, int function_class, int nDof, int64_t nEl,
                         const double *NodeList, int64_t nNodes, const int64_t *IEN, int64_t ldIEN, int nen,
                         const int64_t *ID, int mem_space, sfem_mesh **out) {
    if (!ctx || !out) return SFEM_BAD_ARG;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    if (ndim == 1)
        return sfem_set_error(ctx, SFEM_UNSUPPORTED,
                              "1D assembly: the reference's coords*dN is a dimension mismatch "
                              "(src/fem.jl:75,192)");
    if (ndim != 2 && ndim != 3) return sfem_set_error(ctx, SFEM_BAD_ARG, "ndim must be 2 or 3");
    if (function_class == SFEM_Q1) {
        if (nen != (1 << ndim))
            return sfem_set_error(ctx, SFEM_BAD_ARG, "Q1 in %dD needs %d nodes per element", ndim, 1 << ndim);
    } else if (function_class == SFEM_Q2) {
        if (ndim != 2 || nen != 9)
            return sfem_set_error(ctx, SFEM_UNSUPPORTED, "Q2 is defined for 2D 9-node elements only");
        if (nDof != 1)
            return sfem_set_error(ctx, SFEM_UNSUPPORTED,
                                  "vector Q2 overruns the reference's COO arrays (src/fem.jl:143-145)");
    } else {
        return sfem_set_error(ctx, SFEM_BAD_ARG, "FunctionClass must be SFEM_Q1 or SFEM_Q2");
    }
    if (nDof != 1 && nDof != ndim)
        return sfem_set_error(ctx, SFEM_UNSUPPORTED, "vector assembly needs nDof == ndim (src/fem.jl:210-231)");
    if (nDof > 1 && !ID) return sfem_set_error(ctx, SFEM_BAD_ARG, "ID is required when nDof > 1");
    if (nEl < 0 || nNodes < 1 || nNodes > INT_MAX / 4) return sfem_set_error(ctx, SFEM_BAD_ARG, "bad nEl/nNodes");
    if ((double)nEl * nen > (double)INT_MAX) return sfem_set_error(ctx, SFEM_BAD_ARG, "mesh too large (nEl*nen >= 2^31)");
    if (nEl > ldIEN)
        return sfem_set_error(ctx, SFEM_BAD_INDEX, "IEN has %lld rows but ne^ndim = %lld elements are assembled",
                              (long long)ldIEN, (long long)nEl);
    if (nEl > 0 && (!NodeList || !IEN)) return sfem_set_error(ctx, SFEM_BAD_ARG, "NULL NodeList/IEN");

    sfem_mesh *m = new sfem_mesh();
    m->ctx = ctx;
    m->ndim = ndim;
    m->nen = nen;
    m->fclass = function_class;
    m->b = nDof;
    m->ne = 0;
    m->nEl = nEl;
    m->nN = nNodes;
    int st = SFEM_OK;
    int64_t *tmp = nullptr;
    do {
        if ((st = sfem_dalloc(ctx, (void **)&m->X, sizeof(double) * ndim * nNodes, "NodeList"))) break;
        if ((st = sfem_copy_in(ctx, m->X, NodeList, sizeof(double) * ndim * nNodes, mem_space))) break;
        if ((st = sfem_dalloc(ctx, (void **)&m->ien, sizeof(int) * nen * (nEl ? nEl : 1), "IEN"))) break;
        size_t tmp_elems = (size_t)std::max<int64_t>(nEl * nen, nDof > 1 ? nNodes * nDof : 1);
        if ((st = sfem_dalloc(ctx, (void **)&tmp, sizeof(int64_t) * tmp_elems, "IEN staging"))) break;
        if (nEl > 0) {
            if (ldIEN == nEl) {
                if ((st = sfem_copy_in(ctx, tmp, IEN, sizeof(int64_t) * nEl * nen, mem_space))) break;
            } else {
                if ((st = sfem_check_ptr(ctx, IEN, mem_space))) break;
                st = sfem_cuda_status(ctx,
                                      cudaMemcpy2DAsync(tmp, sizeof(int64_t) * nEl, IEN, sizeof(int64_t) * ldIEN,
                                                        sizeof(int64_t) * nEl, nen, cudaMemcpyDefault, ctx->stream),
                                      "IEN copy");
                if (st) break;
            }
            k_convert_ien<<<blocks_for(nEl * nen, 256), 256, 0, ctx->stream>>>(tmp, nEl, nen, nNodes, m->ien,
                                                                             ctx->d_err);
            SFEM_LAUNCHED(ctx);
        }
        if (nDof > 1) {
            if ((st = sfem_dalloc(ctx, (void **)&m->id, sizeof(int) * nDof * nNodes, "ID"))) break;
            if ((st = sfem_check_device(ctx, "IEN validation"))) break;  // tmp reused below
            if ((st = sfem_copy_in(ctx, tmp, ID, sizeof(int64_t) * nDof * nNodes, mem_space))) break;
            k_convert_id<<<blocks_for(nNodes * nDof, 256), 256, 0, ctx->stream>>>(tmp, nNodes * nDof, m->id,
                                                                                 ctx->d_err);
            SFEM_LAUNCHED(ctx);
        }
        st = sfem_check_device(ctx, "mesh upload");
    } while (0);
    sfem_dfree(ctx, tmp);
    if (st != SFEM_OK) {
        sfem_mesh_release(m);
        return st;
    }
    *out = m;
    return SFEM_OK;
}

void sfem_mesh_release(sfem_mesh *m) {
    if (!m) return;
    if (--m->refcnt > 0) return;
    sfem_ctx *ctx = m->ctx;
    cudaSetDevice(ctx->device);
    void *bufs[] = {m->X, m->ien, m->id, m->n2e_ptr, m->n2e, m->rowlen, m->rowptr, m->sliceptr, m->col, m->g2i};
    for (void *p : bufs) sfem_dfree(ctx, p);
    cudaStreamSynchronize(ctx->stream);
    delete m;
}

extern "C" int sfem_mesh_destroy(sfem_mesh *m) {
    sfem_mesh_release(m);
    return SFEM_OK;
}

extern "C" int sfem_pattern_build(sfem_ctx *ctx, sfem_mesh *m, int64_t *n_out, int64_t *nnz_out) {
    SfemRange range_("sfem pattern");
    if (!ctx || !m) return SFEM_BAD_ARG;
    cudaSetDevice(ctx->device);
    if (m->has_pattern) {
        if (n_out) *n_out = m->n_global;
        if (nnz_out) *nnz_out = m->nnzb * m->b * m->b;
        return SFEM_OK;
    }
    const int64_t nN = m->nN, nEl = m->nEl;
    const int nen = m->nen, b = m->b;
    cudaStream_t s = ctx->stream;
    int *cnt = nullptr;
    unsigned long long *cursor = nullptr;
    int64_t *widths = nullptr;
    int st = SFEM_OK;
    do {
        if ((st = sfem_dalloc(ctx, (void **)&cnt, sizeof(int) * nN, "n2e counts"))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemsetAsync(cnt, 0, sizeof(int) * nN, s), "memset"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&m->n2e_ptr, sizeof(int64_t) * (nN + 1), "n2e_ptr"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&m->n2e, sizeof(int) * (nEl * nen ? nEl * nen : 1), "n2e"))) break;
        if (nEl > 0) {
            k_n2e_count<<<blocks_for(nEl * nen, 256), 256, 0, s>>>(m->ien, nEl, nen, cnt);
            SFEM_LAUNCHED(ctx);
        }
        if ((st = sfem_scan_i32(ctx, cnt, m->n2e_ptr, nN))) break;
        if ((st = sfem_dalloc(ctx, (void **)&cursor, sizeof(int64_t) * nN, "n2e cursor"))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(cursor, m->n2e_ptr, sizeof(int64_t) * nN,
                                                        cudaMemcpyDeviceToDevice, s), "memcpy")))
            break;
        if (nEl > 0) {
            k_n2e_fill<<<blocks_for(nEl * nen, 256), 256, 0, s>>>(m->ien, nEl, nen, cursor, m->n2e);
            SFEM_LAUNCHED(ctx);
        }
        k_n2e_sort<<<blocks_for(nN, 128), 128, 0, s>>>(m->n2e_ptr, m->n2e, nN);
        SFEM_LAUNCHED(ctx);

        // matrix size and global DOF -> internal index
        unsigned int *dmax = (unsigned int *)cursor;  // reuse
        if ((st = sfem_cuda_status(ctx, cudaMemsetAsync(dmax, 0, sizeof(unsigned int), s), "memset")))
            break;
        k_dof_extent<<<blocks_for(nN, 256), 256, 0, s>>>(m->n2e_ptr, m->id, nN, b, dmax, ctx->d_err);
        SFEM_LAUNCHED(ctx);
        unsigned long long *h = (unsigned long long *)ctx->h_small;
        unsigned int *h32 = (unsigned int *)ctx->h_small;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(h32, dmax, 4, cudaMemcpyDeviceToHost, s), "memcpy")))
            break;
        if ((st = sfem_check_device(ctx, "ID validation"))) break;
        int64_t ng = (int64_t)h32[0];
        m->n_global = ng;
        if ((st = sfem_dalloc(ctx, (void **)&m->g2i, sizeof(int) * (ng ? ng : 1), "g2i"))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemsetAsync(m->g2i, 0xff, sizeof(int) * (ng ? ng : 1), s), "memset")))
            break;
        k_g2i<<<blocks_for(nN, 256), 256, 0, s>>>(m->n2e_ptr, m->id, nN, b, ng, m->g2i, ctx->d_err);
        SFEM_LAUNCHED(ctx);

        // rows
        if ((st = sfem_dalloc(ctx, (void **)&m->rowlen, sizeof(int) * nN, "rowlen"))) break;
        // Q1 quads / hexes and Q2 quads: element node lists in registers
        if (nen == 8)
            k_rowlen<8, 8><<<blocks_for(nN, 128), 128, 0, s>>>(m->n2e_ptr, m->n2e, m->ien, nEl, nen, nN, m->rowlen);
        else if (nen == 4)
            k_rowlen<4, 6><<<blocks_for(nN, 128), 128, 0, s>>>(m->n2e_ptr, m->n2e, m->ien, nEl, nen, nN, m->rowlen);
        else if (nen == 9)
            k_rowlen<9, 4><<<blocks_for(nN, 128), 128, 0, s>>>(m->n2e_ptr, m->n2e, m->ien, nEl, nen, nN, m->rowlen);
        else
            k_rowlen<0, 0><<<blocks_for(nN, 128), 128, 0, s>>>(m->n2e_ptr, m->n2e, m->ien, nEl, nen, nN, m->rowlen);
        SFEM_LAUNCHED(ctx);
        m->nslices = sfem_cdiv(nN, 32);
        if ((st = sfem_dalloc(ctx, (void **)&widths, sizeof(int64_t) * m->nslices, "slice widths"))) break;
        k_slice_width<<<blocks_for(m->nslices * 32, 256), 256, 0, s>>>(m->rowlen, nN, m->nslices, widths);
        SFEM_LAUNCHED(ctx);
        if ((st = sfem_dalloc(ctx, (void **)&m->sliceptr, sizeof(int64_t) * (m->nslices + 1), "sliceptr"))) break;
        if ((st = sfem_scan_i64(ctx, widths, m->sliceptr, m->nslices))) break;
        if ((st = sfem_dalloc(ctx, (void **)&m->rowptr, sizeof(int64_t) * (nN + 1), "rowptr"))) break;
        if ((st = sfem_scan_i32(ctx, m->rowlen, m->rowptr, nN))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(h, m->sliceptr + m->nslices, 8, cudaMemcpyDeviceToHost, s),
                                   "memcpy")))
            break;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(h + 1, m->rowptr + nN, 8, cudaMemcpyDeviceToHost, s),
                                   "memcpy")))
            break;
        if ((st = sfem_check_device(ctx, "pattern rows"))) break;
        m->nslabs = (int64_t)h[0];
        m->nnzb = (int64_t)h[1];
        if (m->nslabs * 32 * (int64_t)b * b >= ((int64_t)1 << 40)) {
            st = sfem_set_error(ctx, SFEM_BAD_ARG, "pattern too large");
            break;
        }
        if ((st = sfem_dalloc(ctx, (void **)&m->col, sizeof(int) * m->nslabs * 32, "pattern columns"))) break;
        {
            auto fill = nen == 8 ? k_rowfill<8, 8> : nen == 4 ? k_rowfill<4, 6> : nen == 9 ? k_rowfill<9, 4>
                                                                                          : k_rowfill<0, 0>;
            fill<<<blocks_for(m->nslices * 32, 128), 128, 0, s>>>(m->n2e_ptr, m->n2e, m->ien, nEl, nen, nN,
                                                                  m->rowlen, m->sliceptr, m->col);
        }
        SFEM_LAUNCHED(ctx);
        st = sfem_check_device(ctx, "pattern build");
    } while (0);
    sfem_dfree(ctx, cnt);
    sfem_dfree(ctx, cursor);
    sfem_dfree(ctx, widths);
    if (st != SFEM_OK) return st;
    m->has_pattern = true;
    if (n_out) *n_out = m->n_global;
    if (nnz_out) *nnz_out = m->nnzb * b * b;
    return SFEM_OK;
}

extern "C" int sfem_matrix_info(const sfem_matrix *K, int64_t *n, int64_t *nnz) {
    if (!K) return SFEM_BAD_ARG;
    if (n) *n = K->n;
    if (nnz) *nnz = K->nnz;
    return SFEM_OK;
}

extern "C" int sfem_matrix_export_csc(sfem_ctx *ctx, const sfem_matrix *K, int64_t *colptr, int64_t *rowval,
                                      double *nzval, int mem_space) {
    if (!ctx || !K) return SFEM_BAD_ARG;
    cudaSetDevice(ctx->device);
    const sfem_mesh *m = K->mesh;
    const int64_t n = K->n, nnz = K->nnz, nN = m->nN;
    const int b = m->b;
    cudaStream_t s = ctx->stream;
    int64_t *cnt = nullptr, *cp0 = nullptr, *cp1 = nullptr, *rv = nullptr;
    double *nz = nullptr;
    int st = SFEM_OK;
    do {
        if ((st = sfem_dalloc(ctx, (void **)&cnt, sizeof(int64_t) * (n + 1), "colcount"))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (n + 1), s), "memset"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&cp0, sizeof(int64_t) * (n + 1), "colptr"))) break;
        k_csc_count<<<blocks_for(nN * b, 256), 256, 0, s>>>(m->rowlen, m->id, nN, b, cnt);
        SFEM_LAUNCHED(ctx);
        if ((st = sfem_scan_i64(ctx, cnt, cp0, n))) break;
        if (rowval || nzval) {
            if ((st = sfem_dalloc(ctx, (void **)&rv, sizeof(int64_t) * (nnz ? nnz : 1), "rowval"))) break;
            if (nzval && (st = sfem_dalloc(ctx, (void **)&nz, sizeof(double) * (nnz ? nnz : 1), "nzval"))) break;
            k_csc_fill<<<blocks_for(nN * b, 128), 128, 0, s>>>(m->rowlen, m->id, nN, b, m->sliceptr, m->col, K->val,
                                                               cp0, rv, nz);
            SFEM_LAUNCHED(ctx);
            if (rowval && (st = sfem_copy_out(ctx, rowval, rv, sizeof(int64_t) * nnz, mem_space))) break;
            if (nzval && (st = sfem_copy_out(ctx, nzval, nz, sizeof(double) * nnz, mem_space))) break;
        }
        if (colptr) {
            if ((st = sfem_dalloc(ctx, (void **)&cp1, sizeof(int64_t) * (n + 1), "colptr1"))) break;
            k_colptr_1based<<<blocks_for(n + 1, 256), 256, 0, s>>>(cp0, n, cp1);
            SFEM_LAUNCHED(ctx);
            if ((st = sfem_copy_out(ctx, colptr, cp1, sizeof(int64_t) * (n + 1), mem_space))) break;
        }
        st = sfem_check_device(ctx, "CSC export");
    } while (0);
    sfem_dfree(ctx, cnt);
    sfem_dfree(ctx, cp0);
    sfem_dfree(ctx, cp1);
    sfem_dfree(ctx, rv);
    sfem_dfree(ctx, nz);
    cudaStreamSynchronize(s);
    return st;
}
