// Geometric multigrid preconditioner for structured Q1 meshes (the node
// numbering and connectivity of the reference's meshgrid,
// examples/vector3D.jl:66-101; ne elements per direction, x fastest), used by
// the per-mesh pipeline of batches and servers (process_mesh, one group per
// mesh) and, as grid-wide launches, by the single-mesh mixed solver.
//
// Hierarchy.  Level l has n_l elements per direction; n_{l+1} = ceil(n_l / 2)
// until n <= 2.  Coarse node I sits on fine node c(I) = min(2I, n_l) in each
// direction (an odd n_l leaves one last interval of width 1).  Prolongation
// is the tensor product of the 1D interpolation: weight 1 on the coinciding
// node, 1/2 on an odd fine node between two coarse ones, per displacement
// component.  Fixed DOFs are taken out on both sides: a fine DOF that is
// fixed gets no correction, and a coarse DOF is fixed when its coinciding
// fine DOF is, so P' = diag(free_f) P diag(free_c).
//
// Coarse operators are Galerkin products A_{l+1} = P'^T A_l P' with A_0 the
// masked K rounded to FP32.  Their node pattern is again the 3^ndim
// neighbourhood, so they are stored as stencils: block (I, I + offset s) in
// tiles of 32 nodes (mg_a), zero where the neighbour is off the grid.
//
// Cycle: V(1,1) with l1-scaled block Jacobi (x += w_i D_i^-1 r_i with
// w_i = (4/3) / rho_i, rho_i = max row sum of |D_i^-1 A_i*|; convergent
// without eigenvalue estimates since rho(W D^-1 A) <= 4/3) and an exact solve
// (dense inverse, Gauss-Jordan in FP64) on the coarsest level.  The
// pre-smoothing sweep from zero is x = w D^-1 r; the post-smoothing sweep
// is the same operator, so the cycle is a symmetric positive definite
// preconditioner for CG.
//
// Every pass is a loop over the group's (or the grid's) threads with a
// barrier (or a launch boundary) after it, and no atomics on values: a
// mesh's result does not depend on what else runs.
//
// Included by sfem_meshsolve.cuh after the group SpMV and the group types.
#pragma once

constexpr int MG_MAX_LEVELS = 12;

struct MgLevel {
    int n;              // elements per direction
    int nnode;          // (n + 1)^ndim
    float *A;           // levels >= 1: stencil blocks, see mg_a
    float *minv;        // l1-scaled block-Jacobi inverse [nnode][B][B]
    unsigned char *fr;  // levels >= 1: 1 for a free DOF [nnode * B]
    float *x, *b, *t;   // iterate, right-hand side (levels >= 1), residual / smoothed iterate
};

// Levels at or below this size (with a next-finer level of at most
// MG_SOLO_FINE nodes) are run by one CTA of a group when a thread-block
// cluster works on the mesh: a CTA barrier costs a fraction of a cluster
// barrier, and the few hundred nodes of such a level keep one CTA busy.
constexpr int MG_SOLO_NODES = 1024;
constexpr int MG_SOLO_FINE = 8192;

struct MgMesh {
    int nlev;  // levels, the fine one included (>= 2)
    int ndc;   // DOFs of the coarsest level
    int solo;  // first level run by one CTA of a cluster group (nlev: none)
    MgLevel lev[MG_MAX_LEVELS];
    float *cinv;  // inverse of the coarsest operator [ndc][ndc]; fixed rows and columns zero
    double *gj;   // Gauss-Jordan scratch [ndc][2 ndc]
};

// Levels of a structured mesh with ne elements per direction (0: too small
// for a hierarchy).
inline int mg_levels(int ne) {
    if (ne < 3) return 0;
    int L = 1;
    for (int n = ne; n > 2; n = (n + 1) / 2) ++L;
    return L <= MG_MAX_LEVELS ? L : 0;
}

// Device layout of one mesh's hierarchy: the MgMesh record itself, then the
// arrays, each 256-byte aligned.  With base == nullptr only the size is
// computed.  ndp: the mesh's padded DOF count (fine vectors follow the CG's).
inline int64_t mg_layout(int ndim, int B, int ne, int64_t ndp, char *base, MgMesh *out) {
    const int L = mg_levels(ne);
    if (L == 0) return 0;
    int64_t off = 0;
    auto take = [&](int64_t bytes) -> char * {
        off = (off + 255) / 256 * 256;
        char *p = base ? base + off : nullptr;
        off += bytes > 0 ? bytes : 1;
        return p;
    };
    MgMesh m;
    memset(&m, 0, sizeof(m));
    m.nlev = L;
    take(sizeof(MgMesh));
    const int S = ndim == 2 ? 9 : 27;
    int n = ne;
    for (int l = 0; l < L; ++l) {
        MgLevel &v = m.lev[l];
        v.n = n;
        int64_t nn = 1;
        for (int d = 0; d < ndim; ++d) nn *= (n + 1);
        v.nnode = (int)nn;
        const int64_t nd = l == 0 ? ndp : nn * B;
        v.minv = (float *)take(sizeof(float) * nn * B * B);
        v.x = (float *)take(sizeof(float) * nd);
        v.t = (float *)take(sizeof(float) * nd);
        if (l > 0) {
            v.A = (float *)take(sizeof(float) * S * B * B * ((nn + 31) / 32 * 32));
            v.fr = (unsigned char *)take(nn * B);
            v.b = (float *)take(sizeof(float) * nd);
        }
        if (l == L - 1) m.ndc = (int)(nn * B);
        n = (n + 1) / 2;
    }
    m.solo = L;
    for (int l = L - 1; l >= 1; --l) {
        if (m.lev[l].nnode > MG_SOLO_NODES || m.lev[l - 1].nnode > MG_SOLO_FINE) break;
        m.solo = l;
    }
    m.cinv = (float *)take(sizeof(float) * (int64_t)m.ndc * m.ndc);
    m.gj = (double *)take(sizeof(double) * 2 * (int64_t)m.ndc * m.ndc);
    if (out) *out = m;
    return off;
}

// Candidate elements per direction of a mesh with nN nodes and nEl
// elements: ne with ne^ndim == nEl and (ne + 1)^ndim == nN, else 0.
inline int mg_grid_ne(int ndim, int64_t nN, int64_t nEl) {
    auto ipow = [](int64_t b, int e) {
        int64_t r = 1;
        for (int i = 0; i < e; ++i) r *= b;
        return r;
    };
    int64_t ne = 1;
    while (ipow(ne, ndim) < nEl && ne < (1 << 20)) ++ne;
    return (ipow(ne, ndim) == nEl && ipow(ne + 1, ndim) == nN) ? (int)ne : 0;
}

// Node c (1-based) of structured element e of an ne^ndim grid, the
// reference's meshgrid connectivity (examples/vector3D.jl:76-101).
__host__ __device__ inline int64_t mg_grid_node(int ndim, int64_t ne, int64_t e, int c) {
    const int64_t n1 = ne + 1, p = n1 * n1;
    const int64_t i = e % ne, j = (e / ne) % ne, k = e / (ne * ne);
    if (ndim == 2) {
        const int64_t lo = j * n1 + i + 1, hi = (j + 1) * n1 + i + 1;
        return c == 0 ? lo : (c == 1 ? lo + 1 : (c == 2 ? hi + 1 : hi));
    }
    const int64_t base = k * p + j * n1 + i + 1 + (c >= 4 ? p : 0);
    const int q = c & 3;
    return q == 0 ? base : (q == 1 ? base + 1 : (q == 2 ? base + n1 + 1 : base + n1));
}

// Elements per direction when the mesh is the reference's structured grid
// (nodes x fastest, Q1 connectivity as meshgrid makes it), else 0.  IEN is
// column-major with leading dimension ld, 1-based.
inline int mg_structured_ne(int ndim, int fclass, int nen, int64_t nN, int64_t nEl, const int64_t *IEN, int64_t ld) {
    if (fclass != SFEM_Q1 || nen != (1 << ndim) || nEl < 1) return 0;
    const int ne = mg_grid_ne(ndim, nN, nEl);
    if (ne == 0) return 0;
    for (int64_t e = 0; e < nEl; ++e)
        for (int a = 0; a < nen; ++a)
            if (IEN[e + a * ld] != mg_grid_node(ndim, ne, e, a)) return 0;
    return ne;
}

namespace sfem_dev {

template <int NDIM>
__device__ __forceinline__ void mg_coords(int64_t i, int n, int c[3]) {
    const int64_t n1 = n + 1;
    c[0] = (int)(i % n1);
    c[1] = (int)((i / n1) % n1);
    c[2] = NDIM == 3 ? (int)(i / (n1 * n1)) : 0;
}

template <int NDIM>
__device__ __forceinline__ int64_t mg_index(const int c[3], int n) {
    const int64_t n1 = n + 1;
    return NDIM == 3 ? c[0] + n1 * (c[1] + n1 * (int64_t)c[2]) : c[0] + n1 * c[1];
}

// 1D interpolation weight of coarse node I at fine node i (fine level of n elements).
__device__ __forceinline__ float mg_w1(int i, int I, int n) {
    const int c = min(2 * I, n);
    if (i == c) return 1.0f;
    if ((i & 1) && i < n && (i == c - 1 || i == c + 1)) return 0.5f;
    return 0.0f;
}

// Stencil position of the neighbour offset (j - i), each component in {-1, 0, 1}.
template <int NDIM>
__device__ __forceinline__ int mg_stencil(const int ci[3], const int cj[3]) {
    const int s = (cj[1] - ci[1] + 1) * 3 + (cj[0] - ci[0] + 1);
    return NDIM == 3 ? (cj[2] - ci[2] + 1) * 9 + s : s;
}

// Position of entry e (row-major in the B x B block) of stencil block s of
// node I in a coarse level's A: nodes in tiles of 32, each tile's S * B * B
// entries in order with its 32 nodes contiguous.  A warp on 32 consecutive
// nodes reads one contiguous run of S * B * B * 128 bytes, every load at a
// fixed offset from the tile's start.  Off-grid neighbours' blocks are zero.
template <int NDIM, int B>
__device__ __forceinline__ int64_t mg_a(int64_t I, int s, int e) {
    constexpr int S = NDIM == 2 ? 9 : 27;
    return ((I >> 5) * (S * B * B) + s * B * B + e) * 32 + (I & 31);
}

// Block (slab, lane) of the fine K in FP32: the lane-contiguous FP32 copy of
// the batch and serving pipeline (one vector load), else the FP64 sliced-ELL
// values rounded.
template <int B>
__device__ __forceinline__ void mg_fine_block(const BatchArgs &a, int64_t slab, int lane, float *blk) {
    if (a.val32) {
        load_v32<B, false>(a.val32, slab, lane, blk);
    } else {
#pragma unroll
        for (int e = 0; e < B * B; ++e) blk[e] = (float)a.val64[(slab * B * B + e) * 32 + lane];
    }
}

// Free flags of the DOFs of node ci on level l.
template <int NDIM, int B>
__device__ __forceinline__ void mg_free(const BatchArgs &a, const BatchMesh &M, const MgLevel &L, int l,
                                        const int ci[3], bool f[B]) {
    const int64_t li = mg_index<NDIM>(ci, L.n);
#pragma unroll
    for (int c = 0; c < B; ++c) f[c] = l == 0 ? a.fixed[(M.node0 + li) * B + c] == 0 : L.fr[li * B + c] != 0;
}

// Block A_l(i, j) of neighbours i, j on level l.  Fine level: the
// upper-triangle FP32 copy when there is one, else the sliced-ELL K (its
// FP32 copy, or FP64 rounded); the position of j among i's ascending
// neighbours follows from the grid.  Coarse levels: the stencil.  False
// when the fine pattern is not the structured one.
template <int NDIM, int B>
__device__ __forceinline__ bool mg_block(const BatchArgs &a, const BatchMesh &M, const MgLevel &L, int l,
                                         const int ci[3], const int cj[3], float *blk) {
    const int64_t li = mg_index<NDIM>(ci, L.n);
    if (l == 0 && a.valU) {  // upper-triangle FP32 copy: block (i, j) for j >= i, else (j, i) transposed
        const int64_t gi = M.node0 + li, gj = M.node0 + mg_index<NDIM>(cj, L.n);
        const bool up = gj >= gi;
        const int *ro = up ? ci : cj, *co = up ? cj : ci;  // the owning row and the column, grid coordinates
        int pos = 0, kd = 0, mul = 1;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            const int lo = ro[d] > 0 ? 1 : 0;
            pos += (co[d] - ro[d] + lo) * mul;
            kd += lo * mul;  // the diagonal's position in the full row
            mul *= 1 + lo + (ro[d] < L.n ? 1 : 0);
        }
        const int64_t r = up ? gi : gj, c = up ? gj : gi;
        const int lane = (int)(r & 31);
        const int64_t u0 = a.sptrU[r >> 5], ku = pos - kd;
        if (ku < 0 || ku >= a.sptrU[(r >> 5) + 1] - u0) return false;
        const int64_t slab = u0 + ku;
        if (a.colU[slab * 32 + lane] != (int)c) return false;
        float t[B * B];
        load_v32<B, false>(a.valU, slab, lane, t);
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) blk[i * B + j] = up ? t[i * B + j] : t[j * B + i];
    } else if (l == 0) {
        int pos = 0, mul = 1;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            const int lo = ci[d] > 0 ? 1 : 0;
            pos += (cj[d] - ci[d] + lo) * mul;
            mul *= 1 + lo + (ci[d] < L.n ? 1 : 0);
        }
        const int64_t r = M.node0 + li;
        const int lane = (int)(r & 31);
        const int64_t slab = a.sliceptr[r >> 5] + pos;
        if (pos >= a.rowlen[r] || a.col[slab * 32 + lane] != (int)(M.node0 + mg_index<NDIM>(cj, L.n))) return false;
        mg_fine_block<B>(a, slab, lane, blk);
    } else {
        const int s = mg_stencil<NDIM>(ci, cj);
#pragma unroll
        for (int e = 0; e < B * B; ++e) blk[e] = L.A[mg_a<NDIM, B>(li, s, e)];
    }
    return true;
}

// Inverse of a B x B block with the rows and columns of fixed DOFs taken
// out (zero in the result); false if the free part is singular.
template <int B>
__device__ __forceinline__ bool mg_inv_block(const double *Din, const bool *f, double *I) {
    double D[B][B];
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
        for (int j = 0; j < B; ++j) D[i][j] = (f[i] && f[j]) ? Din[i * B + j] : (i == j ? 1.0 : 0.0);
    double det;
    double C[B][B];
    if constexpr (B == 1) {
        det = D[0][0];
        C[0][0] = 1.0;
    } else if constexpr (B == 2) {
        det = D[0][0] * D[1][1] - D[0][1] * D[1][0];
        C[0][0] = D[1][1];
        C[0][1] = -D[0][1];
        C[1][0] = -D[1][0];
        C[1][1] = D[0][0];
    } else {
        C[0][0] = D[1][1] * D[2][2] - D[1][2] * D[2][1];
        C[0][1] = D[0][2] * D[2][1] - D[0][1] * D[2][2];
        C[0][2] = D[0][1] * D[1][2] - D[0][2] * D[1][1];
        C[1][0] = D[1][2] * D[2][0] - D[1][0] * D[2][2];
        C[1][1] = D[0][0] * D[2][2] - D[0][2] * D[2][0];
        C[1][2] = D[0][2] * D[1][0] - D[0][0] * D[1][2];
        C[2][0] = D[1][0] * D[2][1] - D[1][1] * D[2][0];
        C[2][1] = D[0][1] * D[2][0] - D[0][0] * D[2][1];
        C[2][2] = D[0][0] * D[1][1] - D[0][1] * D[1][0];
        det = D[0][0] * C[0][0] + D[0][1] * C[1][0] + D[0][2] * C[2][0];
    }
    if (!(det != 0.0)) return false;
    const double rd = 1.0 / det;
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
        for (int j = 0; j < B; ++j) I[i * B + j] = (f[i] && f[j]) ? C[i][j] * rd : 0.0;
    return true;
}

// ---- hierarchy set-up, pass by pass.  Each pass is a loop over (gt, gstride)
// that the group driver below (mg_setup) and the grid-wide kernels of the
// single-mesh solver share; a barrier separates consecutive passes.  Failures
// go to *flag (SFEM_SINGULAR, SFEM_BAD_INDEX) by atomicMax.

// Fine level: W D^-1 from the block-Jacobi inverse `bj` (FP32, [node][B][B])
// and the node's row of K.
template <int NDIM, int B>
__device__ __forceinline__ void mg_pass_fine(const BatchArgs &a, const BatchMesh &M, const MgLevel &F,
                                             const float *bj, int64_t gt, int64_t gstride) {
    for (int64_t li = gt; li < F.nnode; li += gstride) {
        const int64_t r = M.node0 + li;
        float Di[B * B];
#pragma unroll
        for (int e = 0; e < B * B; ++e) Di[e] = bj[r * B * B + e];
        float rs[B];
#pragma unroll
        for (int i = 0; i < B; ++i) rs[i] = 0.0f;
        const int len = a.rowlen[r];
        const int64_t slab0 = a.sliceptr[r >> 5];
        const int lane = (int)(r & 31);
        for (int k = 0; k < len; ++k) {
            const int64_t slab = slab0 + k;
            const int c = a.col[slab * 32 + lane];
            float blk[B * B];
            mg_fine_block<B>(a, slab, lane, blk);
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) {
                    if (a.fixed[(int64_t)c * B + j]) continue;
                    float v = 0.0f;
#pragma unroll
                    for (int m = 0; m < B; ++m) v = fmaf(Di[i * B + m], blk[m * B + j], v);
                    rs[i] += fabsf(v);
                }
        }
        float rho = 0.0f;
#pragma unroll
        for (int i = 0; i < B; ++i) rho = fmaxf(rho, rs[i]);
        const float w = rho > 0.0f ? (4.0f / 3.0f) / rho : 0.0f;
#pragma unroll
        for (int e = 0; e < B * B; ++e) F.minv[r * B * B + e] = w * Di[e];
    }
}

// Coarse free flags: the coinciding fine DOF's.
template <int NDIM, int B>
__device__ __forceinline__ void mg_pass_free(const BatchArgs &a, const BatchMesh &M, const MgLevel &F,
                                             const MgLevel &C, int l, int64_t gt, int64_t gstride) {
    for (int64_t I = gt; I < C.nnode; I += gstride) {
        int cI[3], cf[3] = {0, 0, 0};
        mg_coords<NDIM>(I, C.n, cI);
#pragma unroll
        for (int d = 0; d < NDIM; ++d) cf[d] = min(2 * cI[d], F.n);
        bool f[B];
        mg_free<NDIM, B>(a, M, F, l, cf, f);
#pragma unroll
        for (int c = 0; c < B; ++c) C.fr[I * B + c] = f[c] ? 1 : 0;
    }
}

// Block (i, j) of the fine level (l = 0) from the per-mesh sliced-ELL K with
// all its loads issued at once: the slab follows from the grid and is
// clamped into the row's slice, so every load stays in bounds; the column
// check afterwards says whether the pattern is the structured one.
template <int NDIM, int B>
__device__ __forceinline__ bool mg_block0(const BatchArgs &a, const BatchMesh &M, const MgLevel &L, const int ci[3],
                                          const int cj[3], float *blk) {
    int pos = 0, mul = 1;
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
        const int lo = ci[d] > 0 ? 1 : 0;
        pos += (cj[d] - ci[d] + lo) * mul;
        mul *= 1 + lo + (ci[d] < L.n ? 1 : 0);
    }
    const int64_t r = M.node0 + mg_index<NDIM>(ci, L.n);
    const int lane = (int)(r & 31);
    const int64_t s0 = a.sliceptr[r >> 5], s1 = a.sliceptr[(r >> 5) + 1];
    const bool inslice = s1 > s0;
    const int64_t slab = min(s0 + pos, s1 - 1);
    const int len = a.rowlen[r];
    const int c = inslice ? a.col[slab * 32 + lane] : -1;
    if (inslice) {
        mg_fine_block<B>(a, slab, lane, blk);
    } else {
#pragma unroll
        for (int e = 0; e < B * B; ++e) blk[e] = 0.0f;
    }
    return pos < len && c == (int)(M.node0 + mg_index<NDIM>(cj, L.n));
}

// The pairs kx of one (kz, ky) row of the Galerkin sum, NX of them (a fixed
// count, so that their loads are in flight together): on a stencil level
// (L0 false) from the stencil, on the fine level of the per-mesh pipeline
// (L0) from its K.
template <int NDIM, int B, int NX, bool L0>
__device__ __forceinline__ void mg_galerkin_row(const BatchArgs &a, const BatchMesh &M, const MgLevel &F,
                                                const int (&pi)[3][7], const int (&pj)[3][7],
                                                const float (&pw)[3][7], int ky, int kz, float *acc, int *flag) {
#pragma unroll
    for (int kx = 0; kx < NX; ++kx) {
        const int ci[3] = {pi[0][kx], pi[1][ky], pi[2][kz]};
        const int cj[3] = {pj[0][kx], pj[1][ky], pj[2][kz]};
        const float w = pw[0][kx] * pw[1][ky] * pw[2][kz];
        float blk[B * B];
        bool fi[B], fj[B];
        if constexpr (L0) {
            if (!mg_block0<NDIM, B>(a, M, F, ci, cj, blk)) {
                atomicMax(flag, (int)SFEM_BAD_INDEX);
                continue;
            }
            mg_free<NDIM, B>(a, M, F, 0, ci, fi);
            mg_free<NDIM, B>(a, M, F, 0, cj, fj);
        } else {
            const int64_t li = mg_index<NDIM>(ci, F.n), lj = mg_index<NDIM>(cj, F.n);
            const int st = mg_stencil<NDIM>(ci, cj);
#pragma unroll
            for (int e = 0; e < B * B; ++e) blk[e] = F.A[mg_a<NDIM, B>(li, st, e)];
#pragma unroll
            for (int c = 0; c < B; ++c) {
                fi[c] = F.fr[li * B + c] != 0;
                fj[c] = F.fr[lj * B + c] != 0;
            }
        }
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j)
                if (fi[i] && fj[j]) acc[i * B + j] = fmaf(w, blk[i * B + j], acc[i * B + j]);
    }
}

// Galerkin product: one (coarse node, stencil neighbour) block per step.
// On a stencil level (l >= 1) each direction's pair list is padded, after
// its real pairs, with zero-weight pairs (i, i) to 7 (offset 0) or 3
// (offset +-1) entries: the counts are the same for a warp's nodes, the
// innermost loop has a fixed trip count, and the zero terms leave every sum
// bitwise unchanged.
template <int NDIM, int B>
__device__ __forceinline__ void mg_pass_galerkin(const BatchArgs &a, const BatchMesh &M, const MgLevel &F,
                                                 const MgLevel &C, int l, int64_t gt, int64_t gstride, int *flag) {
    constexpr int S = NDIM == 2 ? 9 : 27;
    const int64_t total = (int64_t)C.nnode * S;
    for (int64_t q = gt; q < total; q += gstride) {
        const int64_t I = q % C.nnode;
        const int s = (int)(q / C.nnode);
        int cI[3], cJ[3] = {0, 0, 0};
        mg_coords<NDIM>(I, C.n, cI);
        const int off[3] = {s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1};
        bool valid = true;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            cJ[d] = cI[d] + off[d];
            valid = valid && cJ[d] >= 0 && cJ[d] <= C.n;
        }
        float acc[B * B];
#pragma unroll
        for (int e = 0; e < B * B; ++e) acc[e] = 0.0f;
        if (valid) {
            // per direction: fine pairs (i, j), i in supp(I), j in supp(J), |i - j| <= 1
            int pi[3][7], pj[3][7], np[3] = {1, 1, 1};
            float pw[3][7];
            pi[2][0] = pj[2][0] = 0;
            pw[2][0] = 1.0f;
#pragma unroll
            for (int d = 0; d < NDIM; ++d) {
                int k = 0;
                const int ccI = min(2 * cI[d], F.n);
                for (int i = ccI - 1; i <= ccI + 1; ++i) {
                    if (i < 0 || i > F.n) continue;
                    const float wi = mg_w1(i, cI[d], F.n);
                    if (wi == 0.0f) continue;
                    for (int j = i - 1; j <= i + 1; ++j) {
                        if (j < 0 || j > F.n) continue;
                        const float wj = mg_w1(j, cJ[d], F.n);
                        if (wj == 0.0f) continue;
                        pi[d][k] = i;
                        pj[d][k] = j;
                        pw[d][k] = wi * wj;
                        ++k;
                    }
                }
                if (l >= 1 || !a.valU) {
                    const int npad = off[d] == 0 ? 7 : 3;
                    for (; k < npad; ++k) {
                        pi[d][k] = pj[d][k] = ccI;
                        pw[d][k] = 0.0f;
                    }
                }
                np[d] = k;
            }
            if (l >= 1) {
                for (int kz = 0; kz < np[2]; ++kz)
                    for (int ky = 0; ky < np[1]; ++ky) {
                        if (np[0] == 7) mg_galerkin_row<NDIM, B, 7, false>(a, M, F, pi, pj, pw, ky, kz, acc, flag);
                        else mg_galerkin_row<NDIM, B, 3, false>(a, M, F, pi, pj, pw, ky, kz, acc, flag);
                    }
            } else if (!a.valU) {
                for (int kz = 0; kz < np[2]; ++kz)
                    for (int ky = 0; ky < np[1]; ++ky) {
                        if (np[0] == 7) mg_galerkin_row<NDIM, B, 7, true>(a, M, F, pi, pj, pw, ky, kz, acc, flag);
                        else mg_galerkin_row<NDIM, B, 3, true>(a, M, F, pi, pj, pw, ky, kz, acc, flag);
                    }
            } else {
                for (int kz = 0; kz < np[2]; ++kz)
                    for (int ky = 0; ky < np[1]; ++ky)
                        for (int kx = 0; kx < np[0]; ++kx) {
                            const int ci[3] = {pi[0][kx], pi[1][ky], pi[2][kz]};
                            const int cj[3] = {pj[0][kx], pj[1][ky], pj[2][kz]};
                            const float w = pw[0][kx] * pw[1][ky] * pw[2][kz];
                            float blk[B * B];
                            if (!mg_block<NDIM, B>(a, M, F, l, ci, cj, blk)) {
                                atomicMax(flag, (int)SFEM_BAD_INDEX);
                                continue;
                            }
                            bool fi[B], fj[B];
                            mg_free<NDIM, B>(a, M, F, l, ci, fi);
                            mg_free<NDIM, B>(a, M, F, l, cj, fj);
#pragma unroll
                            for (int i = 0; i < B; ++i)
#pragma unroll
                                for (int j = 0; j < B; ++j)
                                    if (fi[i] && fj[j]) acc[i * B + j] = fmaf(w, blk[i * B + j], acc[i * B + j]);
                        }
            }
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j)
                    if (!C.fr[I * B + i] || !C.fr[mg_index<NDIM>(cJ, C.n) * B + j]) acc[i * B + j] = 0.0f;
        }
#pragma unroll
        for (int e = 0; e < B * B; ++e) C.A[mg_a<NDIM, B>(I, s, e)] = acc[e];
    }
}

// Smoother of a coarse level: W D^-1 from its stencil's centre block and rows.
template <int NDIM, int B>
__device__ __forceinline__ void mg_pass_smoother(const MgLevel &C, int64_t gt, int64_t gstride, int *flag) {
    constexpr int S = NDIM == 2 ? 9 : 27;
    for (int64_t I = gt; I < C.nnode; I += gstride) {
        double D[B * B], Di[B * B];
        bool f[B];
#pragma unroll
        for (int c = 0; c < B; ++c) f[c] = C.fr[I * B + c] != 0;
#pragma unroll
        for (int e = 0; e < B * B; ++e) D[e] = C.A[mg_a<NDIM, B>(I, S / 2, e)];
        if (!mg_inv_block<B>(D, f, Di)) {
            atomicMax(flag, (int)SFEM_SINGULAR);
#pragma unroll
            for (int e = 0; e < B * B; ++e) Di[e] = 0.0;
        }
        float rs[B];
#pragma unroll
        for (int i = 0; i < B; ++i) rs[i] = 0.0f;
        for (int s = 0; s < S; ++s) {
            float blk[B * B];
#pragma unroll
            for (int e = 0; e < B * B; ++e) blk[e] = C.A[mg_a<NDIM, B>(I, s, e)];
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) {
                    float v = 0.0f;
#pragma unroll
                    for (int m = 0; m < B; ++m) v = fmaf((float)Di[i * B + m], blk[m * B + j], v);
                    rs[i] += fabsf(v);
                }
        }
        float rho = 0.0f;
#pragma unroll
        for (int i = 0; i < B; ++i) rho = fmaxf(rho, rs[i]);
        const float w = rho > 0.0f ? (4.0f / 3.0f) / rho : 0.0f;
#pragma unroll
        for (int e = 0; e < B * B; ++e) C.minv[I * B * B + e] = w * (float)Di[e];
    }
}

// Coarsest level: dense inverse by Gauss-Jordan in FP64 (SPD, no pivoting),
// by the threads of ONE CTA (CTA barriers only).
template <int NDIM, int B>
__device__ __forceinline__ void mg_pass_coarsest(const MgLevel &C, int n, float *cinv, double *g, int *flag) {
    const int w2 = 2 * n;
    for (int q = threadIdx.x; q < n * w2; q += blockDim.x) {
        const int r = q / w2, c = q % w2;
        double v = 0.0;
        if (c >= n) {
            v = (c - n == r) ? 1.0 : 0.0;
        } else {
            const int I = r / B, i = r % B, J = c / B, j = c % B;
            if (!C.fr[I * B + i] || !C.fr[J * B + j]) {
                v = (r == c) ? 1.0 : 0.0;
            } else {
                int cI[3], cJ[3];
                mg_coords<NDIM>(I, C.n, cI);
                mg_coords<NDIM>(J, C.n, cJ);
                bool nb = true;
#pragma unroll
                for (int d = 0; d < NDIM; ++d) nb = nb && abs(cI[d] - cJ[d]) <= 1;
                if (nb) v = C.A[mg_a<NDIM, B>(I, mg_stencil<NDIM>(cI, cJ), i * B + j)];
            }
        }
        g[q] = v;
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        const double piv = g[k * w2 + k];
        __syncthreads();  // every thread has the pivot before row k changes
        if (!(piv > 0.0)) {
            if (threadIdx.x == 0) atomicMax(flag, (int)SFEM_SINGULAR);
            break;
        }
        for (int c = threadIdx.x; c < w2; c += blockDim.x) g[k * w2 + c] /= piv;
        __syncthreads();
        for (int q = threadIdx.x; q < n * w2; q += blockDim.x) {
            const int r = q / w2, c = q % w2;
            if (r == k || c == k) continue;  // column k is not read again
            g[q] -= g[r * w2 + k] * g[k * w2 + c];
        }
        __syncthreads();
    }
    for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
        const int r = q / n, c = q % n;
        const bool fr = C.fr[(r / B) * B + r % B] && C.fr[(c / B) * B + c % B];
        cinv[q] = fr ? (float)g[r * w2 + n + c] : 0.0f;
    }
}

// x = C^-1 b on the coarsest level.
__device__ __forceinline__ void mg_coarse_solve(const MgLevel &C, int n, const float *cinv, int64_t gt,
                                                int64_t gstride) {
    for (int64_t q = gt; q < n; q += gstride) {
        float v = 0.0f;
#pragma unroll 27
        for (int c = 0; c < n; ++c) v = fmaf(cinv[q * n + c], C.b[c], v);
        C.x[q] = v;
    }
}

// Hierarchy set-up by one group, after K (FP64), the Dirichlet mask and the
// block-Jacobi inverse `bj` (FP32, [node][B][B]) are in place.
template <class Grp, int NDIM, int B>
__device__ __noinline__ void mg_setup(const Grp &G, const BatchArgs &a, const BatchMesh &M, const MgMesh *mgp,
                                      const float *bj, int *flag) {
    const int64_t gt = (int64_t)G.rank() * blockDim.x + threadIdx.x, gstride = (int64_t)G.size() * blockDim.x;
    const int L = mgp->nlev;
    mg_pass_fine<NDIM, B>(a, M, mgp->lev[0], bj, gt, gstride);
    for (int l = 0; l + 1 < L; ++l) {
        const MgLevel F = mgp->lev[l], C = mgp->lev[l + 1];
        mg_pass_free<NDIM, B>(a, M, F, C, l, gt, gstride);
        G.sync();
        mg_pass_galerkin<NDIM, B>(a, M, F, C, l, gt, gstride, flag);
        G.sync();
        if (l + 2 < L) mg_pass_smoother<NDIM, B>(C, gt, gstride, flag);  // the coarsest is solved exactly
    }
    if (G.rank() == 0) mg_pass_coarsest<NDIM, B>(mgp->lev[L - 1], mgp->ndc, mgp->cinv, mgp->gj, flag);
    G.sync();
}

// Restriction of level l's residual t_l into b_{l+1}; with `smooth`, also
// the pre-smoothing sweep from zero x_{l+1} = W D^-1 b_{l+1}.
// Every coarse node takes the same 3 (x 3 x 3) fine candidates, ascending,
// the ones off the grid or outside its support with weight zero at a clamped
// index: fixed trip counts let all loads of a node be in flight at once, and
// the zero terms leave the sum unchanged.
template <int NDIM, int B>
__device__ __forceinline__ void mg_restrict(const BatchMesh &M, const MgLevel &F, const MgLevel &C, int l, bool smooth,
                                            int64_t gt, int64_t gstride) {
    constexpr int KZ = NDIM == 3 ? 3 : 1;
    for (int64_t I = gt; I < C.nnode; I += gstride) {
        int cI[3];
        mg_coords<NDIM>(I, C.n, cI);
        int fi[3][3];
        float fw[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int cc = d < NDIM ? min(2 * cI[d], F.n) : 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int i = cc - 1 + k;
                const bool in = d < NDIM ? (i >= 0 && i <= F.n) : k == 1;
                fi[d][k] = min(max(i, 0), d < NDIM ? F.n : 0);
                fw[d][k] = !in ? 0.0f : (d < NDIM ? mg_w1(i, cI[d], F.n) : 1.0f);
            }
        }
        float acc[B];
#pragma unroll
        for (int c = 0; c < B; ++c) acc[c] = 0.0f;
        const int64_t off = l == 0 ? M.node0 : 0;
#pragma unroll
        for (int kz = 0; kz < KZ; ++kz)
#pragma unroll
            for (int ky = 0; ky < 3; ++ky)
#pragma unroll
                for (int kx = 0; kx < 3; ++kx) {
                    const int zk = NDIM == 3 ? kz : 1;
                    const int ci[3] = {fi[0][kx], fi[1][ky], fi[2][zk]};
                    const float w = fw[0][kx] * fw[1][ky] * fw[2][zk];
                    const int64_t li = mg_index<NDIM>(ci, F.n) + off;
#pragma unroll
                    for (int c = 0; c < B; ++c) acc[c] = fmaf(w, F.t[li * B + c], acc[c]);  // t = 0 on fixed DOFs
                }
#pragma unroll
        for (int c = 0; c < B; ++c) {
            acc[c] = C.fr[I * B + c] ? acc[c] : 0.0f;
            C.b[I * B + c] = acc[c];
        }
        if (smooth) {
#pragma unroll
            for (int i = 0; i < B; ++i) {
                float v = 0.0f;
#pragma unroll
                for (int j = 0; j < B; ++j) v = fmaf(C.minv[(I * B + i) * B + j], acc[j], v);
                C.x[I * B + i] = v;
            }
        }
    }
}

// x_l += P' xc (xc: level l+1's iterate, zero on its fixed DOFs).  Two coarse
// candidates per direction (the second with weight zero where the fine node
// sits on a coarse one), for the same reason as in mg_restrict.
template <int NDIM, int B>
__device__ __forceinline__ void mg_prolong(const BatchArgs &a, const BatchMesh &M, const MgLevel &F, const MgLevel &C,
                                           int l, const float *xc, int64_t gt, int64_t gstride) {
    constexpr int KZ = NDIM == 3 ? 2 : 1;
    for (int64_t li = gt; li < F.nnode; li += gstride) {
        int ci[3];
        mg_coords<NDIM>(li, F.n, ci);
        int cc[3][2];
        float cw[3][2];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int i = ci[d];
            if (d >= NDIM) {
                cc[d][0] = cc[d][1] = 0;
                cw[d][0] = 1.0f;
                cw[d][1] = 0.0f;
            } else if (i == F.n || !(i & 1)) {
                cc[d][0] = cc[d][1] = i == F.n ? C.n : i / 2;
                cw[d][0] = 1.0f;
                cw[d][1] = 0.0f;
            } else {
                cc[d][0] = (i - 1) / 2;
                cc[d][1] = (i + 1) / 2;
                cw[d][0] = cw[d][1] = 0.5f;
            }
        }
        float acc[B];
#pragma unroll
        for (int c = 0; c < B; ++c) acc[c] = 0.0f;
#pragma unroll
        for (int kz = 0; kz < KZ; ++kz)
#pragma unroll
            for (int ky = 0; ky < 2; ++ky)
#pragma unroll
                for (int kx = 0; kx < 2; ++kx) {
                    const int cI[3] = {cc[0][kx], cc[1][ky], cc[2][kz]};
                    const float w = cw[0][kx] * cw[1][ky] * cw[2][kz];
                    const int64_t I = mg_index<NDIM>(cI, C.n);
#pragma unroll
                    for (int c = 0; c < B; ++c) acc[c] = fmaf(w, xc[I * B + c], acc[c]);
                }
        bool f[B];
        mg_free<NDIM, B>(a, M, F, l, ci, f);
        const int64_t d0 = (l == 0 ? M.node0 + li : li) * B;
#pragma unroll
        for (int c = 0; c < B; ++c)
            if (f[c]) F.x[d0 + c] += acc[c];
    }
}

// One pass of the coarse-level stencil operator: RES t = b - A x, or SMOOTH
// out = x + W D^-1 (b - A x).
template <int NDIM, int B, int EPI>
__device__ __forceinline__ void mg_stencil_pass(const MgLevel &C, float *out, int64_t gt, int64_t gstride) {
    constexpr int S = NDIM == 2 ? 9 : 27;
    for (int64_t I = gt; I < C.nnode; I += gstride) {
        int cI[3];
        mg_coords<NDIM>(I, C.n, cI);
        float acc[B];
#pragma unroll
        for (int c = 0; c < B; ++c) acc[c] = 0.0f;
        const float *At = C.A + mg_a<NDIM, B>(I, 0, 0);
        // off-grid neighbours are clamped onto the grid: their blocks are
        // zero, so they add nothing and the sweep has no branch
        int lo[3], hi[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            lo[d] = d < NDIM && cI[d] > 0 ? -1 : 0;
            hi[d] = d < NDIM && cI[d] < C.n ? 1 : 0;
        }
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const int o[3] = {s % 3 - 1, (s / 3) % 3 - 1, NDIM == 3 ? s / 9 - 1 : 0};
            int cJ[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) cJ[d] = cI[d] + min(max(o[d], lo[d]), hi[d]);
            const int64_t J = mg_index<NDIM>(cJ, C.n);
            float xj[B];
#pragma unroll
            for (int c = 0; c < B; ++c) xj[c] = C.x[J * B + c];
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) acc[i] = fmaf(At[(s * B * B + i * B + j) * 32], xj[j], acc[i]);
        }
        float res[B];
#pragma unroll
        for (int c = 0; c < B; ++c) res[c] = C.fr[I * B + c] ? C.b[I * B + c] - acc[c] : 0.0f;
        if constexpr (EPI == SPMV_RES) {
#pragma unroll
            for (int c = 0; c < B; ++c) out[I * B + c] = res[c];
        } else {
#pragma unroll
            for (int i = 0; i < B; ++i) {
                float v = C.x[I * B + i];
#pragma unroll
                for (int j = 0; j < B; ++j) v = fmaf(C.minv[(I * B + i) * B + j], res[j], v);
                out[I * B + i] = v;
            }
        }
    }
}

// z = V(r): one V(1,1) cycle on the residual r (FP32, the CG's).  On entry
// the fine level's x holds the pre-smoothing sweep W D^-1 r (written by the
// caller's vector update).  Returns this thread's r.z share.
// In a cluster group, the levels from mgp->solo down (restriction into it,
// the coarse solve, and back up to its smoothing) are run by the group's
// first CTA alone with CTA barriers, while the others wait at one cluster
// barrier; each pass computes the same values whoever runs it, so the
// result does not change.
template <class Grp, int NDIM, int B, int U, int W>
__device__ __noinline__ double mg_vcycle(const Grp &G, const BatchArgs &a, const BatchMesh &M, const MgMesh *mgp,
                                         const float *r, float *z) {
    const int tid = threadIdx.x, nw = blockDim.x >> 5;
    const int64_t gt = (int64_t)G.rank() * blockDim.x + tid, gstride = (int64_t)G.size() * blockDim.x;
    const int64_t gw = (int64_t)G.rank() * nw + (tid >> 5), gnw = (int64_t)G.size() * nw;
    const int64_t n1 = M.node0 + M.nnode;
    const int L = mgp->nlev;
    const int S = G.size() > 1 ? min(max(mgp->solo, 1), L) : L;  // one CTA alone: nothing to hand over
    const MgLevel F0 = mgp->lev[0];
    // fine residual t0 = r - A x0
    grp_spmv<float, B, false, U, W, SPMV_RES>(a.sliceptr, a.col, a.val32, M.slice0 + gw, M.slice1, gnw, n1, F0.x,
                                              nullptr, 0.0f, nullptr, F0.t, a.fixed, true, r, nullptr);
    G.sync();
    for (int l = 1; l < S; ++l) {
        const MgLevel F = mgp->lev[l - 1], C = mgp->lev[l];
        mg_restrict<NDIM, B>(M, F, C, l - 1, l + 1 < L, gt, gstride);
        G.sync();
        if (l + 1 < L) {
            mg_stencil_pass<NDIM, B, SPMV_RES>(C, C.t, gt, gstride);
            G.sync();
        }
    }
    const float *xin = mgp->lev[L - 1].x;
    if (S < L) {
        if (G.rank() == 0) {
            const int64_t st = tid, ss = blockDim.x;
            for (int l = S; l < L; ++l) {
                const MgLevel F = mgp->lev[l - 1], C = mgp->lev[l];
                mg_restrict<NDIM, B>(M, F, C, l - 1, l + 1 < L, st, ss);
                __syncthreads();
                if (l + 1 < L) {
                    mg_stencil_pass<NDIM, B, SPMV_RES>(C, C.t, st, ss);
                    __syncthreads();
                }
            }
            mg_coarse_solve(mgp->lev[L - 1], mgp->ndc, mgp->cinv, st, ss);
            __syncthreads();
            for (int l = L - 2; l >= S; --l) {
                const MgLevel F = mgp->lev[l], C = mgp->lev[l + 1];
                mg_prolong<NDIM, B>(a, M, F, C, l, xin, st, ss);
                __syncthreads();
                mg_stencil_pass<NDIM, B, SPMV_SMOOTH>(F, F.t, st, ss);
                __syncthreads();
                xin = F.t;
            }
        }
        G.sync();
        xin = L - 2 >= S ? mgp->lev[S].t : mgp->lev[L - 1].x;
    } else {
        mg_coarse_solve(mgp->lev[L - 1], mgp->ndc, mgp->cinv, gt, gstride);  // coarsest: x = C^-1 b
        G.sync();
    }
    for (int l = min(L - 2, S - 1); l >= 1; --l) {
        const MgLevel F = mgp->lev[l], C = mgp->lev[l + 1];
        mg_prolong<NDIM, B>(a, M, F, C, l, xin, gt, gstride);
        G.sync();
        mg_stencil_pass<NDIM, B, SPMV_SMOOTH>(F, F.t, gt, gstride);
        G.sync();
        xin = F.t;
    }
    mg_prolong<NDIM, B>(a, M, F0, mgp->lev[1], 0, xin, gt, gstride);
    G.sync();
    return grp_spmv<float, B, false, U, W, SPMV_SMOOTH>(a.sliceptr, a.col, a.val32, M.slice0 + gw, M.slice1, gnw, n1,
                                                        F0.x, nullptr, 0.0f, nullptr, z, a.fixed, true, r, F0.minv);
}

}  // namespace sfem_dev
