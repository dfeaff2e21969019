// Numeric assembly of K (src/fem.jl:179-252) in two deterministic passes.
//
// 1. k_element: one CTA per 32 elements, one warp per Gauss point.  Each
//    thread computes, for its (element, Gauss point), the Jacobian
//    J = coords * dN (src/fem.jl:192), w = w_gp |det J| (:194), inv(J) (:195)
//    and dN/dx = dN * inv(J) (:196) in FP64, into shared memory.  Then each
//    thread accumulates, for a share of the element's node pairs (a <= b),
//        S_ab = sum_gp w (dN_a/dx) (dN_b/dx)^T            (ndim x ndim)
//    (for elasticity the shared gradients are stored scaled by sqrt(w), so
//    each term is one product: 9 FMA per pair and Gauss point in 3D)
//    and turns it into the elasticity block
//        K_ab[i][j] = lambda S_ab[i][j] + mu S_ab[j][i] + mu delta_ij tr(S_ab),
//    which is B_a' D B_b for the isotropic D of src/fem.jl:217 (plane stress)
//    and :230 (3D) written with Lame constants; for nDof = 1 the block is the
//    scalar sum_gp w (dN_a/dx . dN_b/dx) of :206.  Only the upper-triangle
//    node pairs are stored (element stiffness is symmetric); diagonal pair
//    blocks are symmetrised so the assembled K is bitwise symmetric.
// 2. k_gather: one warp per 32-row slice of the node-block pattern, one lane
//    per row.  For every slot (row r, neighbour c) the lane walks r's
//    incident elements in ascending element order -- the order in which
//    sparse(E,J,V) folds duplicates (src/fem.jl:253) -- and sums the blocks of
//    the elements that also contain c.  No atomics: every value is written
//    once by one lane, so the result is bitwise reproducible.
#include <math.h>
#include <string.h>

#include "sfem_internal.cuh"

namespace {

struct ElemTable {
    double dN[8][9][3];   // reference gradients at the Gauss points [gp][a][k]
    double w[8];          // Gauss weights, src/fem.jl:161,172
    unsigned char pa[48], pb[48];  // node pair p -> (a, b), a <= b
};

template <int NDIM, int NEN, int NGP, int B>
__global__ void __launch_bounds__(32 * NGP)
k_element(const __grid_constant__ ElemTable tab, const double *__restrict__ X, const int *__restrict__ ien,
          int64_t nEl, const double *__restrict__ Ev, int64_t nE, const double *__restrict__ nuv, int64_t nNu,
          int plane, double *__restrict__ kbuf, DevErr *err) {
    constexpr int GS = NEN * NDIM + 1;  // padded per-(gp, element) stride in doubles
    constexpr int NPAIR = NEN * (NEN + 1) / 2;
    extern __shared__ double sm[];
    double *sG = sm;                    // [NGP][32][GS]
    double *sW = sm + NGP * 32 * GS;    // [NGP][32]
    const int lane = threadIdx.x & 31, gp = threadIdx.x >> 5;
    const int64_t e = (int64_t)blockIdx.x * 32 + lane;

    if (e < nEl) {
        double xe[NEN][NDIM];
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            const int node = ien[(int64_t)a * nEl + e];
#pragma unroll
            for (int i = 0; i < NDIM; ++i) xe[a][i] = X[(int64_t)node * NDIM + i];
        }
        double J[NDIM][NDIM];
#pragma unroll
        for (int i = 0; i < NDIM; ++i)
#pragma unroll
            for (int k = 0; k < NDIM; ++k) {
                double s = 0.0;
#pragma unroll
                for (int a = 0; a < NEN; ++a) s = fma(xe[a][i], tab.dN[gp][a][k], s);
                J[i][k] = s;
            }
        double det, inv[NDIM][NDIM];
        if (NDIM == 2) {
            det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
            const double r = 1.0 / det;
            inv[0][0] = J[1][1] * r;
            inv[0][1] = -J[0][1] * r;
            inv[1][0] = -J[1][0] * r;
            inv[1][1] = J[0][0] * r;
        } else {
            const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
            const double r = 1.0 / det;
            inv[0][0] = c00 * r;
            inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
            inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
            inv[1][0] = c01 * r;
            inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
            inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
            inv[2][0] = c02 * r;
            inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
            inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
        }
        if (det == 0.0) sfem_dev_error(err, SFEM_SINGULAR_JACOBIAN, e);
        if (det < 0.0) atomicAdd(&err->neg_det, 1ull);
        double *g = sG + ((int64_t)gp * 32 + lane) * GS;
        // elasticity stores sqrt(w |det J|) dN/dx, so that each Gauss point's
        // term of a pair's block is a plain product (no weight per pair)
        const double sc = B > 1 ? sqrt(tab.w[gp] * fabs(det)) : 1.0;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int k = 0; k < NDIM; ++k) {
                double s = 0.0;
#pragma unroll
                for (int j = 0; j < NDIM; ++j) s = fma(tab.dN[gp][a][j], inv[j][k], s);
                g[a * NDIM + k] = B > 1 ? s * sc : s;
            }
        sW[gp * 32 + lane] = tab.w[gp] * fabs(det);
    }
    __syncthreads();
    if (e >= nEl) return;

    double lam = 0.0, mu = 0.0;
    if (B > 1) {
        const double E = Ev[nE > 1 ? e : 0], nu = nuv[nNu > 1 ? e : 0];
        if (NDIM == 2 && plane == SFEM_PLANE_STRESS) {
            lam = nu * E / (1 - nu * nu);
            mu = E / (2 * (1 + nu));
        } else {
            const double c = E / ((1 + nu) * (1 - 2 * nu));
            lam = nu * c;
            mu = (1 - 2 * nu) / 2 * c;
        }
    }
    for (int p = gp; p < NPAIR; p += NGP) {
        const int a = tab.pa[p], bq = tab.pb[p];
        if (B == 1) {
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < NGP; ++q) {
                const double *g = sG + ((int64_t)q * 32 + lane) * GS;
                double d = 0.0;
#pragma unroll
                for (int k = 0; k < NDIM; ++k) d = fma(g[a * NDIM + k], g[bq * NDIM + k], d);
                s = fma(sW[q * 32 + lane], d, s);
            }
            kbuf[(int64_t)p * nEl + e] = s;
        } else {
            double S[NDIM][NDIM];
#pragma unroll
            for (int i = 0; i < NDIM; ++i)
#pragma unroll
                for (int j = 0; j < NDIM; ++j) S[i][j] = 0.0;
            if (a == bq) {  // symmetric: the upper triangle only (the pair is warp-uniform)
#pragma unroll
                for (int q = 0; q < NGP; ++q) {
                    const double *g = sG + ((int64_t)q * 32 + lane) * GS;
#pragma unroll
                    for (int i = 0; i < NDIM; ++i) {
                        const double wa = g[a * NDIM + i];
#pragma unroll
                        for (int j = i; j < NDIM; ++j) S[i][j] = fma(wa, g[a * NDIM + j], S[i][j]);
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < NGP; ++q) {
                    const double *g = sG + ((int64_t)q * 32 + lane) * GS;
#pragma unroll
                    for (int i = 0; i < NDIM; ++i) {
                        const double wa = g[a * NDIM + i];
#pragma unroll
                        for (int j = 0; j < NDIM; ++j) S[i][j] = fma(wa, g[bq * NDIM + j], S[i][j]);
                    }
                }
            }
            if (a == bq) {
#pragma unroll
                for (int i = 0; i < NDIM; ++i)
#pragma unroll
                    for (int j = 0; j < i; ++j) S[i][j] = S[j][i];
            }
            double tr = 0.0;
#pragma unroll
            for (int i = 0; i < NDIM; ++i) tr += S[i][i];
#pragma unroll
            for (int i = 0; i < NDIM; ++i)
#pragma unroll
                for (int j = 0; j < NDIM; ++j) {
                    double v = lam * S[i][j] + mu * S[j][i];
                    if (i == j) v += mu * tr;
                    kbuf[((int64_t)p * B * B + i * B + j) * nEl + e] = v;
                }
        }
    }
}

template <int NEN, int B>
__global__ void __launch_bounds__(256, 2)
k_gather(const int64_t *__restrict__ sliceptr, const int *__restrict__ col, const int *__restrict__ rowlen,
         const int64_t *__restrict__ n2e_ptr, const int *__restrict__ n2e, const int *__restrict__ ien,
         int64_t nEl, int64_t nN, int64_t nslices, const double *__restrict__ kbuf, double *__restrict__ val,
         float *__restrict__ val32) {
    const int lane = threadIdx.x & 31;
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (s >= nslices) return;
    const int64_t r64 = s * 32 + lane;
    const int r = (int)r64;
    const bool live = r64 < nN;
    const int64_t slab0 = sliceptr[s], width = sliceptr[s + 1] - slab0;
    const int len = live ? rowlen[r] : 0;
    const int64_t q0 = live ? n2e_ptr[r] : 0, q1 = live ? n2e_ptr[r + 1] : 0;
    GatherRow<NEN> R;
    R.load(n2e, q0, q1, ien, nEl, r);
    // the next slot's column is loaded while this slot's blocks are
    int cnext = width > 0 ? col[slab0 * 32 + lane] : 0;
    for (int64_t k = 0; k < width; ++k) {
        const int64_t slab = slab0 + k;
        const int ccur = cnext;
        if (k + 1 < width) cnext = col[(slab + 1) * 32 + lane];
        double acc[B * B];
#pragma unroll
        for (int i = 0; i < B * B; ++i) acc[i] = 0.0;
        if (k < len && R.fast) {
            R.template add<B>(ccur, kbuf, nEl, acc);
        } else if (k < len) {
            const int c = ccur;
            int prev = -1;
            for (int64_t q = q0; q < q1; ++q) {
                const int e = n2e[q];
                if (e == prev) continue;  // element listed twice (node repeated in it)
                prev = e;
                int nodes[NEN];
#pragma unroll
                for (int a = 0; a < NEN; ++a) nodes[a] = __ldg(&ien[(int64_t)a * nEl + e]);
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    if (nodes[a] != r) continue;
#pragma unroll
                    for (int bq = 0; bq < NEN; ++bq) {
                        if (nodes[bq] != c) continue;
                        if (a <= bq) {
                            const int64_t base = (int64_t)sfem_pair(a, bq, NEN) * B * B;
#pragma unroll
                            for (int i = 0; i < B * B; ++i) acc[i] += __ldg(&kbuf[(base + i) * nEl + e]);
                        } else {
                            const int64_t base = (int64_t)sfem_pair(bq, a, NEN) * B * B;
#pragma unroll
                            for (int i = 0; i < B; ++i)
#pragma unroll
                                for (int j = 0; j < B; ++j)
                                    acc[i * B + j] += __ldg(&kbuf[(base + j * B + i) * nEl + e]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < B * B; ++i) {
            val[(slab * B * B + i) * 32 + lane] = acc[i];
            if (val32) val32[(slab * B * B + i) * 32 + lane] = (float)acc[i];
        }
    }
}

ElemTable make_table(int ndim, int fclass) {
    ElemTable t;
    memset(&t, 0, sizeof(t));
    double xi[2], w[2];
    sfem_gaussian_quadrature(-1, 1, 2, xi, w);
    // Gauss point order of src/fem.jl:161-176
    const int ox[8] = {0, 1, 1, 0, 0, 1, 1, 0};
    const int oy[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    const int oz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    const int ngp = ndim == 2 ? 4 : 8;
    const int nen = fclass == SFEM_Q2 ? 9 : (1 << ndim);
    for (int g = 0; g < ngp; ++g) {
        double N[9], dN[27];
        if (ndim == 2) {
            t.w[g] = w[ox[g]] * w[oy[g]];
            sfem_basis_function(2, fclass, xi[ox[g]], xi[oy[g]], 0.0, N, dN);
        } else {
            t.w[g] = w[ox[g]] * w[oy[g]] * w[oz[g]];
            sfem_basis_function(3, fclass, xi[ox[g]], xi[oy[g]], xi[oz[g]], N, dN);
        }
        for (int a = 0; a < nen; ++a)
            for (int k = 0; k < ndim; ++k) t.dN[g][a][k] = dN[k * nen + a];
    }
    int p = 0;
    for (int a = 0; a < nen; ++a)
        for (int b = a; b < nen; ++b) {
            t.pa[p] = (unsigned char)a;
            t.pb[p] = (unsigned char)b;
            ++p;
        }
    return t;
}

template <int NDIM, int NEN, int NGP, int B>
int launch_element(sfem_ctx *ctx, const sfem_mesh *m, int plane, const double *E, int64_t nE, const double *nu,
                   int64_t nNu, double *kbuf) {
    constexpr int GS = NEN * NDIM + 1;
    const size_t smem = sizeof(double) * (NGP * 32 * GS + NGP * 32);
    auto kern = k_element<NDIM, NEN, NGP, B>;
    SFEM_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const ElemTable tab = make_table(NDIM, m->fclass);
    const unsigned grid = (unsigned)sfem_cdiv(m->nEl, 32);
    kern<<<grid, 32 * NGP, smem, ctx->stream>>>(tab, m->X, m->ien, m->nEl, E, nE, nu, nNu, plane, kbuf, ctx->d_err);
    SFEM_LAUNCHED(ctx);
    return sfem_cuda_status(ctx, cudaGetLastError(), "element kernel launch");
}

template <int NEN, int B>
int launch_gather(sfem_ctx *ctx, const sfem_mesh *m, const double *kbuf, double *val, float *val32) {
    const unsigned grid = (unsigned)sfem_cdiv(m->nslices * 32, 256);
    k_gather<NEN, B><<<grid ? grid : 1, 256, 0, ctx->stream>>>(m->sliceptr, m->col, m->rowlen, m->n2e_ptr, m->n2e,
                                                               m->ien, m->nEl, m->nN, m->nslices, kbuf, val, val32);
    SFEM_LAUNCHED(ctx);
    return sfem_cuda_status(ctx, cudaGetLastError(), "gather kernel launch");
}

}  // namespace

int sfem_element_stiffness(sfem_ctx *ctx, const sfem_mesh *m, int plane, const double *E, int64_t nE,
                           const double *nu, int64_t nNu, double *kbuf) {
    if (m->nEl == 0) return SFEM_OK;
    // the negative-det J count is per assembly: earlier calls on this context must not add to it
    SFEM_CUDA(ctx, cudaMemsetAsync(&ctx->d_err->neg_det, 0, sizeof(ctx->d_err->neg_det), ctx->stream));
    if (m->fclass == SFEM_Q2) return launch_element<2, 9, 4, 1>(ctx, m, plane, E, nE, nu, nNu, kbuf);
    if (m->ndim == 2)
        return m->b == 1 ? launch_element<2, 4, 4, 1>(ctx, m, plane, E, nE, nu, nNu, kbuf)
                         : launch_element<2, 4, 4, 2>(ctx, m, plane, E, nE, nu, nNu, kbuf);
    return m->b == 1 ? launch_element<3, 8, 8, 1>(ctx, m, plane, E, nE, nu, nNu, kbuf)
                     : launch_element<3, 8, 8, 3>(ctx, m, plane, E, nE, nu, nNu, kbuf);
}

int sfem_gather_blocks(sfem_ctx *ctx, const sfem_mesh *m, const double *kbuf, double *val, float *val32) {
    if (m->nslices == 0) return SFEM_OK;
    if (m->fclass == SFEM_Q2) return launch_gather<9, 1>(ctx, m, kbuf, val, val32);
    if (m->ndim == 2)
        return m->b == 1 ? launch_gather<4, 1>(ctx, m, kbuf, val, val32) : launch_gather<4, 2>(ctx, m, kbuf, val, val32);
    return m->b == 1 ? launch_gather<8, 1>(ctx, m, kbuf, val, val32) : launch_gather<8, 3>(ctx, m, kbuf, val, val32);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" int sfem_assemble(sfem_ctx *ctx, sfem_mesh *m, int plane, const double *Young, int64_t nYoung,
                             const double *nu, int64_t nNu, int mem_space, sfem_matrix **out) {
    SfemRange range_("sfem assemble");
    if (!ctx || !m || !out) return SFEM_BAD_ARG;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    if (plane != SFEM_PLANE_STRESS && plane != SFEM_PLANE_STRAIN)
        return sfem_set_error(ctx, SFEM_BAD_ARG, "plane must be SFEM_PLANE_STRESS or SFEM_PLANE_STRAIN");
    const bool vec = m->b > 1;
    if (vec) {
        if (!Young || !nu) return sfem_set_error(ctx, SFEM_BAD_ARG, "Young and nu are required for elasticity");
        if ((nYoung != 1 && nYoung != m->nEl) || (nNu != 1 && nNu != m->nEl))
            return sfem_set_error(ctx, SFEM_BAD_ARG, "Young/nu must have length 1 or ne^ndim");
    }
    SFEM_TRY(sfem_pattern_build(ctx, m, nullptr, nullptr));
    const int b = m->b;
    const int64_t nkbuf = (int64_t)sfem_npairs(m->nen) * b * b * m->nEl;
    double *dE = nullptr, *dnu = nullptr, *kbuf = nullptr;
    sfem_matrix *K = new sfem_matrix();
    K->mesh = m;
    K->plane = plane;
    K->n = m->n_global;
    K->nnz = m->nnzb * b * b;
    m->refcnt++;
    int st = SFEM_OK;
    do {
        if (vec) {
            if ((st = sfem_dalloc(ctx, (void **)&dE, sizeof(double) * nYoung, "Young"))) break;
            if ((st = sfem_dalloc(ctx, (void **)&dnu, sizeof(double) * nNu, "nu"))) break;
            if ((st = sfem_copy_in(ctx, dE, Young, sizeof(double) * nYoung, mem_space))) break;
            if ((st = sfem_copy_in(ctx, dnu, nu, sizeof(double) * nNu, mem_space))) break;
        }
        if ((st = sfem_dalloc(ctx, (void **)&kbuf, sizeof(double) * (nkbuf ? nkbuf : 1), "element stiffness")))
            break;
        if ((st = sfem_dalloc(ctx, (void **)&K->val, sizeof(double) * m->nslabs * 32 * b * b, "K values"))) break;
        if ((st = sfem_element_stiffness(ctx, m, plane, dE, nYoung, dnu, nNu, kbuf))) break;
        if ((st = sfem_gather_blocks(ctx, m, kbuf, K->val, nullptr))) break;
        st = sfem_check_device(ctx, "assembly");
        m->neg_det = ctx->h_err->neg_det;
    } while (0);
    sfem_dfree(ctx, dE);
    sfem_dfree(ctx, dnu);
    sfem_dfree(ctx, kbuf);
    if (st != SFEM_OK) {
        sfem_matrix_destroy(K);
        return st;
    }
    *out = K;
    return SFEM_OK;
}

extern "C" int sfem_assemble_system(sfem_ctx *ctx, int64_t ne, const double *NodeList, int64_t nNodes,
                                    const int64_t *IEN, int64_t ldIEN, int nen, int ndim, int function_class,
                                    int nDof, const int64_t *ID, const double *Young, int64_t nYoung,
                                    const double *nu, int64_t nNu, int plane, int mem_space, sfem_matrix **out,
                                    int64_t *n_out, int64_t *nnz_out) {
    if (!out) return SFEM_BAD_ARG;
    sfem_mesh *m = nullptr;
    SFEM_TRY(sfem_mesh_create(ctx, ndim, function_class, nDof, ne, NodeList, nNodes, IEN, ldIEN, nen, ID, mem_space,
                              &m));
    int st = sfem_assemble(ctx, m, plane, Young, nYoung, nu, nNu, mem_space, out);
    sfem_mesh_release(m);  // the matrix holds its own reference
    if (st != SFEM_OK) return st;
    if (n_out) *n_out = (*out)->n;
    if (nnz_out) *nnz_out = (*out)->nnz;
    return SFEM_OK;
}

extern "C" int sfem_matrix_destroy(sfem_matrix *K) {
    if (!K) return SFEM_OK;
    sfem_ctx *ctx = K->mesh ? K->mesh->ctx : nullptr;
    if (ctx) {
        cudaSetDevice(ctx->device);
        sfem_dfree(ctx, K->val);
        sfem_dfree(ctx, K->val32);
        sfem_sym_free(ctx, K);
        cudaStreamSynchronize(ctx->stream);
    }
    sfem_mesh_release(K->mesh);
    delete K;
    return SFEM_OK;
}
