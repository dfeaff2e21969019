// Surface penalty of the reference's squeeze-flow driver, added to K in place:
//   K <- K + beta * b,   b = sum over surface quads f and their 2x2 Gauss
//   points g of w_g |dx/dxi x dx/deta| (N_a N_b) I_3 on the node pair (a, b)
// (examples/vector3D.jl:175-264 builds b, :306-308 forms K_bar = K + beta*b).
//
// Every node pair of a surface quad is also a pair of the hexahedron under
// it, so b adds only to blocks K already stores (its 3x3 diagonals; b's
// off-diagonal DOF pairs are explicit zeros).  Order of operations follows
// the reference so that b's entries round the same way:
//   * per face and pair: V = sum over Gauss points, in order, of w * (N_a N_b),
//     each product and sum rounded separately (no fused multiply-add);
//   * per matrix slot: faces folded in the reference's COO order -- the face
//     list is [bottom faces; top faces] and each node's incident faces are
//     taken in ascending order;
//   * finally K_ij + (beta * b_ij).
// Three kernels: face weights (thread per face), node -> face incidence
// (count, scan, fill, sort), and the row update (thread per node; a row is
// only ever written by its own thread, so no atomics touch K).
#include <math.h>

#include "sfem_internal.cuh"

namespace {

constexpr int FACE_NEN = 4;     // bilinear quads
constexpr int MAX_ROW = 64;     // node-block row length the row kernel can hold

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

struct FaceTable {
    double N[4][4];      // [gp][a]
    double dN[4][4][2];  // [gp][a][xi/eta]
    double w[4];
};

// Face weights fw[f][a][b] = sum_g w_g |J_g| N_a(g) N_b(g).
__global__ void k_face_weights(const __grid_constant__ FaceTable t, const double *__restrict__ X, int64_t nN,
                               const int *__restrict__ fn, int64_t nF, double *__restrict__ fw,
                               DevErr *err) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nF) return;
    double c[FACE_NEN][3];
    for (int a = 0; a < FACE_NEN; ++a) {
        const int n = fn[f * FACE_NEN + a];
        for (int k = 0; k < 3; ++k) c[a][k] = X[(int64_t)n * 3 + k];
    }
    double acc[FACE_NEN][FACE_NEN];
    for (int a = 0; a < FACE_NEN; ++a)
        for (int b = 0; b < FACE_NEN; ++b) acc[a][b] = 0.0;
    for (int g = 0; g < 4; ++g) {
        double J[3][2];  // dx/dxi, dx/deta = coords * dN
        for (int k = 0; k < 3; ++k)
            for (int d = 0; d < 2; ++d) {
                double s = 0.0;
                for (int a = 0; a < FACE_NEN; ++a) s = add(s, mul(c[a][k], t.dN[g][a][d]));
                J[k][d] = s;
            }
        const double cx = add(mul(J[1][0], J[2][1]), -mul(J[2][0], J[1][1]));
        const double cy = add(mul(J[2][0], J[0][1]), -mul(J[0][0], J[2][1]));
        const double cz = add(mul(J[0][0], J[1][1]), -mul(J[1][0], J[0][1]));
        const double area = sqrt(add(add(mul(cx, cx), mul(cy, cy)), mul(cz, cz)));
        const double w = mul(t.w[g], area);
        for (int a = 0; a < FACE_NEN; ++a)
            for (int b = 0; b < FACE_NEN; ++b) acc[a][b] = add(acc[a][b], mul(w, mul(t.N[g][a], t.N[g][b])));
    }
    for (int a = 0; a < FACE_NEN; ++a)
        for (int b = 0; b < FACE_NEN; ++b) fw[(f * FACE_NEN + a) * FACE_NEN + b] = acc[a][b];
    (void)nN;
    (void)err;
}

__global__ void k_face_nodes(const int64_t *__restrict__ ien, int64_t nF, int64_t nN, int *__restrict__ fn,
                             DevErr *err) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nF * FACE_NEN) return;
    const int64_t f = t % nF, a = t / nF;  // column-major input: face index fastest
    const int64_t v = ien[t];
    if (v < 1 || v > nN) {
        sfem_dev_error(err, SFEM_BAD_INDEX, t);
        fn[f * FACE_NEN + a] = 0;
        return;
    }
    fn[f * FACE_NEN + a] = (int)(v - 1);
}

__global__ void k_n2f_count(const int *__restrict__ fn, int64_t nF, int *__restrict__ cnt) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nF * FACE_NEN) atomicAdd(&cnt[fn[t]], 1);
}

__global__ void k_n2f_fill(const int *__restrict__ fn, int64_t nF, unsigned long long *__restrict__ cursor,
                           int *__restrict__ n2f) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nF * FACE_NEN) return;
    const unsigned long long p = atomicAdd(&cursor[fn[t]], 1ull);
    n2f[p] = (int)(t / FACE_NEN);
}

__global__ void k_n2f_sort(const int64_t *__restrict__ ptr, int *__restrict__ n2f, int64_t nN) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nN) return;
    const int64_t s = ptr[r], e = ptr[r + 1];
    for (int64_t i = s + 1; i < e; ++i) {
        const int v = n2f[i];
        int64_t j = i - 1;
        while (j >= s && n2f[j] > v) {
            n2f[j + 1] = n2f[j];
            --j;
        }
        n2f[j + 1] = v;
    }
}

// Row a of K: fold its faces' weights per slot, then add beta * b to the
// diagonal of each touched 3x3 block.
template <int B>
__global__ void k_penalty_rows(const int64_t *__restrict__ n2f_ptr, const int *__restrict__ n2f,
                               const int *__restrict__ fn, const double *__restrict__ fw, int64_t nN,
                               const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                               const int *__restrict__ rowlen, double *__restrict__ val, double beta, DevErr *err) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nN) return;
    const int64_t s = n2f_ptr[a], e = n2f_ptr[a + 1];
    if (s == e) return;
    const int len = rowlen[a];
    if (len > MAX_ROW) {
        sfem_dev_error(err, SFEM_UNSUPPORTED, a);
        return;
    }
    const int64_t slab0 = sliceptr[a >> 5];
    const int ln = (int)(a & 31);
    double acc[MAX_ROW];
    bool hit[MAX_ROW];
    for (int k = 0; k < len; ++k) {
        acc[k] = 0.0;
        hit[k] = false;
    }
    for (int64_t q = s; q < e; ++q) {
        const int f = n2f[q];
        int al = 0;
        while (al < FACE_NEN && fn[f * FACE_NEN + al] != (int)a) ++al;
        for (int bl = 0; bl < FACE_NEN; ++bl) {
            const int nb = fn[f * FACE_NEN + bl];
            int k = 0;
            while (k < len && col[(slab0 + k) * 32 + ln] != nb) ++k;
            if (k == len) {  // the face couples nodes that share no element of K
                sfem_dev_error(err, SFEM_BAD_INDEX, a);
                return;
            }
            acc[k] = add(acc[k], fw[((int64_t)f * FACE_NEN + al) * FACE_NEN + bl]);
            hit[k] = true;
        }
    }
    for (int k = 0; k < len; ++k) {
        if (!hit[k]) continue;
        const double pb = mul(beta, acc[k]);
        for (int i = 0; i < B; ++i) {
            double &v = val[((slab0 + k) * B * B + i * B + i) * 32 + ln];
            v = add(v, pb);
        }
    }
}

__global__ void k_penalty_fp32(int64_t n, const double *__restrict__ v, float *__restrict__ v32) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v32[i] = (float)v[i];
}

unsigned blocks_for(int64_t n, int t) { return (unsigned)sfem_cdiv(n > 0 ? n : 1, t); }

FaceTable make_face_table() {
    FaceTable t;
    double xi[2], w[2];
    sfem_gaussian_quadrature(-1, 1, 2, xi, w);
    // Gauss point order of examples/vector3D.jl:203-207: (xi1,eta1), (xi2,eta1), (xi2,eta2), (xi1,eta2)
    const int ox[4] = {0, 1, 1, 0}, oy[4] = {0, 0, 1, 1};
    for (int g = 0; g < 4; ++g) {
        t.w[g] = w[ox[g]] * w[oy[g]];
        double N[4], dN[8];
        sfem_basis_function(2, SFEM_Q1, xi[ox[g]], xi[oy[g]], 0.0, N, dN);
        for (int a = 0; a < 4; ++a) {
            t.N[g][a] = N[a];
            t.dN[g][a][0] = dN[a];
            t.dN[g][a][1] = dN[4 + a];
        }
    }
    return t;
}

}  // namespace

extern "C" int sfem_penalty_add(sfem_ctx *ctx, sfem_matrix *K, const double *NodeList, const int64_t *IEN_faces,
                                int64_t nFaces, int nenFace, double beta, int mem_space) {
    if (!ctx || !K || !K->mesh || !NodeList || (nFaces > 0 && !IEN_faces) || nFaces < 0) return SFEM_BAD_ARG;
    sfem_mesh *m = K->mesh;
    if (m->ctx != ctx) return sfem_set_error(ctx, SFEM_BAD_ARG, "matrix belongs to another context");
    if (m->ndim != 3 || m->fclass != SFEM_Q1 || m->b != 3)
        return sfem_set_error(ctx, SFEM_UNSUPPORTED,
                              "surface penalty is defined for 3D Q1 elasticity only (the reference's 2D branch "
                              "takes cross() of 2-vectors)");
    if (nenFace != FACE_NEN) return sfem_set_error(ctx, SFEM_BAD_ARG, "faces must be 4-node quads");
    if (!(beta == beta)) return sfem_set_error(ctx, SFEM_BAD_ARG, "beta is NaN");
    SFEM_TRY(sfem_check_ptr(ctx, NodeList, mem_space));
    SFEM_TRY(sfem_check_ptr(ctx, IEN_faces, mem_space));
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        cudaGetLastError();
        return sfem_set_error(ctx, SFEM_CUDA_ERROR, "cudaSetDevice(%d) failed", ctx->device);
    }
    if (nFaces == 0) return SFEM_OK;
    const int64_t nN = m->nN;
    cudaStream_t s = ctx->stream;
    double *X = nullptr, *fw = nullptr;
    int64_t *ien = nullptr, *n2f_ptr = nullptr;
    int *fn = nullptr, *cnt = nullptr, *n2f = nullptr;
    unsigned long long *cursor = nullptr;
    int st = SFEM_OK;
    do {
        if ((st = sfem_dalloc(ctx, (void **)&X, sizeof(double) * 3 * nN, "penalty coordinates"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&ien, sizeof(int64_t) * FACE_NEN * nFaces, "penalty faces"))) break;
        if ((st = sfem_copy_in(ctx, X, NodeList, sizeof(double) * 3 * nN, mem_space))) break;
        if ((st = sfem_copy_in(ctx, ien, IEN_faces, sizeof(int64_t) * FACE_NEN * nFaces, mem_space))) break;
        if ((st = sfem_dalloc(ctx, (void **)&fn, sizeof(int) * FACE_NEN * nFaces, "face nodes"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&fw, sizeof(double) * FACE_NEN * FACE_NEN * nFaces, "face weights")))
            break;
        if ((st = sfem_dalloc(ctx, (void **)&cnt, sizeof(int) * nN, "face counts"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&n2f_ptr, sizeof(int64_t) * (nN + 1), "node faces ptr"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&n2f, sizeof(int) * FACE_NEN * nFaces, "node faces"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&cursor, sizeof(unsigned long long) * nN, "face cursor"))) break;
        k_face_nodes<<<blocks_for(FACE_NEN * nFaces, 256), 256, 0, s>>>(ien, nFaces, nN, fn, ctx->d_err);
        SFEM_LAUNCHED(ctx);
        if ((st = sfem_check_device(ctx, "surface connectivity"))) break;
        const FaceTable tab = make_face_table();
        k_face_weights<<<blocks_for(nFaces, 128), 128, 0, s>>>(tab, X, nN, fn, nFaces, fw, ctx->d_err);
        SFEM_LAUNCHED(ctx);
        if ((st = sfem_cuda_status(ctx, cudaMemsetAsync(cnt, 0, sizeof(int) * nN, s), "memset"))) break;
        k_n2f_count<<<blocks_for(FACE_NEN * nFaces, 256), 256, 0, s>>>(fn, nFaces, cnt);
        SFEM_LAUNCHED(ctx);
        if ((st = sfem_scan_i32(ctx, cnt, n2f_ptr, nN))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(cursor, n2f_ptr, sizeof(int64_t) * nN,
                                                        cudaMemcpyDeviceToDevice, s), "memcpy")))
            break;
        k_n2f_fill<<<blocks_for(FACE_NEN * nFaces, 256), 256, 0, s>>>(fn, nFaces, cursor, n2f);
        SFEM_LAUNCHED(ctx);
        k_n2f_sort<<<blocks_for(nN, 128), 128, 0, s>>>(n2f_ptr, n2f, nN);
        SFEM_LAUNCHED(ctx);
        k_penalty_rows<3><<<blocks_for(nN, 128), 128, 0, s>>>(n2f_ptr, n2f, fn, fw, nN, m->sliceptr, m->col,
                                                              m->rowlen, K->val, beta, ctx->d_err);
        SFEM_LAUNCHED(ctx);
        if ((st = sfem_check_device(ctx, "surface penalty"))) break;
        if (K->val32) {  // keep the FP32 copies used by the mixed solver consistent
            const int64_t nv = m->nslabs * 32 * 9;
            k_penalty_fp32<<<blocks_for(nv, 256), 256, 0, s>>>(nv, K->val, K->val32);
            SFEM_LAUNCHED(ctx);
        }
        if ((st = sfem_sym_refresh_values(ctx, K))) break;
        st = sfem_check_device(ctx, "surface penalty refresh");
    } while (0);
    void *bufs[] = {X, ien, fn, fw, cnt, n2f_ptr, n2f, cursor};
    for (void *p : bufs) sfem_dfree(ctx, p);
    return st;
}
