// Per-mesh assemble-and-solve pipeline on the device, shared by the batch
// kernel (sfem_batch.cu) and the serving kernel (sfem_serve.cu).
//
// process_mesh<Group>() runs, for one mesh and one group of CTAs (one CTA on
// its own, or a thread-block cluster):
//   1. element stiffness of the mesh's elements (FP64),
//   2. deterministic gather into the mesh's K blocks, FP64 and FP32,
//   3. Dirichlet set-up: mask, lift q_d, right-hand side -K q_d,
//   4. nodal block-Jacobi (or Jacobi) inverse,
//   5. preconditioned CG: FP64, or FP32 recurrences refreshed from an FP64
//      residual whenever the FP32 residual drops by `reliable_delta`,
//   6. u = q_d + x in the mesh's own DOF numbering.
// All reductions are group-wide in a fixed order and no group ever waits on
// another, so a mesh's result does not depend on what else runs beside it.
#pragma once

#include <math.h>
#include <string.h>

#include <cooperative_groups.h>
#include <type_traits>

#include "sfem_internal.cuh"

namespace cgrp = cooperative_groups;

struct MgMesh;  // multigrid hierarchy of one structured mesh (sfem_mg.cuh)

struct BatchMesh {
    int64_t node0, nnode;      // combined (padded) node range start, real node count
    int64_t slice0, slice1;    // its slices
    int64_t elem0, elem1;      // its elements in the combined numbering
    int64_t dof0, ndof;        // its block of u: global DOFs [dof0, dof0 + ndof)
    int64_t fix0, fix1;        // its entries of the fixed-DOF arrays
};

namespace sfem_dev {

struct ElemTableB {
    double dN[8][9][3];
    double w[8];
    unsigned char pa[48], pb[48];
};

inline ElemTableB make_table_b(int ndim, int fclass) {
    ElemTableB t;
    memset(&t, 0, sizeof(t));
    double xi[2], w[2];
    sfem_gaussian_quadrature(-1, 1, 2, xi, w);
    const int ox[8] = {0, 1, 1, 0, 0, 1, 1, 0}, oy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, oz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
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

struct BatchArgs {
    const BatchMesh *meshes;
    const int *order;     // large meshes first (cluster work), then small ones
    int64_t nmesh, nbig;  // meshes in `order`, of which the first nbig are large
    int64_t nmesh_all;    // meshes in the batch (per-mesh material arrays)
    unsigned *queue;      // [0]: next large mesh, [1]: next small mesh
    // combined mesh
    const double *X;
    const int *ien;
    int64_t nEl;
    const int64_t *n2e_ptr;
    const int *n2e;
    const int *rowlen;
    const int64_t *sliceptr;
    const int *col;
    const int *g2i;
    const int *id;   // [b][nN] combined global DOF (0-based) of (node, comp); null for b == 1
    int64_t nN, n_global;
    // material and boundary data
    const double *E;
    int64_t nE;      // 1, nmesh or nEl (combined)
    const double *nu;
    int64_t nNu;
    int plane;
    const int64_t *fix_dofs;  // mesh-local, 1-based
    const double *fix_vals;
    // buffers
    double *kbuf, *val64;
    float *val32;
    unsigned char *fixed, *gfixed;
    double *ud, *b64, *x64, *q64;
    void *vecT;      // x, r, z, p, q, p' (type T, nd each) then minv (nN * b * b)
    int64_t nd;
    double *u_out;
    int64_t u_len;   // entries of u_out (zeroed by the serving kernel)
    const double *u_init;  // initial guess in u_out's numbering (a previous solution), or null
    const MgMesh *mg;      // per mesh: multigrid hierarchy (used when its nlev >= 2), or null
    // upper-triangle FP32 copy of K (single-mesh solver), read by the hierarchy's Galerkin pass
    const int64_t *sptrU;
    const int *colU;
    const float *valU;
    // solver
    double rtol, delta2;
    int maxit, block_jacobi;
    sfem_batch_stats *stats;
    DevErr *err;
};

// Internal index (node*B + comp) of the mesh-local DOF gl (0-based), or -1
// when no element uses it.  Scalar meshes have no ID: DOF = node.
template <int B>
__device__ __forceinline__ int local_to_internal(const BatchArgs &a, const BatchMesh &M, int64_t gl) {
    const int64_t g = B == 1 ? M.node0 + gl : M.dof0 + gl;
    return g < a.n_global ? a.g2i[g] : -1;
}

// Output position (global DOF of u) of internal DOF (node, comp).
template <int B>
__device__ __forceinline__ int64_t internal_to_output(const BatchArgs &a, const BatchMesh &M, int64_t node, int comp) {
    return B == 1 ? M.dof0 + (node - M.node0) : (int64_t)a.id[(int64_t)comp * a.nN + node];
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// CTA-wide sums of (a, b) in a fixed order, returned to every thread.
// Successive calls alternate between the two halves of `sh` (128 doubles,
// half = ph & 1): a half is written again only after every thread has
// passed the barrier of the call in between, so no closing barrier is needed.
__device__ __forceinline__ double2 block_sum2(double a, double b, double *sh, int ph) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    sh += 64 * (ph & 1);
    a = warp_sum_d(a);
    b = warp_sum_d(b);
    if (lane == 0) {
        sh[warp] = a;
        sh[32 + warp] = b;
    }
    __syncthreads();
    double x = 0.0, y = 0.0;
    for (int w = 0; w < nw; ++w) {
        x += sh[w];
        y += sh[32 + w];
    }
    return make_double2(x, y);
}

// Block of K at (slab, lane): FP32 from the per-mesh layout above, FP64 from
// the sliced-ELL layout (entry-major).
template <typename T, int B>
__device__ __forceinline__ void load_block(const T *__restrict__ val, int64_t slab, int lane, T *out) {
    if constexpr (sizeof(T) == 4) {
        load_v32<B, true>(val, slab, lane, out);
    } else {
#pragma unroll
        for (int e = 0; e < B * B; ++e) out[e] = __ldcs(val + (slab * B * B + e) * 32 + lane);
    }
}

// The B entries of node c of the multiplied vector (see spmv_operand); 2D
// FP32 vectors are read as one float2 per array.
template <bool FUSE_P, typename T, int B>
__device__ __forceinline__ void gather_node(const T *__restrict__ x, const T *__restrict__ z, T beta, int64_t c,
                                            T *g) {
    if constexpr (sizeof(T) == 4 && B == 2) {
        const float2 xv = *reinterpret_cast<const float2 *>(x + c * 2);
        if constexpr (FUSE_P) {
            const float2 zv = *reinterpret_cast<const float2 *>(z + c * 2);
            g[0] = fmaf(beta, xv.x, zv.x);
            g[1] = fmaf(beta, xv.y, zv.y);
        } else {
            g[0] = xv.x;
            g[1] = xv.y;
        }
    } else {
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if constexpr (FUSE_P) g[j] = fma(beta, x[c * B + j], z[c * B + j]);
            else g[j] = x[c * B + j];
        }
    }
}

// Entry idx of the multiplied vector: x itself, or with FUSE_P the CG search
// direction z + beta * x formed on the fly (x = the previous direction).
template <bool FUSE_P, typename T>
__device__ __forceinline__ T spmv_operand(const T *__restrict__ x, const T *__restrict__ z, T beta, int64_t idx) {
    if constexpr (FUSE_P) return fma(beta, x[idx], z[idx]);
    else return x[idx];
}

// y = (mask ? 0 : K v) over the mesh's slices, v = x or (FUSE_P) z + beta x;
// returns this thread's v.y share.  With FUSE_P this thread's rows of v are
// stored to pnew.  Rows at or beyond `rend` (the padding that rounds a mesh
// up to whole slices) are neither written nor counted: their vector entries
// are unset.  Slices sfirst, sfirst + sstride, ... below s1 (one warp each).
//
// A resident CTA or two per SM leave few warps to hide memory latency, so
// the loads are batched: a thread keeps U slabs in flight, loads its own
// row's entries up front and the slice extents ahead of use.  With W > 0,
// slices exactly W slabs wide (the interior of a structured 2D Q1 mesh: 9)
// take a pipelined path: their column indices were loaded while the
// previous slice was multiplied, so values, gathers and the next slice's
// indices all go out together -- one memory round trip per slice.  K and
// its column indices are read once per product and are loaded with the
// streaming hint, which leaves the L1 to the gathered vector entries.  The
// products are added in slab order on every path, so sums do not depend on
// U, W or the path taken.
//
// EPI selects what is stored per row (masked rows always get 0):
//   SPMV_Y       y = K v, and the v.y share is returned;
//   SPMV_RES     y = bv - K v (a residual);
//   SPMV_SMOOTH  y = v + Mv (bv - K v) with Mv the row's b x b block
//                ([node][i][j]), one damped block-Jacobi sweep; returns
//                this thread's bv.y share.
enum { SPMV_Y = 0, SPMV_RES = 1, SPMV_SMOOTH = 2 };
template <typename T, int B, bool FUSE_P, int U, int W = 0, int EPI = SPMV_Y>
__device__ __forceinline__ double grp_spmv(const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                                           const T *__restrict__ val, int64_t sfirst, int64_t s1, int64_t sstride,
                                           int64_t rend, const T *__restrict__ x, const T *__restrict__ z, T beta,
                                           T *__restrict__ pnew, T *__restrict__ y, const unsigned char *__restrict__ fixed,
                                           bool masked, const T *__restrict__ bv = nullptr,
                                           const T *__restrict__ Mv = nullptr) {
    constexpr int WP = W > 0 ? W : 1;
    const int lane = threadIdx.x & 31;
    double dot = 0.0;
    int64_t k0 = 0, k1 = 0, nk0 = 0, nk1 = 0;  // this slice's and the next slice's extents
    if (sfirst < s1) {
        k0 = sliceptr[sfirst];
        k1 = sliceptr[sfirst + 1];
    }
    if (sfirst + sstride < s1) {
        nk0 = sliceptr[sfirst + sstride];
        nk1 = sliceptr[sfirst + sstride + 1];
    }
    int cn[WP];  // column indices of this slice when it is exactly W wide
    if constexpr (W > 0) {
        if (k1 - k0 == W) {
#pragma unroll
            for (int u = 0; u < W; ++u) cn[u] = __ldcs(col + (k0 + u) * 32 + lane);
        }
    }
    for (int64_t s = sfirst; s < s1; s += sstride) {
        const int64_t r = s * 32 + lane;
        const bool own = r < rend;
        int64_t nnk0 = 0, nnk1 = 0;  // two slices ahead
        if (s + 2 * sstride < s1) {
            nnk0 = sliceptr[s + 2 * sstride];
            nnk1 = sliceptr[s + 2 * sstride + 1];
        }
        T pd[B];
        bool fx[B];
#pragma unroll
        for (int i = 0; i < B; ++i) {
            pd[i] = own ? spmv_operand<FUSE_P>(x, z, beta, r * B + i) : T(0);
            fx[i] = own && masked && fixed[r * B + i];
        }
        T acc[B];
#pragma unroll
        for (int i = 0; i < B; ++i) acc[i] = T(0);
        int ncn[WP];
        if (W > 0 && k1 - k0 == W) {
            T v[WP][B * B], g[WP][B];
#pragma unroll
            for (int u = 0; u < WP; ++u) load_block<T, B>(val, k0 + u, lane, v[u]);
#pragma unroll
            for (int u = 0; u < WP; ++u) gather_node<FUSE_P, T, B>(x, z, beta, (int64_t)cn[u], g[u]);
            if (nk1 - nk0 == W) {
#pragma unroll
                for (int u = 0; u < WP; ++u) ncn[u] = __ldcs(col + (nk0 + u) * 32 + lane);
            }
#pragma unroll
            for (int u = 0; u < WP; ++u)
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) acc[i] = fma(v[u][i * B + j], g[u][j], acc[i]);
        } else {
            if (W > 0 && nk1 - nk0 == W) {
#pragma unroll
                for (int u = 0; u < WP; ++u) ncn[u] = __ldcs(col + (nk0 + u) * 32 + lane);
            }
            int64_t k = k0;
            for (; k + U <= k1; k += U) {
                int c[U];
                T v[U][B * B], g[U][B];
#pragma unroll
                for (int u = 0; u < U; ++u) c[u] = __ldcs(col + (k + u) * 32 + lane);
#pragma unroll
                for (int u = 0; u < U; ++u) load_block<T, B>(val, k + u, lane, v[u]);
#pragma unroll
                for (int u = 0; u < U; ++u) gather_node<FUSE_P, T, B>(x, z, beta, (int64_t)c[u], g[u]);
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int i = 0; i < B; ++i)
#pragma unroll
                        for (int j = 0; j < B; ++j) acc[i] = fma(v[u][i * B + j], g[u][j], acc[i]);
            }
            for (; k < k1; ++k) {
                const int c = __ldcs(col + k * 32 + lane);
                T v[B * B], g[B];
                load_block<T, B>(val, k, lane, v);
                gather_node<FUSE_P, T, B>(x, z, beta, (int64_t)c, g);
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) acc[i] = fma(v[i * B + j], g[j], acc[i]);
            }
        }
        if (own) {
            if constexpr (EPI == SPMV_Y) {
                T rowdot = T(0);  // FP32: the row's share in FP32, one FP64 add per row
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    const int64_t d = r * B + i;
                    if constexpr (FUSE_P) pnew[d] = pd[i];
                    const T out = fx[i] ? T(0) : acc[i];
                    y[d] = out;
                    if constexpr (sizeof(T) == 4) rowdot = fma(pd[i], out, rowdot);
                    else dot += (double)pd[i] * (double)out;
                }
                if constexpr (sizeof(T) == 4) dot += (double)rowdot;
            } else {
                T res[B];
#pragma unroll
                for (int i = 0; i < B; ++i) res[i] = fx[i] ? T(0) : bv[r * B + i] - acc[i];
                if constexpr (EPI == SPMV_RES) {
#pragma unroll
                    for (int i = 0; i < B; ++i) y[r * B + i] = res[i];
                } else {
                    T rowdot = T(0);
#pragma unroll
                    for (int i = 0; i < B; ++i) {
                        T o = pd[i];
#pragma unroll
                        for (int j = 0; j < B; ++j) o = fma(Mv[(r * B + i) * B + j], res[j], o);
                        y[r * B + i] = o;
                        if constexpr (sizeof(T) == 4) rowdot = fma(bv[r * B + i], o, rowdot);
                        else dot += (double)bv[r * B + i] * (double)o;
                    }
                    if constexpr (sizeof(T) == 4) dot += (double)rowdot;
                }
            }
        }
        if constexpr (W > 0) {
#pragma unroll
            for (int u = 0; u < WP; ++u) cn[u] = ncn[u];
        }
        k0 = nk0;
        k1 = nk1;
        nk0 = nnk0;
        nk1 = nnk1;
    }
    return dot;
}

// grp_spmv as a separate function: a kernel that inlines several element
// classes' pipelines allocates registers for all of them at once, and the
// CG's SpMV of one class can come out slower there than on its own.  Called
// once per CG iteration, the call costs nothing measurable and the SpMV keeps
// the register allocation it gets in a single-class kernel.
template <typename T, int B, bool FUSE_P, int U, int W>
__device__ __noinline__ double grp_spmv_call(const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                                             const T *__restrict__ val, int64_t sfirst, int64_t s1, int64_t sstride,
                                             int64_t rend, const T *__restrict__ x, const T *__restrict__ z, T beta,
                                             T *__restrict__ pnew, T *__restrict__ y,
                                             const unsigned char *__restrict__ fixed, bool masked) {
    return grp_spmv<T, B, FUSE_P, U, W>(sliceptr, col, val, sfirst, s1, sstride, rend, x, z, beta, pnew, y, fixed,
                                        masked);
}

// The CG vector update of one group's nodes: x += alpha p, r -= alpha q,
// z = M^-1 r, and this thread's shares of r.z and r.r.
template <typename T, int B, int NVF>
__device__ __forceinline__ double2 cg_update(T *__restrict__ xv, T *__restrict__ rv, T *__restrict__ zv,
                                             const T *__restrict__ pv, const T *__restrict__ qv,
                                             const T *__restrict__ minv, T alpha, int64_t n0, int64_t n1, int64_t gt,
                                             int64_t gstride) {
    double prz = 0.0, prr = 0.0;
    // x += alpha p, r -= alpha q, z = M^-1 r; NV nodes per thread per step (loads first)
    constexpr int NV = sizeof(T) == 8 ? 1 : NVF;
    for (int64_t nb = n0 + gt; nb < n1; nb += NV * gstride) {
        T P[NV][B], X[NV][B], Q[NV][B], R[NV][B], Mi[NV][B * B];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const int64_t node = nb + v * gstride;
            if (node < n1) {
                if constexpr (sizeof(T) == 4 && B == 2) {  // one vector load per array
                    const float2 p2 = *reinterpret_cast<const float2 *>(pv + node * 2);
                    const float2 x2 = *reinterpret_cast<const float2 *>(xv + node * 2);
                    const float2 q2 = *reinterpret_cast<const float2 *>(qv + node * 2);
                    const float2 r2 = *reinterpret_cast<const float2 *>(rv + node * 2);
                    const float4 m4 = *reinterpret_cast<const float4 *>(minv + node * 4);
                    P[v][0] = p2.x, P[v][1] = p2.y, X[v][0] = x2.x, X[v][1] = x2.y;
                    Q[v][0] = q2.x, Q[v][1] = q2.y, R[v][0] = r2.x, R[v][1] = r2.y;
                    Mi[v][0] = m4.x, Mi[v][1] = m4.y, Mi[v][2] = m4.z, Mi[v][3] = m4.w;
                } else {
#pragma unroll
                    for (int i = 0; i < B; ++i) {
                        const int64_t d = node * B + i;
                        P[v][i] = pv[d];
                        X[v][i] = xv[d];
                        Q[v][i] = qv[d];
                        R[v][i] = rv[d];
                    }
#pragma unroll
                    for (int e = 0; e < B * B; ++e) Mi[v][e] = minv[node * B * B + e];
                }
            }
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const int64_t node = nb + v * gstride;
            if (node < n1) {
                T Xn[B], Z[B];
                T nrr = T(0), nrz = T(0);  // FP32: the node's shares in FP32, one FP64 add each
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    Xn[i] = fma(alpha, P[v][i], X[v][i]);
                    R[v][i] = fma(-alpha, Q[v][i], R[v][i]);
                    if constexpr (sizeof(T) == 4) nrr = fma(R[v][i], R[v][i], nrr);
                    else prr += (double)(R[v][i] * R[v][i]);
                }
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    T zi = T(0);
#pragma unroll
                    for (int j = 0; j < B; ++j) zi = fma(Mi[v][i * B + j], R[v][j], zi);
                    Z[i] = zi;
                    if constexpr (sizeof(T) == 4) nrz = fma(R[v][i], zi, nrz);
                    else prz += (double)(R[v][i] * zi);
                }
                if constexpr (sizeof(T) == 4) {
                    prr += (double)nrr;
                    prz += (double)nrz;
                }
                if constexpr (sizeof(T) == 4 && B == 2) {
                    *reinterpret_cast<float2 *>(xv + node * 2) = make_float2(Xn[0], Xn[1]);
                    *reinterpret_cast<float2 *>(rv + node * 2) = make_float2(R[v][0], R[v][1]);
                    *reinterpret_cast<float2 *>(zv + node * 2) = make_float2(Z[0], Z[1]);
                } else {
#pragma unroll
                    for (int i = 0; i < B; ++i) {
                        xv[node * B + i] = Xn[i];
                        rv[node * B + i] = R[v][i];
                        zv[node * B + i] = Z[i];
                    }
                }
            }
        }
    }
    return make_double2(prz, prr);
}

// One CTA working alone on a mesh.
struct SoloGroup {
    __device__ __forceinline__ int rank() const { return 0; }
    __device__ __forceinline__ int size() const { return 1; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ double2 sum2(double a, double b, double *red, double *, int ph) const { return block_sum2(a, b, red, ph); }
    __device__ __forceinline__ int max_flag(int *flag) const {
        __syncthreads();
        const int f = *flag;
        __syncthreads();
        return f;
    }
};

// A thread-block cluster working together on a mesh: hardware cluster
// barrier, partial sums exchanged through distributed shared memory and
// added in rank order (deterministic).
struct ClusterGroup {
    __device__ __forceinline__ int rank() const { return (int)cgrp::this_cluster().block_rank(); }
    __device__ __forceinline__ int size() const { return (int)cgrp::this_cluster().num_blocks(); }
    __device__ __forceinline__ void sync() const { cgrp::this_cluster().sync(); }
    // xch: 4 doubles, alternating halves like block_sum2's buffer (one cluster barrier per call)
    __device__ __forceinline__ double2 sum2(double a, double b, double *red, double *xch, int ph) const {
        const double2 p = block_sum2(a, b, red, ph);
        cgrp::cluster_group cl = cgrp::this_cluster();
        xch += 2 * (ph & 1);
        if (threadIdx.x == 0) {
            xch[0] = p.x;
            xch[1] = p.y;
        }
        cl.sync();
        double x = 0.0, y = 0.0;
        for (unsigned r = 0; r < cl.num_blocks(); ++r) {
            const double *rx = cl.map_shared_rank(xch, r);
            x += rx[0];
            y += rx[1];
        }
        return make_double2(x, y);
    }
    __device__ __forceinline__ int max_flag(int *flag) const {
        cgrp::cluster_group cl = cgrp::this_cluster();
        cl.sync();
        int f = 0;
        for (unsigned r = 0; r < cl.num_blocks(); ++r) f = max(f, *cl.map_shared_rank(flag, r));
        cl.sync();
        return f;
    }
};

}  // namespace sfem_dev

#include "sfem_mg.cuh"

namespace sfem_dev {

// Assemble and solve mesh `mb` with group G (a CTA or a cluster).
// UF: slabs in flight per thread in the CG loop's SpMV, WF: slice width of
// its pipelined path (0: none), NV: nodes per thread and step of the vector
// update.  The register budget of the calling kernel decides what fits.
template <class Grp, int NDIM, int NEN, int NGP, int B, bool MIXED, int UF = 4, int WF = 0, int NVF = 1,
          bool SPMV_CALL = false, bool MG = false>
__device__ __forceinline__ void process_mesh(const Grp &G, const ElemTableB &tab, const BatchArgs &a, int mb, double *red, double *xch,
                             int *s_flag) {
    using T = typename std::conditional<MIXED, float, double>::type;
    constexpr int GS = NEN * NDIM + 1;
    constexpr int NPAIR = NEN * (NEN + 1) / 2;
    extern __shared__ double smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const int grank = G.rank(), gsize = G.size();
    const int64_t gt = (int64_t)grank * blockDim.x + tid, gstride = (int64_t)gsize * blockDim.x;
    const int64_t gw = (int64_t)grank * nw + warp, gnw = (int64_t)gsize * nw;
    const int ngroups = nw / NGP;  // element groups of NGP warps
    const int grp = warp / NGP, gp = warp % NGP;
    double *sG = smem + (int64_t)grp * (NGP * 32 * GS + NGP * 32);
    double *sW = sG + NGP * 32 * GS;
    T *xv = (T *)a.vecT;
    T *rv = xv + a.nd, *zv = rv + a.nd, *pv = zv + a.nd, *qv = pv + a.nd, *pw = qv + a.nd;  // pv/pw: directions, alternating
    T *minv = pw + a.nd;  // [nN][B][B]
    int ph = 0;           // parity of the reduction buffers
    const T *valT = MIXED ? (const T *)a.val32 : (const T *)a.val64;
    const BatchMesh M = a.meshes[mb];
    // multigrid (MG): structured Q1 meshes in the mixed solver; compiled only
    // into the instantiations that ask for it, so the others keep their
    // register allocation
    constexpr bool MGOK = MG && MIXED && NEN == (1 << NDIM);
    const MgMesh *mgp = nullptr;
    if constexpr (MGOK) {
        if (a.mg && a.mg[mb].nlev >= 2) mgp = a.mg + mb;
    }
    T *zpre = zv;           // where the vector updates put M^-1 r: z, or the
    const T *mpre = minv;   // multigrid's pre-smoothing sweep
    if constexpr (MGOK) {
        if (mgp) {
            zpre = mgp->lev[0].x;
            mpre = mgp->lev[0].minv;
        }
    }
    unsigned long long t_start = 0;
    if (tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
    {
        const int64_t n0 = M.node0, n1 = M.node0 + M.nnode;      // real nodes
        const int64_t d0 = n0 * B, d1 = (M.node0 + ((M.nnode + 31) / 32) * 32) * B;  // padded DOF range

        // ---- 1. element stiffness (FP64), NGP warps per group of 32 elements
        const int64_t nel = M.elem1 - M.elem0;
        const int64_t rounds = (nel + 32 * ngroups * gsize - 1) / (32 * ngroups * gsize);
        for (int64_t rd = 0; rd < rounds; ++rd) {
            const int64_t e = M.elem0 + ((rd * gsize + grank) * ngroups + grp) * 32 + lane;
            const bool live = grp < ngroups && e < M.elem1;
            if (live) {
                double xe[NEN][NDIM];
#pragma unroll
                for (int an = 0; an < NEN; ++an) {
                    const int node = a.ien[(int64_t)an * a.nEl + e];
#pragma unroll
                    for (int i = 0; i < NDIM; ++i) xe[an][i] = a.X[(int64_t)node * NDIM + i];
                }
                double J[NDIM][NDIM];
#pragma unroll
                for (int i = 0; i < NDIM; ++i)
#pragma unroll
                    for (int k = 0; k < NDIM; ++k) {
                        double s = 0.0;
#pragma unroll
                        for (int an = 0; an < NEN; ++an) s = fma(xe[an][i], tab.dN[gp][an][k], s);
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
                if (det == 0.0) sfem_dev_error(a.err, SFEM_SINGULAR_JACOBIAN, e);
                double *g = sG + ((int64_t)gp * 32 + lane) * GS;
                // elasticity: sqrt(w |det J|) dN/dx (see k_element)
                const double sc = B > 1 ? sqrt(tab.w[gp] * fabs(det)) : 1.0;
#pragma unroll
                for (int an = 0; an < NEN; ++an)
#pragma unroll
                    for (int k = 0; k < NDIM; ++k) {
                        double s = 0.0;
#pragma unroll
                        for (int j = 0; j < NDIM; ++j) s = fma(tab.dN[gp][an][j], inv[j][k], s);
                        g[an * NDIM + k] = B > 1 ? s * sc : s;
                    }
                sW[gp * 32 + lane] = tab.w[gp] * fabs(det);
            }
            __syncthreads();
            if (live) {
                double lam = 0.0, mu = 0.0;
                if (B > 1) {
                    const int64_t iE = a.nE == 1 ? 0 : (a.nE == a.nmesh_all ? mb : e);
                    const int64_t iN = a.nNu == 1 ? 0 : (a.nNu == a.nmesh_all ? mb : e);
                    const double E = a.E[iE], nu = a.nu[iN];
                    if (NDIM == 2 && a.plane == SFEM_PLANE_STRESS) {
                        lam = nu * E / (1 - nu * nu);
                        mu = E / (2 * (1 + nu));
                    } else {
                        const double c = E / ((1 + nu) * (1 - 2 * nu));
                        lam = nu * c;
                        mu = (1 - 2 * nu) / 2 * c;
                    }
                }
                for (int p = gp; p < NPAIR; p += NGP) {
                    const int pa = tab.pa[p], pb = tab.pb[p];
                    if (B == 1) {
                        double s = 0.0;
#pragma unroll
                        for (int qg = 0; qg < NGP; ++qg) {
                            const double *g = sG + ((int64_t)qg * 32 + lane) * GS;
                            double dd = 0.0;
#pragma unroll
                            for (int k = 0; k < NDIM; ++k) dd = fma(g[pa * NDIM + k], g[pb * NDIM + k], dd);
                            s = fma(sW[qg * 32 + lane], dd, s);
                        }
                        a.kbuf[(int64_t)p * a.nEl + e] = s;
                    } else {
                        double S[NDIM][NDIM];
#pragma unroll
                        for (int i = 0; i < NDIM; ++i)
#pragma unroll
                            for (int j = 0; j < NDIM; ++j) S[i][j] = 0.0;
#pragma unroll
                        for (int qg = 0; qg < NGP; ++qg) {
                            const double *g = sG + ((int64_t)qg * 32 + lane) * GS;
#pragma unroll
                            for (int i = 0; i < NDIM; ++i) {
                                const double wa = g[pa * NDIM + i];
#pragma unroll
                                for (int j = 0; j < NDIM; ++j) S[i][j] = fma(wa, g[pb * NDIM + j], S[i][j]);
                            }
                        }
                        if (pa == pb) {
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
                                a.kbuf[((int64_t)p * B * B + i * B + j) * a.nEl + e] = v;
                            }
                    }
                }
            }
            __syncthreads();
        }

        G.sync();  // every element block of the mesh is in kbuf
        // ---- 2. gather into the mesh's K blocks (ascending element order)
        for (int64_t s = M.slice0 + gw; s < M.slice1; s += gnw) {
            const int64_t r64 = s * 32 + lane;
            const int r = (int)r64;
            const bool liver = r64 < a.nN;
            const int64_t slab0 = a.sliceptr[s], width = a.sliceptr[s + 1] - slab0;
            const int len = liver ? a.rowlen[r] : 0;
            const int64_t q0 = liver ? a.n2e_ptr[r] : 0, q1 = liver ? a.n2e_ptr[r + 1] : 0;
            // the multigrid instantiations (calls of their own in the serving kernel) read each
            // row's element lists once; the others keep the loop below and its register budget
            GatherRow<NEN> R;
            R.fast = false;
            if constexpr (MGOK) R.load(a.n2e, q0, q1, a.ien, a.nEl, r);
            for (int64_t k = 0; k < width; ++k) {
                const int64_t slab = slab0 + k;
                double acc[B * B];
#pragma unroll
                for (int i = 0; i < B * B; ++i) acc[i] = 0.0;
                if (MGOK && k < len && R.fast) {
                    R.template add<B>(a.col[slab * 32 + lane], a.kbuf, a.nEl, acc);
                } else if (k < len) {
                    const int c = a.col[slab * 32 + lane];
                    int prev = -1;
                    for (int64_t qq = q0; qq < q1; ++qq) {
                        const int e = a.n2e[qq];
                        if (e == prev) continue;
                        prev = e;
                        int nodes[NEN];
#pragma unroll
                        for (int an = 0; an < NEN; ++an) nodes[an] = a.ien[(int64_t)an * a.nEl + e];
#pragma unroll
                        for (int an = 0; an < NEN; ++an) {
                            if (nodes[an] != r) continue;
#pragma unroll
                            for (int bq = 0; bq < NEN; ++bq) {
                                if (nodes[bq] != c) continue;
                                if (an <= bq) {
                                    const int64_t base = (int64_t)sfem_pair(an, bq, NEN) * B * B;
#pragma unroll
                                    for (int i = 0; i < B * B; ++i) acc[i] += a.kbuf[(base + i) * a.nEl + e];
                                } else {
                                    const int64_t base = (int64_t)sfem_pair(bq, an, NEN) * B * B;
#pragma unroll
                                    for (int i = 0; i < B; ++i)
#pragma unroll
                                        for (int j = 0; j < B; ++j)
                                            acc[i * B + j] += a.kbuf[(base + j * B + i) * a.nEl + e];
                                }
                            }
                        }
                    }
                }
#pragma unroll
                for (int i = 0; i < B * B; ++i) {
                    a.val64[(slab * B * B + i) * 32 + lane] = acc[i];
                    if (MIXED) a.val32[v32_at<B>(slab, lane, i)] = (float)acc[i];
                }
            }
        }
        if (tid == 0) *s_flag = SFEM_OK;
        G.sync();

        // ---- 3. Dirichlet set-up
        for (int64_t d = d0 + gt; d < d1; d += gstride) {
            const int64_t node = d / B;
            a.fixed[d] = (node >= n1 || a.rowlen[node] == 0) ? 1 : 0;
            a.ud[d] = 0.0;
            a.x64[d] = 0.0;
            xv[d] = T(0);
        }
        for (int64_t g = M.dof0 + gt; g < M.dof0 + M.ndof; g += gstride) a.gfixed[g] = 0;
        G.sync();
        for (int64_t t = M.fix0 + gt; t < M.fix1; t += gstride) {
            const int64_t gl = a.fix_dofs[t] - 1;
            if (gl < 0 || gl >= M.ndof) {
                atomicMax(s_flag, (int)SFEM_BAD_INDEX);
                continue;
            }
            a.gfixed[M.dof0 + gl] = 1;
            const int i = local_to_internal<B>(a, M, gl);
            if (i >= 0) {
                a.fixed[i] = 1;
                a.ud[i] = a.fix_vals[t];
            }
        }
        G.sync();
        for (int64_t gl = gt; gl < M.ndof; gl += gstride) {
            if (local_to_internal<B>(a, M, gl) < 0 && !a.gfixed[M.dof0 + gl])
                atomicMax(s_flag, (int)SFEM_SINGULAR);  // a free DOF with no row in K
        }
        // b = -K q_d on the free DOFs (FP64)
        grp_spmv<double, B, false, 2>(a.sliceptr, a.col, a.val64, M.slice0 + gw, M.slice1, gnw, n1, a.ud, nullptr, 0.0,
                                   nullptr, a.q64, a.fixed, false);
        G.sync();
        for (int64_t d = n0 * B + gt; d < n1 * B; d += gstride) a.b64[d] = a.fixed[d] ? 0.0 : -a.q64[d];

        // ---- 4. preconditioner: inverse of each node's free-restricted diagonal block
        for (int64_t node = n0 + gt; node < n1; node += gstride) {
            double D[B][B];
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) D[i][j] = 0.0;
            const int len = a.rowlen[node];
            const int64_t slab0 = a.sliceptr[node >> 5];
            const int ln = (int)(node & 31);
            for (int k = 0; k < len; ++k)
                if (a.col[(slab0 + k) * 32 + ln] == (int)node) {
#pragma unroll
                    for (int i = 0; i < B; ++i)
#pragma unroll
                        for (int j = 0; j < B; ++j) D[i][j] = a.val64[((slab0 + k) * B * B + i * B + j) * 32 + ln];
                    break;
                }
            bool fx[B];
#pragma unroll
            for (int i = 0; i < B; ++i) fx[i] = a.fixed[node * B + i] != 0;
            double I[B][B];
            bool bad = false;
            if (B == 1 || !a.block_jacobi) {
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) I[i][j] = 0.0;
#pragma unroll
                for (int i = 0; i < B; ++i)
                    if (!fx[i]) {
                        if (!(D[i][i] != 0.0)) bad = true;
                        else I[i][i] = 1.0 / D[i][i];
                    }
            } else {
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j)
                        if (fx[i] || fx[j]) D[i][j] = (i == j) ? 1.0 : 0.0;
                double det;
                if (B == 2) {
                    det = D[0][0] * D[1][1] - D[0][1] * D[1][0];
                    I[0][0] = D[1][1];
                    I[0][1] = -D[0][1];
                    I[1][0] = -D[1][0];
                    I[1][1] = D[0][0];
                } else {
                    I[0][0] = D[1][1] * D[2][2] - D[1][2] * D[2][1];
                    I[0][1] = D[0][2] * D[2][1] - D[0][1] * D[2][2];
                    I[0][2] = D[0][1] * D[1][2] - D[0][2] * D[1][1];
                    I[1][0] = D[1][2] * D[2][0] - D[1][0] * D[2][2];
                    I[1][1] = D[0][0] * D[2][2] - D[0][2] * D[2][0];
                    I[1][2] = D[0][2] * D[1][0] - D[0][0] * D[1][2];
                    I[2][0] = D[1][0] * D[2][1] - D[1][1] * D[2][0];
                    I[2][1] = D[0][1] * D[2][0] - D[0][0] * D[2][1];
                    I[2][2] = D[0][0] * D[1][1] - D[0][1] * D[1][0];
                    det = D[0][0] * I[0][0] + D[0][1] * I[1][0] + D[0][2] * I[2][0];
                }
                if (!(det != 0.0)) bad = true;
                const double rd = det != 0.0 ? 1.0 / det : 0.0;
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) I[i][j] = (fx[i] || fx[j]) ? 0.0 : I[i][j] * rd;
            }
            if (bad) atomicMax(s_flag, (int)SFEM_SINGULAR);
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) minv[(node * B + i) * B + j] = (T)I[i][j];
        }
        G.sync();
        if constexpr (MGOK) {
            if (mgp) mg_setup<Grp, NDIM, B>(G, a, M, mgp, minv, s_flag);
        }

        // ---- 5. preconditioned CG
        // warm start: x = the free part of u_init (in x64 for the mixed
        // solver, whose FP32 iterate is a correction; in x for FP64), and the
        // initial residual b - K x in FP64
        const bool warm = a.u_init != nullptr;
        if (warm) {
            double *x0 = MIXED ? a.x64 : (double *)(void *)xv;
            for (int64_t node = n0 + gt; node < n1; node += gstride) {
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    const int64_t d = node * B + i;
                    const int64_t g = internal_to_output<B>(a, M, node, i);
                    x0[d] = (g >= 0 && !a.fixed[d]) ? a.u_init[g] : 0.0;
                }
            }
            G.sync();
            grp_spmv<double, B, false, 2>(a.sliceptr, a.col, a.val64, M.slice0 + gw, M.slice1, gnw, n1, x0, nullptr, 0.0,
                                          nullptr, a.q64, a.fixed, true);
            G.sync();
        }
        double rz = 0.0, bb = 0.0, rr0 = 0.0;
        {
            double prz = 0.0, pbb = 0.0, prr = 0.0;
            for (int64_t node = n0 + gt; node < n1; node += gstride) {
                T r[B];
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    const int64_t d = node * B + i;
                    const double bv = a.b64[d];
                    const double r0 = warm ? (a.fixed[d] ? 0.0 : bv - a.q64[d]) : bv;
                    r[i] = (T)r0;
                    rv[d] = r[i];
                    pv[d] = T(0);
                    pbb += bv * bv;
                    prr += r0 * r0;
                }
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    T zi = T(0);
#pragma unroll
                    for (int j = 0; j < B; ++j) zi = fma(mpre[(node * B + i) * B + j], r[j], zi);
                    zpre[node * B + i] = zi;
                    prz += (double)(r[i] * zi);
                }
            }
            constexpr int USM = sizeof(T) == 8 ? 2 : UF, WSM = sizeof(T) == 8 ? 0 : WF;
            if constexpr (MGOK) {
                if (mgp) {
                    G.sync();
                    prz = mg_vcycle<Grp, NDIM, B, USM, WSM>(G, a, M, mgp, rv, zv);
                }
            }
            const double2 t = G.sum2(prz, pbb, red, xch, ph++);
            rz = t.x;
            bb = t.y;
            rr0 = warm ? G.sum2(prr, 0.0, red, xch, ph++).x : bb;
        }
        const double tol2 = a.rtol * a.rtol * bb;
        double rr_ref = rr0, rr = rr0, beta = 0.0;
        int it = 0, refreshes = 0, status = G.max_flag(s_flag);
        bool done = status != SFEM_OK || !(bb > 0.0) || rr0 <= tol2;
        while (!done) {
            // q = K p with p = z + beta p_prev formed inside the SpMV (stored to pw)
            constexpr int US = sizeof(T) == 8 ? 2 : UF, WS = sizeof(T) == 8 ? 0 : WF;
            double pq;
            if constexpr (SPMV_CALL)
                pq = grp_spmv_call<T, B, true, US, WS>(a.sliceptr, a.col, valT, M.slice0 + gw, M.slice1, gnw, n1, pv,
                                                       zv, (T)beta, pw, qv, a.fixed, true);
            else
                pq = grp_spmv<T, B, true, US, WS>(a.sliceptr, a.col, valT, M.slice0 + gw, M.slice1, gnw, n1, pv, zv,
                                                  (T)beta, pw, qv, a.fixed, true);
            {
                T *t = pv;  // pv: the current direction
                pv = pw;
                pw = t;
            }
            pq = G.sum2(pq, 0.0, red, xch, ph++).x;
            if (!(pq > 0.0)) {
                status = SFEM_SINGULAR;
                break;
            }
            const T alpha = (T)(rz / pq);
            double prz, prr;
            {
                const double2 pr = cg_update<T, B, NVF>(xv, rv, zpre, pv, qv, mpre, alpha, n0, n1, gt, gstride);
                prz = pr.x;
                prr = pr.y;
                if constexpr (MGOK) {
                    if (mgp) {
                        G.sync();
                        prz = mg_vcycle<Grp, NDIM, B, US, WS>(G, a, M, mgp, rv, zv);
                    }
                }
            }
            const double2 t = G.sum2(prz, prr, red, xch, ph++);
            ++it;
            const double rz_prev = rz;
            rz = t.x;
            rr = t.y;
            beta = rz_prev != 0.0 ? rz / rz_prev : 0.0;
            if (!(rr == rr)) {
                status = SFEM_SINGULAR;
                break;
            }
            const bool at_tol = rr <= tol2, at_max = it >= a.maxit;
            if (!MIXED) {
                if (at_tol) break;
                if (at_max) {
                    status = SFEM_NOT_CONVERGED;
                    break;
                }
                continue;
            }
            if (at_tol || at_max || rr <= a.delta2 * rr_ref) {
                // FP64 refresh: fold the FP32 iterate, recompute r = b - K x in FP64
                for (int64_t d = n0 * B + gt; d < n1 * B; d += gstride) {
                    a.x64[d] += (double)xv[d];
                    xv[d] = T(0);
                }
                G.sync();
                grp_spmv<double, B, false, 2>(a.sliceptr, a.col, a.val64, M.slice0 + gw, M.slice1, gnw, n1, a.x64,
                                           nullptr, 0.0, nullptr, a.q64, a.fixed, true);
                G.sync();
                double frz = 0.0, frr = 0.0;
                for (int64_t node = n0 + gt; node < n1; node += gstride) {
                    T r[B];
#pragma unroll
                    for (int i = 0; i < B; ++i) {
                        const int64_t d = node * B + i;
                        const double v = a.fixed[d] ? 0.0 : a.b64[d] - a.q64[d];
                        r[i] = (T)v;
                        rv[d] = r[i];
                        frr += v * v;
                    }
#pragma unroll
                    for (int i = 0; i < B; ++i) {
                        T zi = T(0);
#pragma unroll
                        for (int j = 0; j < B; ++j) zi = fma(mpre[(node * B + i) * B + j], r[j], zi);
                        zpre[node * B + i] = zi;
                        frz += (double)(r[i] * zi);
                    }
                }
                if constexpr (MGOK) {
                    if (mgp) {
                        G.sync();
                        frz = mg_vcycle<Grp, NDIM, B, US, WS>(G, a, M, mgp, rv, zv);
                    }
                }
                const double2 f = G.sum2(frz, frr, red, xch, ph++);
                ++refreshes;
                rz = f.x;
                rr = f.y;
                rr_ref = rr;
                beta = rz_prev != 0.0 ? rz / rz_prev : 0.0;
                if (rr <= tol2) break;
                if (at_max) {
                    status = SFEM_NOT_CONVERGED;
                    break;
                }
            }
        }
        if (!MIXED && status != SFEM_SINGULAR) {
            for (int64_t d = n0 * B + gt; d < n1 * B; d += gstride) a.x64[d] = (double)xv[d];
        }
        G.sync();

        // ---- 6. u = q_d + x in the mesh's DOF numbering
        for (int64_t node = n0 + gt; node < n1; node += gstride) {
            if (a.rowlen[node] == 0) continue;
#pragma unroll
            for (int i = 0; i < B; ++i) {
                const int64_t g = internal_to_output<B>(a, M, node, i);
                if (g >= 0) a.u_out[g] = a.ud[node * B + i] + a.x64[node * B + i];
            }
        }
        for (int64_t t = M.fix0 + gt; t < M.fix1; t += gstride) {  // prescribed DOFs outside K
            const int64_t gl = a.fix_dofs[t] - 1;
            if (gl < 0 || gl >= M.ndof) continue;
            if (local_to_internal<B>(a, M, gl) < 0) a.u_out[M.dof0 + gl] = a.fix_vals[t];
        }
        if (grank == 0 && tid == 0) {
            unsigned long long t_end;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_end));
            sfem_batch_stats st;
            st.status = status;
            st.iterations = it;
            st.refreshes = refreshes;
            st.group_ctas = gsize;
            st.relres = bb > 0.0 ? sqrt(rr / bb) : 0.0;
            st.ms = (double)(t_end - t_start) * 1e-6;
            a.stats[mb] = st;
        }
    }
}

// process_mesh with the multigrid preconditioner, as a function of its own: a
// kernel that also runs meshes without it keeps the register allocation of
// its other paths (the hierarchy's set-up and cycle are calls).
template <class Grp, int NDIM, int NEN, int NGP, int B, bool MIXED, int UF, int WF, int NVF, bool SPMV_CALL>
__device__ __noinline__ void process_mesh_mg(const Grp &G, const ElemTableB &tab, const BatchArgs &a, int mb,
                                             double *red, double *xch, int *s_flag) {
    process_mesh<Grp, NDIM, NEN, NGP, B, MIXED, UF, WF, NVF, SPMV_CALL, true>(G, tab, a, mb, red, xch, s_flag);
}

// 2D classes fit two 512-thread CTAs per SM (64 registers); 3D elasticity
// needs the full register file of one.
}  // namespace sfem_dev
