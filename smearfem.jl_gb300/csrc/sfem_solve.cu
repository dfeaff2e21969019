// Dirichlet elimination and preconditioned CG (examples/vector3D.jl:314-322).
//
// The reference forms K_free = C'KC and inverts it densely.  Here the
// elimination is implicit: vectors keep every internal DOF, constrained DOFs
// are held at zero by a mask applied in the SpMV and the preconditioner, so
// CG on the full-length vectors performs exactly the arithmetic of CG on
// K_free.  The right-hand side is the lift C'(f - K q_d) and the result is
// q_d + C q_f.
//
// Kernels (all on the context stream):
//   k_spmv       y = mask .* (K x), sliced-ELL node-block rows, one lane per
//                node row, b x b block FMAs, coalesced 32-lane value loads;
//                optionally fuses the dot product x.y (the CG denominator)
//   k_update     x += alpha p, r -= alpha q, z = M^-1 r (Jacobi or nodal
//                block-Jacobi), fused r.z and r.r
//   k_update_p   p = z + beta p
// Global reductions are deterministic: each CTA writes a partial, the last
// CTA to arrive (atomic ticket) sums all partials in a fixed order and
// updates the CG scalars on the device, so the host only polls a flag once
// per chunk of iterations.  Nothing in these kernels waits on another CTA.
//
// Precision modes: SFEM_FP64 runs everything in FP64.  SFEM_MIXED runs the
// CG recurrences (matrix values, vectors, preconditioner, SpMV accumulation)
// in FP32 and keeps FP64 for the accumulated solution, the true residual
// b - K x (FP64 SpMV) and the Dirichlet lift: whenever the FP32 residual
// has dropped by `reliable_delta` since the last refresh, the FP32 iterate
// is folded into the FP64 solution and the residual is recomputed in FP64
// (iterative refinement that keeps the Krylov direction p).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "sfem_meshsolve.cuh"

namespace {

constexpr int SPMV_T = 256;
constexpr int UPD_T = 256;

struct CgScalars {
    double rz, rz_prev, pAp, alpha, beta, rr, bb, tol2, rr_ref, delta2;
    int it, done, status, maxit;
    int refresh;      // mixed: FP64 residual refresh requested by k_update
    int maxit_hit;    // mixed: stop after the pending refresh
    int nrefresh;     // mixed: refreshes performed
    unsigned int ticket[4];
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-reduce (a, b), publish the block partials, and let the last CTA sum
// all partials in a fixed order.  Returns true in every thread of the last
// CTA, with the totals in *ta / *tb (valid in thread 0).
__device__ bool reduce2_last(double a, double b, double *partial, unsigned int *ticket, double *ta, double *tb) {
    __shared__ double sa[32], sb[32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        sa[warp] = a;
        sb[warp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0, y = 0;
        for (int w = 0; w < nw; ++w) {
            x += sa[w];
            y += sb[w];
        }
        partial[2 * blockIdx.x] = x;
        partial[2 * blockIdx.x + 1] = y;
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double x = 0, y = 0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
        x += __ldcg(&partial[2 * i]);
        y += __ldcg(&partial[2 * i + 1]);
    }
    x = warp_sum(x);
    y = warp_sum(y);
    __syncthreads();
    if (lane == 0) {
        sa[warp] = x;
        sb[warp] = y;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double X = 0, Y = 0;
        for (int w = 0; w < nw; ++w) {
            X += sa[w];
            Y += sb[w];
        }
        *ta = X;
        *tb = Y;
        *ticket = 0;
    }
    return true;
}

// y = mask .* (K x); MODE 1 additionally reduces x.y into pAp and sets alpha;
// MODE 2 runs only while a mixed-precision refresh is pending.  MODE 4 (the
// Dirichlet lift K q_d, q_d zero but on the prescribed DOFs) skips the
// blocks whose column entries of x are all zero: their terms are zeros, so
// every sum is the same, and only rows next to prescribed DOFs read values.
template <typename T, int B, int MODE>
__global__ void __launch_bounds__(SPMV_T)
k_spmv(const int64_t *__restrict__ sliceptr, const int *__restrict__ col, const T *__restrict__ val, int64_t nN,
       int64_t nslices, const T *__restrict__ x, T *__restrict__ y, const unsigned char *__restrict__ fixed,
       CgScalars *S, double *partial) {
    if (MODE == 1 && S->done) return;
    if (MODE == 2 && !S->refresh) return;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    double dot = 0.0;
    // one warp per 32-row slice; grid-stride so a small grid can cover all slices
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += nwarps) {
        const int64_t r = s * 32 + lane;
        const int64_t slab0 = sliceptr[s], slab1 = sliceptr[s + 1];
        T acc[B];
#pragma unroll
        for (int i = 0; i < B; ++i) acc[i] = T(0);
        const int *cp = col + slab0 * 32 + lane;
        const T *vp = val + slab0 * (32 * B * B) + lane;
#pragma unroll 2
        for (int64_t k = slab0; k < slab1; ++k) {
            const int c = __ldg(cp);
            if constexpr (MODE == 4) {
                bool nz = false;
#pragma unroll
                for (int j = 0; j < B; ++j) nz = nz || __ldg(&x[(int64_t)c * B + j]) != T(0);
                if (!nz) {
                    cp += 32;
                    vp += 32 * B * B;
                    continue;
                }
            }
            T v[B * B];
#pragma unroll
            for (int i = 0; i < B * B; ++i) v[i] = __ldg(vp + i * 32);
            T xc[B];
#pragma unroll
            for (int j = 0; j < B; ++j) xc[j] = __ldg(&x[(int64_t)c * B + j]);
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) acc[i] = fma(v[i * B + j], xc[j], acc[i]);
            cp += 32;
            vp += 32 * B * B;
        }
        if (r < nN) {
            T rowdot = T(0);  // FP32: the row's share in FP32, one FP64 add
#pragma unroll
            for (int i = 0; i < B; ++i) {
                const int64_t d = r * B + i;
                const T out = fixed[d] ? T(0) : acc[i];
                y[d] = out;
                if (MODE == 1) {
                    if constexpr (sizeof(T) == 4) rowdot = fma(x[d], out, rowdot);
                    else dot += (double)(x[d] * out);
                }
            }
            if (MODE == 1 && sizeof(T) == 4) dot += (double)rowdot;
        }
    }
    if (MODE == 1) {
        double tot, dummy;
        if (reduce2_last(dot, 0.0, partial, &S->ticket[0], &tot, &dummy) && threadIdx.x == 0) {
            S->pAp = tot;
            if (!(tot > 0.0)) {  // K_free not positive definite along p (or NaN)
                S->status = SFEM_SINGULAR;
                S->done = 1;
                S->alpha = 0.0;
            } else {
                S->alpha = S->rz / tot;
            }
        }
    }
}

// The same product from the upper-triangle copy (sfem_sym.cu):
// y_r = sum_{c>=r} A_rc x_c + sum_{c<r} A_cr^T x_c, one lane per row, the
// upper part first, then the lower part, each in a fixed order (the result
// is deterministic).
// FUSE: the multiplied vector is the new CG direction p = z + beta x
// (x = the previous direction), formed on the fly from the gathered entries;
// each lane stores its own rows of p to pout.  This replaces the separate
// direction update (one pass over three vectors per iteration).
// EPI (multigrid V-cycle on the fine level): SPMV_RES stores y = bv - K x,
// SPMV_SMOOTH stores y = x + Mv (bv - K x) (Mv: the smoother's b x b blocks)
// and, with MODE 3, reduces bv.y into rz and sets beta = rz / rz_prev.
// Both skip once the solve is done.
//
// Traffic.  Every upper block is read twice: by its own row and, transposed,
// by its column's row.  Both reads come from DRAM only once if the second
// follows the first while the block is still in L2, i.e. if the slices in
// flight at any moment hold less than the L2.  So the grid is persistent (the
// CTAs that fit at once, striding over the slices in order) and each lane
// keeps U blocks of its row in flight, with the next batch's column indices
// (lower entries) already loaded: about 24 warps per SM cover the memory
// latency, and the open slices (~3.6k at 128^3, ~75 MB) stay well inside the
// L2.  A one-slice-per-warp grid kept ~10k slices (~200 MB) open and read
// 19-26% more than the algorithmic bytes.
template <typename T, int B, int MODE, bool FUSE = false, int EPI = sfem_dev::SPMV_Y, int U = 4>
__global__ void __launch_bounds__(SPMV_T)
k_spmv_sym(const int64_t *__restrict__ sptrU, const int *__restrict__ colU, const T *__restrict__ valU,
            const int64_t *__restrict__ sptrL, const int2 *__restrict__ lo, int64_t nN, int64_t nslices,
            const T *__restrict__ x, T *__restrict__ y, const unsigned char *__restrict__ fixed, CgScalars *S,
            double *partial, const T *__restrict__ z = nullptr, T *__restrict__ pout = nullptr,
            const T *__restrict__ bv = nullptr, const T *__restrict__ Mv = nullptr) {
    if ((MODE == 1 || MODE == 3 || EPI != sfem_dev::SPMV_Y) && S->done) return;
    const T beta = FUSE ? (T)S->beta : T(0);
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    double dot = 0.0;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += nwarps) {
        const int64_t r = s * 32 + lane;
        T acc[B];
#pragma unroll
        for (int i = 0; i < B; ++i) acc[i] = T(0);
        const int64_t u0 = sptrU[s], nu = sptrU[s + 1] - u0;
        const int64_t l0 = sptrL[s], nl = sptrL[s + 1] - l0;
        // upper part: A_rc x_c
        int cn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) cn[u] = u < nu ? __ldcs(&colU[(u0 + u) * 32 + lane]) : 0;
        for (int64_t k0 = 0; k0 < nu; k0 += U) {
            int c[U];
            T v[U][B * B];
            T xc[U][B];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                c[u] = cn[u];
                if (k0 + u < nu) {
                    load_v32<B, false>(valU, u0 + k0 + u, lane, v[u]);
                } else {
#pragma unroll
                    for (int e = 0; e < B * B; ++e) v[u][e] = T(0);
                }
#pragma unroll
                for (int j = 0; j < B; ++j) {
                    xc[u][j] = __ldg(&x[(int64_t)c[u] * B + j]);
                    if (FUSE) xc[u][j] = fma(beta, xc[u][j], __ldg(&z[(int64_t)c[u] * B + j]));
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) cn[u] = k0 + U + u < nu ? __ldcs(&colU[(u0 + k0 + U + u) * 32 + lane]) : 0;
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) acc[i] = fma(v[u][i * B + j], xc[u][j], acc[i]);
        }
        // lower part: A_cr^T x_c from c's upper storage
        int2 en[U];
#pragma unroll
        for (int u = 0; u < U; ++u) en[u] = u < nl ? __ldcs(&lo[(l0 + u) * 32 + lane]) : make_int2(-1, 0);
        for (int64_t k0 = 0; k0 < nl; k0 += U) {
            T v[U][B * B];
            T xc[U][B];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int2 e = en[u];
                if (e.x >= 0) {
                    load_v32<B, false>(valU, e.x >> 5, e.x & 31, v[u]);
                } else {
#pragma unroll
                    for (int q = 0; q < B * B; ++q) v[u][q] = T(0);
                }
                const int c = e.x >= 0 ? e.y : 0;
#pragma unroll
                for (int j = 0; j < B; ++j) {
                    xc[u][j] = __ldg(&x[(int64_t)c * B + j]);
                    if (FUSE) xc[u][j] = fma(beta, xc[u][j], __ldg(&z[(int64_t)c * B + j]));
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                en[u] = k0 + U + u < nl ? __ldcs(&lo[(l0 + k0 + U + u) * 32 + lane]) : make_int2(-1, 0);
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) acc[i] = fma(v[u][j * B + i], xc[u][j], acc[i]);
        }
        if (r < nN) {
            if constexpr (EPI == sfem_dev::SPMV_Y) {
                T rowdot = T(0);  // the row's share in T, one FP64 add per row (FP64 is a slow pipe on GB300)
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    const int64_t d = r * B + i;
                    const T out = fixed[d] ? T(0) : acc[i];
                    y[d] = out;
                    T pd = x[d];
                    if (FUSE) {
                        pd = fma(beta, pd, z[d]);
                        pout[d] = pd;
                    }
                    if (MODE == 1) rowdot = fma(pd, out, rowdot);
                }
                if (MODE == 1) dot += (double)rowdot;
            } else {
                T res[B];
#pragma unroll
                for (int i = 0; i < B; ++i) res[i] = fixed[r * B + i] ? T(0) : bv[r * B + i] - acc[i];
                T rowdot = T(0);
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    T o = res[i];
                    if constexpr (EPI == sfem_dev::SPMV_SMOOTH) {
                        o = x[r * B + i];
#pragma unroll
                        for (int j = 0; j < B; ++j) o = fma(Mv[(r * B + i) * B + j], res[j], o);
                        rowdot = fma(bv[r * B + i], o, rowdot);
                    }
                    y[r * B + i] = o;
                }
                if constexpr (EPI == sfem_dev::SPMV_SMOOTH) dot += (double)rowdot;
            }
        }
    }
    if (MODE == 3) {
        double tot, dummy;
        if (reduce2_last(dot, 0.0, partial, &S->ticket[0], &tot, &dummy) && threadIdx.x == 0) {
            S->rz_prev = S->rz;
            S->rz = tot;
            S->beta = S->rz_prev != 0.0 ? tot / S->rz_prev : 0.0;
        }
    }
    if (MODE == 1) {
        double tot, dummy;
        if (reduce2_last(dot, 0.0, partial, &S->ticket[0], &tot, &dummy) && threadIdx.x == 0) {
            S->pAp = tot;
            if (!(tot > 0.0)) {
                S->status = SFEM_SINGULAR;
                S->done = 1;
                S->alpha = 0.0;
            } else {
                S->alpha = S->rz / tot;
            }
        }
    }
}

// x += alpha p; r -= alpha q; z = M^-1 r; reduce r.z and r.r; CG scalar update.
// PC: 0 Jacobi (minv per DOF), 1 block-Jacobi (minv: B x B per node).
// MIXED: the recursive FP32 residual never ends the solve; reaching the
// tolerance, dropping by delta since the last refresh, or hitting maxit
// requests an FP64 refresh instead (k_fold / k_spmv MODE 2 / k_refresh).
// Each thread owns NPT = 16 bytes / sizeof(T) consecutive nodes (4 in FP32,
// 2 in FP64): their B * NPT entries of x, p, q, r are B 16-byte vectors, and
// their inverse blocks MW 16-byte vectors, so every load and store is a
// 16-byte access and the block product needs no data from other threads.
// (One node per thread issued four times the load instructions, with a
// 12-byte stride, and filled the load queues.)  Nodes after the last whole
// group are handled one per thread.
// MGPRE (multigrid): z and minv are the fine level's pre-smoothing sweep and
// smoother; r.z and beta are left to the cycle's last product.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using V = float4;
    static constexpr int E = 4;
};
template <>
struct Vec16<double> {
    using V = double2;
    static constexpr int E = 2;
};

template <typename T, int B, int PC, bool MIXED, bool MGPRE = false>
__global__ void __launch_bounds__(UPD_T)
k_update_node(int64_t nN, T *__restrict__ x, T *__restrict__ r, T *__restrict__ z, const T *__restrict__ p,
              const T *__restrict__ q, const T *__restrict__ minv, CgScalars *S, double *partial) {
    if (S->done) return;
    using V = typename Vec16<T>::V;
    constexpr int NPT = Vec16<T>::E;                           // nodes per thread
    constexpr int MW = (PC == 0 || B == 1) ? B : B * B;        // inverse entries per node
    const T alpha = (T)S->alpha;
    double rz = 0.0, rr = 0.0;
    const int64_t ngrp = nN / NPT;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t g = tid0; g < ngrp; g += stride) {
        V xv[B], pv[B], qv[B], rv[B], mv[MW];
        const V *xs = reinterpret_cast<const V *>(x + g * NPT * B);
        const V *ps = reinterpret_cast<const V *>(p + g * NPT * B);
        const V *qs = reinterpret_cast<const V *>(q + g * NPT * B);
        const V *rs = reinterpret_cast<const V *>(r + g * NPT * B);
        const V *ms = reinterpret_cast<const V *>(minv + g * NPT * MW);
#pragma unroll
        for (int k = 0; k < B; ++k) {
            xv[k] = xs[k];
            pv[k] = ps[k];
            qv[k] = qs[k];
            rv[k] = rs[k];
        }
#pragma unroll
        for (int k = 0; k < MW; ++k) mv[k] = ms[k];
        T *xe = reinterpret_cast<T *>(xv);
        const T *pe = reinterpret_cast<const T *>(pv);
        const T *qe = reinterpret_cast<const T *>(qv);
        T *re = reinterpret_cast<T *>(rv);
        const T *me = reinterpret_cast<const T *>(mv);
#pragma unroll
        for (int i = 0; i < NPT * B; ++i) {
            xe[i] = fma(alpha, pe[i], xe[i]);
            re[i] = fma(-alpha, qe[i], re[i]);
        }
        V zv[B];
        T *ze = reinterpret_cast<T *>(zv);
        T grz = T(0), grr = T(0);  // FP32: the group's shares in FP32, one FP64 add each
#pragma unroll
        for (int n = 0; n < NPT; ++n)
#pragma unroll
            for (int i = 0; i < B; ++i) {
                T zi;
                if (MW == B) {
                    zi = me[n * B + i] * re[n * B + i];
                } else {
                    zi = T(0);
#pragma unroll
                    for (int j = 0; j < B; ++j) zi = fma(me[(n * B + i) * B + j], re[n * B + j], zi);
                }
                ze[n * B + i] = zi;
                if constexpr (sizeof(T) == 4) {
                    grz = fma(re[n * B + i], zi, grz);
                    grr = fma(re[n * B + i], re[n * B + i], grr);
                } else {
                    rz += (double)(re[n * B + i] * zi);
                    rr += (double)(re[n * B + i] * re[n * B + i]);
                }
            }
        if constexpr (sizeof(T) == 4) {
            rz += (double)grz;
            rr += (double)grr;
        }
        V *xd = reinterpret_cast<V *>(x + g * NPT * B);
        V *rd = reinterpret_cast<V *>(r + g * NPT * B);
        V *zd = reinterpret_cast<V *>(z + g * NPT * B);
#pragma unroll
        for (int k = 0; k < B; ++k) {
            xd[k] = xv[k];
            rd[k] = rv[k];
            zd[k] = zv[k];
        }
    }
    // the last nN % NPT nodes, one per thread
    for (int64_t node = ngrp * NPT + tid0; node < nN; node += stride) {
        T rl[B];
#pragma unroll
        for (int i = 0; i < B; ++i) {
            const int64_t d = node * B + i;
            x[d] = fma(alpha, p[d], x[d]);
            rl[i] = fma(-alpha, q[d], r[d]);
            r[d] = rl[i];
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
            T zi;
            if (MW == B) {
                zi = minv[node * B + i] * rl[i];
            } else {
                zi = T(0);
#pragma unroll
                for (int j = 0; j < B; ++j) zi = fma(minv[(node * B + i) * B + j], rl[j], zi);
            }
            z[node * B + i] = zi;
            rz += (double)(rl[i] * zi);
            rr += (double)(rl[i] * rl[i]);
        }
    }
    double trz, trr;
    if (reduce2_last(rz, rr, partial, &S->ticket[1], &trz, &trr) && threadIdx.x == 0) {
        S->rr = trr;
        S->it += 1;
        if (!MGPRE) {
            S->rz_prev = S->rz;
            S->rz = trz;
            S->beta = S->rz_prev != 0.0 ? trz / S->rz_prev : 0.0;
        }
        if (!(trr == trr)) {
            S->done = 1;
            S->status = SFEM_SINGULAR;
        } else if (MIXED) {
            if (S->it >= S->maxit) S->maxit_hit = 1;
            if (trr <= S->tol2 || trr <= S->delta2 * S->rr_ref || S->maxit_hit) S->refresh = 1;
        } else if (trr <= S->tol2) {
            S->done = 1;
            S->status = SFEM_OK;
        } else if (S->it >= S->maxit) {
            S->done = 1;
            S->status = SFEM_NOT_CONVERGED;
        }
    }
}

template <typename T>
__global__ void k_update_p(int64_t n, T *__restrict__ p, const T *__restrict__ z, const CgScalars *S) {
    if (S->done) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = fma((T)S->beta, p[i], z[i]);
}

// ---- set-up kernels --------------------------------------------------------

// Mark every internal DOF of a node no element uses as fixed (it is not in K).
__global__ void k_mask_inactive(const int *__restrict__ rowlen, int64_t nN, int b, unsigned char *__restrict__ fixed) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nN * b) return;
    fixed[t] = rowlen[t / b] == 0 ? 1 : 0;
}

__global__ void k_fix(const int64_t *__restrict__ dofs, const double *__restrict__ vals, int64_t nfix, int64_t n,
                      const int *__restrict__ g2i, unsigned char *__restrict__ fixed, double *__restrict__ ud,
                      unsigned char *__restrict__ gfixed, DevErr *err) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nfix) return;
    const int64_t g = dofs[t] - 1;
    if (g < 0 || g >= n) {
        sfem_dev_error(err, SFEM_BAD_INDEX, t);
        return;
    }
    gfixed[g] = 1;
    const int i = g2i[g];
    if (i < 0) return;  // empty row/column of K
    fixed[i] = 1;
    ud[i] = vals[t];
}

// Internal vector from a global one (f), zero where no global DOF maps.
__global__ void k_gather_global(const double *__restrict__ fg, int64_t n, const int *__restrict__ g2i,
                                double *__restrict__ fi) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const int i = g2i[g];
    if (i >= 0) fi[i] = fg[g];
}

__global__ void k_zero_fixed(int64_t nd, const unsigned char *__restrict__ fixed, double *__restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nd && fixed[i]) x[i] = 0.0;
}

// b = f - K ud on free DOFs (0 on fixed).
__global__ void k_rhs(int64_t nd, const double *__restrict__ f, const double *__restrict__ Kud,
                      const unsigned char *__restrict__ fixed, double *__restrict__ bvec) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nd) return;
    bvec[i] = fixed[i] ? 0.0 : (f ? f[i] : 0.0) - Kud[i];
}

// Global DOFs that are free but have no row in K make K_free singular.
__global__ void k_check_empty(int64_t n, const int *__restrict__ g2i, const unsigned char *__restrict__ gfixed,
                              DevErr *err) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    if (g2i[g] < 0 && !gfixed[g]) sfem_dev_error(err, SFEM_SINGULAR, g);
}

// Preconditioner from the diagonal blocks.  PC 0: 1/K_ii; PC 1: inverse of the
// node's b x b block restricted to its free components.
template <typename T, int B, int PC>
__global__ void k_precond(const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                          const double *__restrict__ val, const int *__restrict__ rowlen, int64_t nN,
                          const unsigned char *__restrict__ fixed, T *__restrict__ minv, DevErr *err) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nN) return;
    double D[B][B];
    for (int i = 0; i < B; ++i)
        for (int j = 0; j < B; ++j) D[i][j] = 0.0;
    const int len = rowlen[node];
    const int64_t s = node >> 5;
    const int lane = (int)(node & 31);
    const int64_t slab0 = sliceptr[s];
    for (int k = 0; k < len; ++k) {
        const int64_t slab = slab0 + k;
        if (col[slab * 32 + lane] == (int)node) {
            for (int i = 0; i < B; ++i)
                for (int j = 0; j < B; ++j) D[i][j] = val[(slab * B * B + i * B + j) * 32 + lane];
            break;
        }
    }
    bool fx[B];
    bool any_free = false;
    for (int i = 0; i < B; ++i) {
        fx[i] = fixed[node * B + i] != 0;
        any_free |= !fx[i];
    }
    if (PC == 0 || B == 1) {
        for (int i = 0; i < B; ++i) {
            T v = T(0);
            if (!fx[i]) {
                if (!(D[i][i] != 0.0) || !isfinite(D[i][i])) sfem_dev_error(err, SFEM_SINGULAR, node * B + i);
                else v = (T)(1.0 / D[i][i]);
            }
            if (PC == 0) minv[node * B + i] = v;
            else minv[(node * B + i) * B + i] = v;
        }
        return;
    }
    // free-restricted block: fixed rows/cols -> identity, invert, zero them again
    for (int i = 0; i < B; ++i)
        for (int j = 0; j < B; ++j)
            if (fx[i] || fx[j]) D[i][j] = (i == j) ? 1.0 : 0.0;
    double I[B][B];
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
    if (any_free && (!(det != 0.0) || !isfinite(det))) sfem_dev_error(err, SFEM_SINGULAR, node * B);
    const double rdet = det != 0.0 ? 1.0 / det : 0.0;
    for (int i = 0; i < B; ++i)
        for (int j = 0; j < B; ++j)
            minv[(node * B + i) * B + j] = (fx[i] || fx[j]) ? T(0) : (T)(I[i][j] * rdet);
}

// u_global[g] = ud[i] + x[i]  (or the prescribed value for DOFs outside K)
__global__ void k_scatter_out(int64_t n, const int *__restrict__ g2i, const double *__restrict__ ud,
                              const double *__restrict__ x, double *__restrict__ ug) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const int i = g2i[g];
    ug[g] = i >= 0 ? ud[i] + x[i] : 0.0;
}

__global__ void k_fixed_out(const int64_t *__restrict__ dofs, const double *__restrict__ vals, int64_t nfix,
                            const int *__restrict__ g2i, double *__restrict__ ug) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nfix) return;
    const int64_t g = dofs[t] - 1;
    if (g2i[g] < 0) ug[g] = vals[t];
}

// ---- mixed-precision glue ---------------------------------------------------

template <typename T>
__global__ void k_cast(int64_t n, const double *__restrict__ a, T *__restrict__ b) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (T)a[i];
}

__global__ void k_fold(int64_t n, double *__restrict__ x64, float *__restrict__ x32, const CgScalars *S) {
    if (!S->refresh) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x64[i] += (double)x32[i];
        x32[i] = 0.0f;
    }
}

// r64 = b - Kx64 (masked), r32 = (float) r64, z32 = M^-1 r32; reduce r.z, r.r.
template <int B, int PC, bool MGPRE = false>
__global__ void __launch_bounds__(UPD_T)
k_refresh(int64_t nN, const double *__restrict__ bvec, const double *__restrict__ Kx, const unsigned char *__restrict__ fixed,
          double *__restrict__ r64, float *__restrict__ r32, float *__restrict__ z32, const float *__restrict__ minv,
          CgScalars *S, double *partial) {
    if (!S->refresh) return;
    double rz = 0.0, rr = 0.0;
    for (int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; node < nN;
         node += (int64_t)gridDim.x * blockDim.x) {
        float rv[B];
#pragma unroll
        for (int i = 0; i < B; ++i) {
            const int64_t d = node * B + i;
            const double v = fixed[d] ? 0.0 : bvec[d] - Kx[d];
            r64[d] = v;
            rv[i] = (float)v;
            r32[d] = rv[i];
            rr += v * v;
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
            float zi;
            if (PC == 0) {
                zi = minv[node * B + i] * rv[i];
            } else {
                zi = 0.0f;
#pragma unroll
                for (int j = 0; j < B; ++j) zi = fmaf(minv[(node * B + i) * B + j], rv[j], zi);
            }
            z32[node * B + i] = zi;
            rz += (double)(rv[i] * zi);
        }
    }
    double trz, trr;
    if (reduce2_last(rz, rr, partial, &S->ticket[2], &trz, &trr) && threadIdx.x == 0) {
        S->rr = trr;
        S->rr_ref = trr;
        if (!MGPRE) {
            S->rz = trz;
            S->beta = S->rz_prev != 0.0 ? trz / S->rz_prev : 0.0;
        }
        S->refresh = 0;
        S->nrefresh += 1;
        if (trr <= S->tol2) {
            S->done = 1;
            S->status = SFEM_OK;
        } else if (S->maxit_hit) {
            S->done = 1;
            S->status = SFEM_NOT_CONVERGED;
        }
    }
}

// ||mask .* (b - K x)||^2 into S->rr (final true residual of the FP64 path)
__global__ void __launch_bounds__(UPD_T)
k_true_residual(int64_t nd, const double *__restrict__ bvec, const double *__restrict__ Kx,
                const unsigned char *__restrict__ fixed, CgScalars *S, double *partial) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0;
    if (i < nd && !fixed[i]) {
        const double v = bvec[i] - Kx[i];
        rr = v * v;
    }
    double t, dummy;
    if (reduce2_last(rr, 0.0, partial, &S->ticket[2], &t, &dummy) && threadIdx.x == 0) S->rr = t;
}

// initial z = M^-1 r and rz, rr (FP64 or FP32 vectors)
// MGPRE: z and minv are the multigrid's pre-smoothing sweep and smoother;
// r.z is left at zero for the cycle's last product to set.
template <typename T, int B, int PC, bool MGPRE = false>
__global__ void __launch_bounds__(UPD_T)
k_init(int64_t nN, const T *__restrict__ r, T *__restrict__ z, T *__restrict__ p, const T *__restrict__ minv,
       CgScalars *S, double *partial) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double rz = 0.0, rr = 0.0;
    if (node < nN) {
#pragma unroll
        for (int i = 0; i < B; ++i) {
            const int64_t d = node * B + i;
            T zi;
            if (PC == 0) {
                zi = minv[d] * r[d];
            } else {
                zi = T(0);
#pragma unroll
                for (int j = 0; j < B; ++j) zi = fma(minv[d * B + j], r[node * B + j], zi);
            }
            z[d] = zi;
            p[d] = T(0);
            rz += (double)(r[d] * zi);
            rr += (double)r[d] * (double)r[d];
        }
    }
    double trz, trr;
    if (reduce2_last(rz, rr, partial, &S->ticket[3], &trz, &trr) && threadIdx.x == 0) {
        if (MGPRE) trz = 0.0;
        S->rz = trz;
        S->rz_prev = trz;
        S->rr = trr;
        S->rr_ref = trr;
        S->beta = 0.0;
    }
}

// ---- multigrid (sfem_mg.cuh) on the whole GPU: one launch per pass ----------

// Structured-grid check of a mesh (0-based node ids, element index fastest):
// *ok is cleared when an element differs from the meshgrid connectivity.
__global__ void k_grid_check(const int *__restrict__ ien, int64_t nEl, int nen, int ndim, int ne, int *ok) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nEl) return;
    for (int c = 0; c < nen; ++c)
        if ((int64_t)ien[(int64_t)c * nEl + e] != mg_grid_node(ndim, ne, e, c) - 1) *ok = 0;
}

#define SFEM_GRID_LOOP                                                                 \
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;                 \
    const int64_t gs = (int64_t)gridDim.x * blockDim.x;

template <int NDIM, int B>
__global__ void k_mg_free(const sfem_dev::BatchArgs a, const BatchMesh M, const MgLevel F, const MgLevel C, int l) {
    SFEM_GRID_LOOP
    sfem_dev::mg_pass_free<NDIM, B>(a, M, F, C, l, gt, gs);
}
// Fine level as a stencil level for the Galerkin pass: F.A (tiled stencil
// blocks, the FP32 values of the upper-triangle copy, lower blocks
// transposed) and F.fr (free flags) from K's upper-triangle storage; one lane
// per row, one warp per slice.  Off-grid neighbours get zero blocks; a
// column that is not a grid neighbour sets SFEM_BAD_INDEX.
template <int NDIM, int B>
__global__ void k_mg_fine_stencil(const int64_t *__restrict__ sptrU, const int *__restrict__ colU,
                                  const float *__restrict__ valU, const int64_t *__restrict__ sptrL,
                                  const int2 *__restrict__ lo, const unsigned char *__restrict__ fixed, int64_t nslices,
                                  const MgLevel F, int *flag) {
    constexpr int S = NDIM == 2 ? 9 : 27;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t sl = t >> 5;
    const int lane = (int)(t & 31);
    if (sl >= nslices) return;
    const int64_t r = sl * 32 + lane;
    if (r >= F.nnode) return;
    int ci[3];
    sfem_dev::mg_coords<NDIM>(r, F.n, ci);
    unsigned written = 0;
    auto put = [&](int c, const float *blk, bool transpose) {
        int cj[3];
        sfem_dev::mg_coords<NDIM>(c, F.n, cj);
        bool nb = true;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) nb = nb && abs(cj[d] - ci[d]) <= 1;
        if (!nb) {
            atomicMax(flag, (int)SFEM_BAD_INDEX);
            return;
        }
        const int st = sfem_dev::mg_stencil<NDIM>(ci, cj);
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j)
                F.A[sfem_dev::mg_a<NDIM, B>(r, st, i * B + j)] = transpose ? blk[j * B + i] : blk[i * B + j];
        written |= 1u << st;
    };
    const int64_t u0 = sptrU[sl], nu = sptrU[sl + 1] - u0;
    for (int64_t k = 0; k < nu; ++k) {
        const int c = colU[(u0 + k) * 32 + lane];
        if (k > 0 && c == (int)r) continue;  // padding (the diagonal is the first upper entry)
        float blk[B * B];
        load_v32<B, false>(valU, u0 + k, lane, blk);
        put(c, blk, false);
    }
    const int64_t l0 = sptrL[sl], nl = sptrL[sl + 1] - l0;
    for (int64_t k = 0; k < nl; ++k) {
        const int2 e = lo[(l0 + k) * 32 + lane];
        if (e.x < 0) continue;
        float blk[B * B];
        load_v32<B, false>(valU, e.x >> 5, e.x & 31, blk);
        put(e.y, blk, true);
    }
#pragma unroll
    for (int st = 0; st < S; ++st)
        if (!(written >> st & 1u))
#pragma unroll
            for (int e = 0; e < B * B; ++e) F.A[sfem_dev::mg_a<NDIM, B>(r, st, e)] = 0.0f;
#pragma unroll
    for (int c = 0; c < B; ++c) F.fr[r * B + c] = fixed[r * B + c] ? 0 : 1;
}

// Fine-level smoother W D^-1 (mg_pass_fine) from the fine stencil copy: the
// same row sums in the same (ascending column) order, with fixed trip counts;
// off-grid blocks are zero and add nothing.
template <int NDIM, int B>
__global__ void __launch_bounds__(256) k_mg_fine_st(const MgLevel F, const float *__restrict__ bj, float *minv) {
    constexpr int S = NDIM == 2 ? 9 : 27;
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= F.nnode) return;
    int ci[3];
    sfem_dev::mg_coords<NDIM>(r, F.n, ci);
    float Di[B * B];
#pragma unroll
    for (int e = 0; e < B * B; ++e) Di[e] = bj[r * B * B + e];
    float rs[B];
#pragma unroll
    for (int i = 0; i < B; ++i) rs[i] = 0.0f;
#pragma unroll 3
    for (int st = 0; st < S; ++st) {
        int cj[3] = {0, 0, 0};
        const int o[3] = {st % 3 - 1, (st / 3) % 3 - 1, NDIM == 3 ? st / 9 - 1 : 0};
#pragma unroll
        for (int d = 0; d < NDIM; ++d) cj[d] = min(max(ci[d] + o[d], 0), F.n);
        const int64_t c = sfem_dev::mg_index<NDIM>(cj, F.n);
        float blk[B * B];
#pragma unroll
        for (int e = 0; e < B * B; ++e) blk[e] = F.A[sfem_dev::mg_a<NDIM, B>(r, st, e)];
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) {
                if (!F.fr[c * B + j]) continue;
                float v = 0.0f;
#pragma unroll
                for (int mm = 0; mm < B; ++mm) v = fmaf(Di[i * B + mm], blk[mm * B + j], v);
                rs[i] += fabsf(v);
            }
    }
    float rho = 0.0f;
#pragma unroll
    for (int i = 0; i < B; ++i) rho = fmaxf(rho, rs[i]);
    const float w = rho > 0.0f ? (4.0f / 3.0f) / rho : 0.0f;
#pragma unroll
    for (int e = 0; e < B * B; ++e) minv[r * B * B + e] = w * Di[e];
}

// Galerkin product of the single-mesh set-up, one direction at a time.
// The prolongation is the tensor product of the 1D interpolations (per
// direction the weights mg_w1), so A_{l+1} = P'^T A_l P' is three (2D: two)
// coarsenings of one direction each, on box grids coarse in the directions
// done so far.  Each keeps the 3^ndim stencil: output block (OD in DIR,
// the other offsets unchanged) of node I sums, over the 3 fine candidates
// ia of I and the 3 offsets od in DIR, w(ia, I) w(ia + od, I + OD) times
// input block (od, others) of row ia.  The first pass masks the input with
// the free flags of its row and column DOFs (the fine pairs the direct
// product skips), the last one zeroes the rows and columns of fixed coarse
// DOFs, as the direct product does; zero weights stand for pairs outside
// the supports or the grid, and off-grid blocks are zero.  ~7 loads per
// output block against ~81 for the direct product (mg_pass_galerkin, which
// the batch and serving kernels keep: it needs no scratch).
struct MgBox {
    int n[3];  // elements per direction (n[2] = 0 in 2D)
};
__device__ __forceinline__ int64_t box_index(const MgBox &g, const int c[3]) {
    return c[0] + (int64_t)(g.n[0] + 1) * (c[1] + (int64_t)(g.n[1] + 1) * c[2]);
}
template <int NDIM>
__device__ __forceinline__ int box_stencil(const int o[3]) {
    return NDIM == 3 ? (o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1) : (o[1] + 1) * 3 + (o[0] + 1);
}
template <int NDIM, int B, int DIR, bool MASK, bool FINAL>
__global__ void __launch_bounds__(256)
k_mg_coarsen(const float *__restrict__ Ain, const MgBox gin, const unsigned char *__restrict__ frin,
             float *__restrict__ Aout, const MgBox gout, const unsigned char *__restrict__ frout, int64_t nout) {
    constexpr int NO = NDIM == 3 ? 9 : 3;  // offsets of the other directions
    constexpr int D1 = DIR == 0 ? 1 : 0, D2 = NDIM == 3 ? (DIR == 2 ? 1 : 2) : 2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nout * NO) return;
    const int64_t I = t % nout;
    const int oo = (int)(t / nout);
    int cI[3];
    {
        const int64_t n0 = gout.n[0] + 1, n1 = gout.n[1] + 1;
        cI[0] = (int)(I % n0);
        cI[1] = (int)((I / n0) % n1);
        cI[2] = (int)(I / (n0 * n1));
    }
    int o[3] = {0, 0, 0};
    o[D1] = oo % 3 - 1;
    if (NDIM == 3) o[D2] = oo / 3 - 1;
    const int nf = gin.n[DIR], nc = gout.n[DIR], Ic = cI[DIR];
    const int cc = min(2 * Ic, nf);
    float acc[3][B * B];
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
        for (int e = 0; e < B * B; ++e) acc[q][e] = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int ia = cc - 1 + a;
        const bool ina = ia >= 0 && ia <= nf;
        const float wI = ina ? sfem_dev::mg_w1(ia, Ic, nf) : 0.0f;
        int rc[3] = {cI[0], cI[1], cI[2]};
        rc[DIR] = min(max(ia, 0), nf);
        const int64_t row = box_index(gin, rc);
#pragma unroll
        for (int od = -1; od <= 1; ++od) {
            int oi[3] = {o[0], o[1], o[2]};
            oi[DIR] = od;
            const int sin = box_stencil<NDIM>(oi);
            float blk[B * B];
#pragma unroll
            for (int e = 0; e < B * B; ++e) blk[e] = Ain[sfem_dev::mg_a<NDIM, B>(row, sin, e)];
            if constexpr (MASK) {
                int cj[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) cj[d] = min(max(rc[d] + oi[d], 0), gin.n[d]);
                const int64_t colj = box_index(gin, cj);
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j)
                        if (!frin[row * B + i] || !frin[colj * B + j]) blk[i * B + j] = 0.0f;
            }
            const int j1 = ia + od;
#pragma unroll
            for (int OD = -1; OD <= 1; ++OD) {
                const int J = Ic + OD;
                const float wJ = (ina && J >= 0 && J <= nc && j1 >= 0 && j1 <= nf) ? sfem_dev::mg_w1(j1, J, nf) : 0.0f;
                const float w = wI * wJ;
#pragma unroll
                for (int e = 0; e < B * B; ++e) acc[OD + 1][e] = fmaf(w, blk[e], acc[OD + 1][e]);
            }
        }
    }
#pragma unroll
    for (int OD = -1; OD <= 1; ++OD) {
        int oc[3] = {o[0], o[1], o[2]};
        oc[DIR] = OD;
        if constexpr (FINAL) {
            int cJ[3];
            bool valid = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                cJ[d] = cI[d] + oc[d];
                valid = valid && cJ[d] >= 0 && cJ[d] <= gout.n[d];
            }
            if (valid) {
                const int64_t Jn = box_index(gout, cJ);
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j)
                        if (!frout[I * B + i] || !frout[Jn * B + j]) acc[OD + 1][i * B + j] = 0.0f;
            }
        }
        const int sout = box_stencil<NDIM>(oc);
#pragma unroll
        for (int e = 0; e < B * B; ++e) Aout[sfem_dev::mg_a<NDIM, B>(I, sout, e)] = acc[OD + 1][e];
    }
}

template <int NDIM, int B>
__global__ void k_mg_smoother(const MgLevel C, int *flag) {
    SFEM_GRID_LOOP
    sfem_dev::mg_pass_smoother<NDIM, B>(C, gt, gs, flag);
}
template <int NDIM, int B>
__global__ void k_mg_coarsest(const MgLevel C, int n, float *cinv, double *gj, int *flag) {  // one CTA
    sfem_dev::mg_pass_coarsest<NDIM, B>(C, n, cinv, gj, flag);
}
// cycle passes: each exits at once when the solve is done
template <int NDIM, int B>
__global__ void k_mg_restrict(const BatchMesh M, const MgLevel F, const MgLevel C, int l, int smooth,
                              const CgScalars *S) {
    if (S->done) return;
    SFEM_GRID_LOOP
    sfem_dev::mg_restrict<NDIM, B>(M, F, C, l, smooth != 0, gt, gs);
}
template <int NDIM, int B, int EPI>
__global__ void k_mg_stencil(const MgLevel C, float *out, const CgScalars *S) {
    if (S->done) return;
    SFEM_GRID_LOOP
    sfem_dev::mg_stencil_pass<NDIM, B, EPI>(C, out, gt, gs);
}
template <int NDIM, int B>
__global__ void k_mg_prolong(const sfem_dev::BatchArgs a, const BatchMesh M, const MgLevel F, const MgLevel C, int l,
                             const float *xc, const CgScalars *S) {
    if (S->done) return;
    SFEM_GRID_LOOP
    sfem_dev::mg_prolong<NDIM, B>(a, M, F, C, l, xc, gt, gs);
}
__global__ void k_mg_csolve(const MgLevel C, int n, const float *cinv, const CgScalars *S) {
    if (S->done) return;
    SFEM_GRID_LOOP
    sfem_dev::mg_coarse_solve(C, n, cinv, gt, gs);
}
#undef SFEM_GRID_LOOP

// The levels from `solo` down, their coarse solve and the way back up to
// level solo's smoothing, by ONE CTA with CTA barriers: the few thousand
// nodes of these levels keep one CTA busy, and one launch replaces two per
// level (each of them bound by a few memory round trips, not by bytes).
// The passes and their order are those of the grid-wide kernels.
constexpr int MG_SOLO_T = 1024;
constexpr int64_t MG_SOLO_MAX_NODES = 1024;  // largest level (and its finer neighbour / 8) run by the one CTA
template <int NDIM, int B>
__global__ void __launch_bounds__(MG_SOLO_T)
k_mg_solo(const sfem_dev::BatchArgs a, const BatchMesh M, const __grid_constant__ MgMesh mg, int solo,
          const CgScalars *S) {
    if (S->done) return;
    const int64_t st = threadIdx.x, ss = blockDim.x;
    const int L = mg.nlev;
    for (int l = solo; l < L; ++l) {
        sfem_dev::mg_restrict<NDIM, B>(M, mg.lev[l - 1], mg.lev[l], l - 1, l + 1 < L, st, ss);
        __syncthreads();
        if (l + 1 < L) {
            sfem_dev::mg_stencil_pass<NDIM, B, sfem_dev::SPMV_RES>(mg.lev[l], mg.lev[l].t, st, ss);
            __syncthreads();
        }
    }
    sfem_dev::mg_coarse_solve(mg.lev[L - 1], mg.ndc, mg.cinv, st, ss);
    __syncthreads();
    const float *xin = mg.lev[L - 1].x;
    for (int l = L - 2; l >= solo; --l) {
        sfem_dev::mg_prolong<NDIM, B>(a, M, mg.lev[l], mg.lev[l + 1], l, xin, st, ss);
        __syncthreads();
        sfem_dev::mg_stencil_pass<NDIM, B, sfem_dev::SPMV_SMOOTH>(mg.lev[l], mg.lev[l].t, st, ss);
        __syncthreads();
        xin = mg.lev[l].t;
    }
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------

template <typename T>
struct Vecs {
    T *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *minv = nullptr;
};

// Grid that fills the GPU once: resident CTAs per SM x SMs, capped at `need`.
template <typename K>
unsigned resident_grid(sfem_ctx *ctx, K kernel, int threads, int64_t need) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int64_t g = (int64_t)per_sm * ctx->num_sms;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, need > 0 ? need : 1));
}

class Solver {
   public:
    Solver(sfem_ctx *c, sfem_matrix *K, const sfem_solve_opts &o) : ctx(c), K(K), m(K->mesh), opts(o) {}
    ~Solver() {
        for (void *p : owned) sfem_dfree(ctx, p);
        if (gexec) cudaGraphExecDestroy(gexec);
        for (auto &e : events) cudaEventDestroy(e);
        cudaStreamSynchronize(ctx->stream);
    }

    // u0: optional initial guess in global DOF numbering (its prescribed
    // entries are ignored); NULL starts from zero.
    int run(const int64_t *fixed_dofs, int64_t nfix, const double *fixed_vals, const double *f, double *u_out,
            int mem_space, sfem_solve_stats *stats, const double *u0 = nullptr);

   private:
    template <typename T>
    int alloc(T **p, int64_t n, const char *what) {
        SFEM_TRY(sfem_dalloc(ctx, (void **)p, sizeof(T) * (n > 0 ? n : 1), what));
        owned.push_back(*p);
        return SFEM_OK;
    }
    template <int B>
    int solve_b(double *x64_out);
    template <typename T, int B, int PC, bool MIXED>
    int cg_loop(Vecs<T> &v, double *x64, double *r64, double *q64);
    template <typename T, int B>
    void launch_spmv(const T *val, const T *x, T *y, bool fused);
    int read_scalars(CgScalars *h);
    // multigrid (mixed precision, structured meshes)
    int mg_detect();
    template <int NDIM, int B>
    int mg_build(const float *bj);
    template <int NDIM, int B>
    int mg_cycle(const float *r, float *z);
    template <int B>
    int mg_cycle_b(const float *r, float *z) {
        if (m->ndim == 2) {
            if constexpr (B <= 2) return mg_cycle<2, B>(r, z);
        } else {
            if constexpr (B != 2) return mg_cycle<3, B>(r, z);
        }
        return SFEM_UNSUPPORTED;
    }

    sfem_ctx *ctx;
    sfem_matrix *K;
    sfem_mesh *m;
    sfem_solve_opts opts;
    std::vector<void *> owned;
    unsigned char *fixed = nullptr, *gfixed = nullptr;
    double *ud = nullptr, *bvec = nullptr, *partial = nullptr;
    double *r0vec = nullptr;  // initial residual: bvec, or b - K x0 for a warm start
    CgScalars *S = nullptr;
    int64_t nd = 0;  // internal DOFs = nN * b
    unsigned spmv_grid = 1, upd_grid = 1, vec_grid = 1;
    cudaGraphExec_t gexec = nullptr;
    std::vector<cudaEvent_t> events;
    double ms_spmv = 0.0;
    int spmv_timed = 0;
    int reliable = 0;
    int iterations = 0;
    int status = SFEM_OK;
    double relres = 0.0;
    bool use_mg = false;
    MgMesh mg{};
    sfem_dev::BatchArgs mga{};  // the fields the hierarchy passes read: pattern, FP64 K, mask
    BatchMesh mgM{};
    int mg_launches = 0;        // kernels per cycle
};

// Elements per direction when the matrix's mesh is the structured meshgrid
// grid (checked on the device once per mesh), else 0.
int Solver::mg_detect() {
    if (m->mg_ne >= 0) return m->mg_ne;
    int ne = (m->fclass == SFEM_Q1 && m->nen == (1 << m->ndim)) ? mg_grid_ne(m->ndim, m->nN, m->nEl) : 0;
    if (mg_levels(ne) < 2) ne = 0;
    if (ne > 0) {
        int *ok = nullptr, one = 1;
        SFEM_TRY(alloc(&ok, 1, "grid check"));
        SFEM_TRY(sfem_copy_in(ctx, ok, &one, sizeof(int), SFEM_MEM_HOST));
        k_grid_check<<<(unsigned)sfem_cdiv(m->nEl, 256), 256, 0, ctx->stream>>>(m->ien, m->nEl, m->nen, m->ndim, ne, ok);
        SFEM_LAUNCHED(ctx);
        SFEM_TRY(sfem_copy_out(ctx, &one, ok, sizeof(int), SFEM_MEM_HOST));
        if (!one) ne = 0;
    }
    m->mg_ne = ne;
    return ne;
}

// The hierarchy of this solve's K: layout, fine smoother, Galerkin levels,
// coarsest inverse.  bj: the FP32 block-Jacobi inverse.
template <int NDIM, int B>
int Solver::mg_build(const float *bj) {
    SfemRange range_("sfem multigrid set-up");
    const int ne = m->mg_ne;
    const int64_t bytes = mg_layout(NDIM, B, ne, nd, nullptr, nullptr);
    char *buf = nullptr;
    SFEM_TRY(alloc(&buf, bytes, "multigrid"));
    mg_layout(NDIM, B, ne, nd, buf, &mg);
    memset(&mga, 0, sizeof(mga));
    mga.sliceptr = m->sliceptr;
    mga.col = m->col;
    mga.rowlen = m->rowlen;
    mga.val64 = K->val;
    mga.fixed = fixed;
    mga.sptrU = K->sptrU;  // the Galerkin pass reads the upper-triangle FP32 copy
    mga.colU = K->colU;
    mga.valU = K->valU;
    memset(&mgM, 0, sizeof(mgM));
    mgM.nnode = m->nN;
    mgM.slice1 = m->nslices;
    int *flag = nullptr, zero = 0;
    SFEM_TRY(alloc(&flag, 1, "multigrid status"));
    SFEM_TRY(sfem_copy_in(ctx, flag, &zero, sizeof(int), SFEM_MEM_HOST));
    auto grid = [&](int64_t work) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(sfem_cdiv(work, 256), 64 * ctx->num_sms)); };
    const int L = mg.nlev, S = NDIM == 2 ? 9 : 27;
    // the fine level as a stencil level (scratch for this set-up): the
    // Galerkin pass then reads each fine block with one load group
    MgLevel F0 = mg.lev[0];
    struct Scratch {  // freed in stream order when the set-up has been enqueued
        sfem_ctx *ctx;
        void *p[4] = {nullptr, nullptr, nullptr, nullptr};
        ~Scratch() {
            for (void *q : p) sfem_dfree(ctx, q);
        }
    } scratch{ctx};
    {
        const int64_t nn = (int64_t)F0.nnode;
        SFEM_TRY(sfem_dalloc(ctx, &scratch.p[0], sizeof(float) * S * B * B * ((nn + 31) / 32 * 32),
                             "multigrid fine stencil"));
        SFEM_TRY(sfem_dalloc(ctx, &scratch.p[1], (size_t)(nn * B), "multigrid fine flags"));
        F0.A = (float *)scratch.p[0];
        F0.fr = (unsigned char *)scratch.p[1];
        k_mg_fine_stencil<NDIM, B><<<(unsigned)sfem_cdiv(m->nslices * 32, 256), 256, 0, ctx->stream>>>(
            K->sptrU, K->colU, K->valU, K->sptrL, K->lo, fixed, m->nslices, F0, flag);
        // the fine smoother from the copy
        k_mg_fine_st<NDIM, B><<<(unsigned)sfem_cdiv(nn, 256), 256, 0, ctx->stream>>>(F0, bj, mg.lev[0].minv);
        ctx->launches += 2;
    }
    // scratch of the direction-wise Galerkin passes, sized for level 0 -> 1
    float *T1 = nullptr, *T2 = nullptr;
    {
        const int64_t nf1 = mg.lev[0].n + 1, nc1 = mg.lev[1].n + 1;
        const int64_t t1 = NDIM == 3 ? nc1 * nf1 * nf1 : nc1 * nf1, t2 = NDIM == 3 ? nc1 * nc1 * nf1 : 1;
        SFEM_TRY(sfem_dalloc(ctx, &scratch.p[2], sizeof(float) * S * B * B * ((t1 + 31) / 32 * 32),
                             "multigrid Galerkin scratch"));
        SFEM_TRY(sfem_dalloc(ctx, &scratch.p[3], sizeof(float) * S * B * B * ((t2 + 31) / 32 * 32),
                             "multigrid Galerkin scratch"));
        T1 = (float *)scratch.p[2];
        T2 = (float *)scratch.p[3];
    }
    auto cgrid = [&](int64_t n) { return (unsigned)sfem_cdiv(n, 256); };
    for (int l = 0; l + 1 < L; ++l) {
        k_mg_free<NDIM, B><<<grid(mg.lev[l + 1].nnode), 256, 0, ctx->stream>>>(mga, mgM, mg.lev[l], mg.lev[l + 1], l);
        // level 0 through its stencil copy
        const MgLevel &Fl = l == 0 ? F0 : mg.lev[l];
        const MgLevel &Cl = mg.lev[l + 1];
        const int nf = Fl.n, nc = Cl.n;
        constexpr int NO = NDIM == 3 ? 9 : 3;
        const MgBox g0{{nf, nf, NDIM == 3 ? nf : 0}}, g1{{nc, nf, NDIM == 3 ? nf : 0}}, g2{{nc, nc, nf}},
            g3{{nc, nc, NDIM == 3 ? nc : 0}};
        auto nodes = [](const MgBox &g) { return (int64_t)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1); };
        if constexpr (NDIM == 3) {
            k_mg_coarsen<NDIM, B, 0, true, false><<<cgrid(nodes(g1) * NO), 256, 0, ctx->stream>>>(
                Fl.A, g0, Fl.fr, T1, g1, nullptr, nodes(g1));
            k_mg_coarsen<NDIM, B, 1, false, false><<<cgrid(nodes(g2) * NO), 256, 0, ctx->stream>>>(
                T1, g1, nullptr, T2, g2, nullptr, nodes(g2));
            k_mg_coarsen<NDIM, B, 2, false, true><<<cgrid(nodes(g3) * NO), 256, 0, ctx->stream>>>(
                T2, g2, nullptr, Cl.A, g3, Cl.fr, nodes(g3));
            ctx->launches += 4;
        } else {
            k_mg_coarsen<NDIM, B, 0, true, false><<<cgrid(nodes(g1) * NO), 256, 0, ctx->stream>>>(
                Fl.A, g0, Fl.fr, T1, g1, nullptr, nodes(g1));
            k_mg_coarsen<NDIM, B, 1, false, true><<<cgrid(nodes(g3) * NO), 256, 0, ctx->stream>>>(
                T1, g1, nullptr, Cl.A, g3, Cl.fr, nodes(g3));
            ctx->launches += 3;
        }
        if (l + 2 < L) {
            k_mg_smoother<NDIM, B><<<grid(mg.lev[l + 1].nnode), 256, 0, ctx->stream>>>(mg.lev[l + 1], flag);
            SFEM_LAUNCHED(ctx);
        }
    }
    k_mg_coarsest<NDIM, B><<<1, 512, 0, ctx->stream>>>(mg.lev[L - 1], mg.ndc, mg.cinv, mg.gj, flag);
    SFEM_LAUNCHED(ctx);
    int f = 0;
    SFEM_TRY(sfem_copy_out(ctx, &f, flag, sizeof(int), SFEM_MEM_HOST));
    if (f != 0) return sfem_set_error(ctx, f, "multigrid set-up failed (%d)", f);
    return SFEM_OK;
}

// z = V(r) with the fine level's pre-smoothing sweep already in lev[0].x;
// the last product reduces r.z and sets beta.  Every kernel exits at once
// when the solve is done.
template <int NDIM, int B>
int Solver::mg_cycle(const float *r, float *z) {
    using namespace sfem_dev;
    const int L = mg.nlev;
    auto grid = [&](int64_t work) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(sfem_cdiv(work, 256), 8 * ctx->num_sms)); };
    const MgLevel &F0 = mg.lev[0];
    int n = 0;
    {
        auto kern = k_spmv_sym<float, B, 0, false, SPMV_RES>;
        kern<<<resident_grid(ctx, kern, SPMV_T, spmv_grid), SPMV_T, 0, ctx->stream>>>(
            K->sptrU, K->colU, K->valU, K->sptrL, K->lo, m->nN, m->nslices, F0.x, F0.t, fixed, S, partial, nullptr,
            nullptr, r, nullptr);
    }
    ++n;
    // levels solo.. run by one CTA (k_mg_solo); solo = L: none
    int solo = L;
    for (int l = 2; l < L; ++l)
        if (mg.lev[l].nnode <= MG_SOLO_MAX_NODES && mg.lev[l - 1].nnode <= 8 * MG_SOLO_MAX_NODES) {
            solo = l;
            break;
        }
    for (int l = 1; l < solo; ++l) {
        k_mg_restrict<NDIM, B><<<grid(mg.lev[l].nnode), 256, 0, ctx->stream>>>(mgM, mg.lev[l - 1], mg.lev[l], l - 1,
                                                                               l + 1 < L ? 1 : 0, S);
        ++n;
        if (l + 1 < L) {
            k_mg_stencil<NDIM, B, SPMV_RES><<<grid(mg.lev[l].nnode), 256, 0, ctx->stream>>>(mg.lev[l], mg.lev[l].t, S);
            ++n;
        }
    }
    const float *xin = mg.lev[L - 1].x;
    if (solo < L) {
        k_mg_solo<NDIM, B><<<1, MG_SOLO_T, 0, ctx->stream>>>(mga, mgM, mg, solo, S);
        ++n;
        if (solo <= L - 2) xin = mg.lev[solo].t;
    } else {
        k_mg_csolve<<<1, 256, 0, ctx->stream>>>(mg.lev[L - 1], mg.ndc, mg.cinv, S);
        ++n;
    }
    for (int l = std::min(L - 2, solo - 1); l >= 1; --l) {
        k_mg_prolong<NDIM, B><<<grid(mg.lev[l].nnode), 256, 0, ctx->stream>>>(mga, mgM, mg.lev[l], mg.lev[l + 1], l,
                                                                              xin, S);
        k_mg_stencil<NDIM, B, SPMV_SMOOTH><<<grid(mg.lev[l].nnode), 256, 0, ctx->stream>>>(mg.lev[l], mg.lev[l].t, S);
        n += 2;
        xin = mg.lev[l].t;
    }
    k_mg_prolong<NDIM, B><<<grid(F0.nnode), 256, 0, ctx->stream>>>(mga, mgM, F0, mg.lev[1], 0, xin, S);
    {
        auto kern = k_spmv_sym<float, B, 3, false, SPMV_SMOOTH>;
        kern<<<resident_grid(ctx, kern, SPMV_T, spmv_grid), SPMV_T, 0, ctx->stream>>>(
            K->sptrU, K->colU, K->valU, K->sptrL, K->lo, m->nN, m->nslices, F0.x, z, fixed, S, partial, nullptr,
            nullptr, r, F0.minv);
    }
    n += 2;
    ctx->launches += n;
    mg_launches = n;
    return sfem_cuda_status(ctx, cudaGetLastError(), "multigrid cycle launch");
}

template <typename T, int B>
void Solver::launch_spmv(const T *val, const T *x, T *y, bool fused) {
    if constexpr (sizeof(T) == 4) {
        if (K->sym_state == 1 && opts.fp32_storage == SFEM_FP32_UPPER) {
            if (fused) {
                auto kern = k_spmv_sym<float, B, 1>;
                kern<<<resident_grid(ctx, kern, SPMV_T, spmv_grid), SPMV_T, 0, ctx->stream>>>(
                    K->sptrU, K->colU, K->valU, K->sptrL, K->lo, m->nN, m->nslices, x, y, fixed, S, partial,
                    nullptr, nullptr, nullptr, nullptr);
            } else {
                auto kern = k_spmv_sym<float, B, 0>;
                kern<<<resident_grid(ctx, kern, SPMV_T, spmv_grid), SPMV_T, 0, ctx->stream>>>(
                    K->sptrU, K->colU, K->valU, K->sptrL, K->lo, m->nN, m->nslices, x, y, fixed, S, partial,
                    nullptr, nullptr, nullptr, nullptr);
            }
            SFEM_LAUNCHED(ctx);
            return;
        }
    }
    if (fused) {
        auto kern = k_spmv<T, B, 1>;
        kern<<<spmv_grid, SPMV_T, 0, ctx->stream>>>(
            m->sliceptr, m->col, val, m->nN, m->nslices, x, y, fixed, S, partial);
    } else {
        auto kern = k_spmv<T, B, 0>;
        kern<<<spmv_grid, SPMV_T, 0, ctx->stream>>>(
            m->sliceptr, m->col, val, m->nN, m->nslices, x, y, fixed, S, partial);
    }
    SFEM_LAUNCHED(ctx);
}

int Solver::read_scalars(CgScalars *h) {
    SFEM_CUDA(ctx, cudaMemcpyAsync(h, S, sizeof(CgScalars), cudaMemcpyDeviceToHost, ctx->stream));
    SFEM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SFEM_OK;
}

template <typename T, int B, int PC, bool MIXED>
int Solver::cg_loop(Vecs<T> &v, double *x64, double *r64, double *q64) {
    SfemRange range_("sfem pcg");
    const T *val = nullptr;
    if constexpr (sizeof(T) == 8) val = (const T *)K->val;
    else val = (const T *)K->val32;
    CgScalars *h = (CgScalars *)ctx->h_small;
    const int chunk = opts.check_every > 0 ? opts.check_every : 32;
    const bool profile = opts.profile != 0;
    // With the upper-triangle FP32 SpMV the direction update is folded into
    // the SpMV, which writes p to the other of two buffers; an even chunk keeps
    // the buffers' roles the same at every graph launch.
    T *p2 = nullptr;
    bool fuse_p = false;
    if constexpr (sizeof(T) == 4) {
        fuse_p = K->sym_state == 1 && opts.fp32_storage == SFEM_FP32_UPPER && chunk % 2 == 0;
        if (fuse_p) SFEM_TRY(alloc(&p2, nd, "p (second buffer)"));
    }
    auto enqueue_iter = [&](int slot) {
        T *pcur = v.p;
        bool done_spmv = false;
        if constexpr (sizeof(T) == 4) {
            if (fuse_p) {
                T *pin = (slot % 2 == 0) ? v.p : p2, *pout = (slot % 2 == 0) ? p2 : v.p;
                if (profile) cudaEventRecord(events[2 * slot], ctx->stream);
                auto kern = k_spmv_sym<float, B, 1, true>;
                kern<<<resident_grid(ctx, kern, SPMV_T, spmv_grid), SPMV_T, 0, ctx->stream>>>(
                    K->sptrU, K->colU, K->valU, K->sptrL, K->lo, m->nN,
                                                             m->nslices, pin, v.q, fixed, S, partial, v.z, pout,
                                                             nullptr, nullptr);
                SFEM_LAUNCHED(ctx);
                if (profile) cudaEventRecord(events[2 * slot + 1], ctx->stream);
                pcur = pout;
                done_spmv = true;
            }
        }
        if (!done_spmv) {
            k_update_p<T><<<vec_grid, 256, 0, ctx->stream>>>(nd, v.p, v.z, S);
            SFEM_LAUNCHED(ctx);
            if (profile) cudaEventRecord(events[2 * slot], ctx->stream);
            launch_spmv<T, B>(val, v.p, v.q, true);
            if (profile) cudaEventRecord(events[2 * slot + 1], ctx->stream);
        }
        bool mg_now = false;
        if constexpr (MIXED) {
            if (use_mg) {  // x, r and the multigrid's pre-smoothing sweep; r.z comes from the cycle
                mg_now = true;
                auto kern = k_update_node<T, B, PC, MIXED, true>;
                kern<<<resident_grid(ctx, kern, UPD_T, upd_grid), UPD_T, 0, ctx->stream>>>(
                    m->nN, v.x, v.r, mg.lev[0].x, pcur, v.q, mg.lev[0].minv, S, partial);
            }
        }
        if (!mg_now) {
            auto kern = k_update_node<T, B, PC, MIXED>;
            kern<<<resident_grid(ctx, kern, UPD_T, upd_grid), UPD_T, 0, ctx->stream>>>(
                m->nN, v.x, v.r, v.z, pcur, v.q, v.minv, S, partial);
        }
        SFEM_LAUNCHED(ctx);
        if constexpr (MIXED) {
            // FP64 refresh, skipped on the device unless k_update requested it
            // small grid-stride grids: these launches exit at once on most iterations
            const unsigned small = (unsigned)(4 * ctx->num_sms);
            k_fold<<<std::min(vec_grid, small), 256, 0, ctx->stream>>>(nd, x64, (float *)v.x, S);
            k_spmv<double, B, 2><<<std::min(spmv_grid, small), SPMV_T, 0, ctx->stream>>>(
                m->sliceptr, m->col, K->val, m->nN, m->nslices, x64, q64, fixed, S, partial);
            if (mg_now)
                k_refresh<B, PC, true><<<std::min(upd_grid, small), UPD_T, 0, ctx->stream>>>(
                    m->nN, bvec, q64, fixed, r64, (float *)v.r, mg.lev[0].x, mg.lev[0].minv, S, partial);
            else
                k_refresh<B, PC><<<std::min(upd_grid, small), UPD_T, 0, ctx->stream>>>(
                    m->nN, bvec, q64, fixed, r64, (float *)v.r, (float *)v.z, (const float *)v.minv, S, partial);
            ctx->launches += 3;
            if (mg_now) (void)mg_cycle_b<B>((const float *)v.r, (float *)v.z);
        }
    };
    const int per_iter = (MIXED ? 6 : 3) - (fuse_p ? 1 : 0) + (use_mg ? mg_launches : 0);
    if (profile) {
        events.resize(2 * chunk);
        for (auto &e : events) SFEM_CUDA(ctx, cudaEventCreate(&e));
    } else {
        cudaGraph_t g;
        const long long before = ctx->launches;
        SFEM_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < chunk; ++i) enqueue_iter(i);
        SFEM_CUDA(ctx, cudaStreamEndCapture(ctx->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&gexec, g, 0);
        cudaGraphDestroy(g);
        SFEM_CUDA(ctx, e);
        ctx->launches = before;  // counted per graph launch below
    }
    int it_prev = 0;
    while (true) {
        if (profile) {
            for (int i = 0; i < chunk; ++i) enqueue_iter(i);
        } else {
            SFEM_CUDA(ctx, cudaGraphLaunch(gexec, ctx->stream));
            ctx->launches += (long long)per_iter * chunk;
        }
        SFEM_TRY(read_scalars(h));
        if (profile) {
            // only the iterations that ran (kernels after convergence exit at once)
            const int ran = std::min(chunk, std::max(0, h->it - it_prev));
            for (int i = 0; i < ran; ++i) {
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, events[2 * i], events[2 * i + 1]) == cudaSuccess) {
                    ms_spmv += ms;
                    spmv_timed++;
                }
            }
        }
        it_prev = h->it;
        if (h->done) break;
    }
    reliable = h->nrefresh;
    iterations = h->it;
    status = h->status;
    if constexpr (sizeof(T) == 8) {
        if (status != SFEM_SINGULAR) {
            // report the true FP64 residual of the returned iterate
            launch_spmv<double, B>(K->val, v.x, v.q, false);
            k_true_residual<<<vec_grid, UPD_T, 0, ctx->stream>>>(nd, bvec, v.q, fixed, S, partial);
            SFEM_LAUNCHED(ctx);
            SFEM_TRY(read_scalars(h));
        }
    }
    relres = h->bb > 0 ? sqrt(h->rr / h->bb) : 0.0;
    return SFEM_OK;
}

template <int B>
int Solver::solve_b(double *x64) {
    const bool mixed = opts.precision == SFEM_MIXED;
    const bool block = opts.precond != SFEM_PC_JACOBI && B > 1;  // multigrid smooths with the block inverse
    const int mwidth = block ? B * B : B;
    // FP64 preconditioner inverse is built first, then cast for the FP32 path
    double *minv64 = nullptr;
    SFEM_TRY(alloc(&minv64, m->nN * mwidth, "preconditioner"));
    if (block)
        k_precond<double, B, 1><<<(unsigned)sfem_cdiv(m->nN, 256), 256, 0, ctx->stream>>>(
            m->sliceptr, m->col, K->val, m->rowlen, m->nN, fixed, minv64, ctx->d_err);
    else
        k_precond<double, B, 0><<<(unsigned)sfem_cdiv(m->nN, 256), 256, 0, ctx->stream>>>(
            m->sliceptr, m->col, K->val, m->rowlen, m->nN, fixed, minv64, ctx->d_err);
    SFEM_LAUNCHED(ctx);
    SFEM_TRY(sfem_check_device(ctx, "preconditioner"));

    if (!mixed) {
        Vecs<double> v;
        v.x = x64;
        SFEM_TRY(alloc(&v.r, nd, "r"));
        SFEM_TRY(alloc(&v.z, nd, "z"));
        SFEM_TRY(alloc(&v.p, nd, "p"));
        SFEM_TRY(alloc(&v.q, nd, "q"));
        v.minv = minv64;
        SFEM_CUDA(ctx, cudaMemcpyAsync(v.r, r0vec, sizeof(double) * nd, cudaMemcpyDeviceToDevice, ctx->stream));
        if (block)
            k_init<double, B, 1><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, v.r, v.z, v.p, v.minv, S, partial);
        else
            k_init<double, B, 0><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, v.r, v.z, v.p, v.minv, S, partial);
        SFEM_LAUNCHED(ctx);
        SFEM_TRY(block ? cg_loop<double, B, 1, false>(v, nullptr, nullptr, nullptr)
                       : cg_loop<double, B, 0, false>(v, nullptr, nullptr, nullptr));
    } else {
        if (opts.fp32_storage == SFEM_FP32_UPPER && K->sym_state == 0) SFEM_TRY(sfem_sym_build(ctx, K));
        if ((K->sym_state != 1 || opts.fp32_storage == SFEM_FP32_FULL) && !K->val32) {
            const int64_t nv = m->nslabs * 32 * B * B;
            SFEM_TRY(sfem_dalloc(ctx, (void **)&K->val32, sizeof(float) * (nv ? nv : 1), "FP32 K values"));
            k_cast<float><<<(unsigned)sfem_cdiv(nv > 0 ? nv : 1, 256), 256, 0, ctx->stream>>>(nv, K->val, K->val32);
            SFEM_LAUNCHED(ctx);
        }
        Vecs<float> v;
        SFEM_TRY(alloc(&v.x, nd, "x32"));
        SFEM_TRY(alloc(&v.r, nd, "r32"));
        SFEM_TRY(alloc(&v.z, nd, "z32"));
        SFEM_TRY(alloc(&v.p, nd, "p32"));
        SFEM_TRY(alloc(&v.q, nd, "q32"));
        SFEM_TRY(alloc(&v.minv, m->nN * mwidth, "minv32"));
        double *r64 = nullptr, *q64 = nullptr;
        SFEM_TRY(alloc(&r64, nd, "r64"));
        SFEM_TRY(alloc(&q64, nd, "q64"));
        SFEM_CUDA(ctx, cudaMemsetAsync(v.x, 0, sizeof(float) * nd, ctx->stream));
        k_cast<float><<<(unsigned)sfem_cdiv(m->nN * mwidth, 256), 256, 0, ctx->stream>>>(m->nN * mwidth, minv64,
                                                                                           v.minv);
        k_cast<float><<<vec_grid, 256, 0, ctx->stream>>>(nd, r0vec, v.r);
        SFEM_LAUNCHED(ctx);
        SFEM_LAUNCHED(ctx);
        // multigrid: structured meshes with the upper-triangle FP32 K (else block Jacobi)
        use_mg = false;
        if (opts.precond == SFEM_PC_MULTIGRID && K->sym_state == 1 && opts.fp32_storage == SFEM_FP32_UPPER &&
            mg_detect() > 0) {
            if (m->ndim == 2) {
                if constexpr (B <= 2) {
                    SFEM_TRY((mg_build<2, B>(v.minv)));
                    use_mg = true;
                }
            } else {
                if constexpr (B != 2) {
                    SFEM_TRY((mg_build<3, B>(v.minv)));
                    use_mg = true;
                }
            }
        }
        if (use_mg) {
            // first direction: z = V(r), with the pre-smoothing sweep from k_init
            if (block)
                k_init<float, B, 1, true><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, v.r, mg.lev[0].x, v.p,
                                                                              mg.lev[0].minv, S, partial);
            else
                k_init<float, B, 0, true><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, v.r, mg.lev[0].x, v.p,
                                                                              mg.lev[0].minv, S, partial);
            SFEM_LAUNCHED(ctx);
            SFEM_TRY(mg_cycle_b<B>(v.r, v.z));
        } else {
            if (block)
                k_init<float, B, 1><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, v.r, v.z, v.p, v.minv, S, partial);
            else
                k_init<float, B, 0><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, v.r, v.z, v.p, v.minv, S, partial);
            SFEM_LAUNCHED(ctx);
        }
        SFEM_TRY(block ? cg_loop<float, B, 1, true>(v, x64, r64, q64) : cg_loop<float, B, 0, true>(v, x64, r64, q64));
    }
    return SFEM_OK;
}

int Solver::run(const int64_t *fixed_dofs, int64_t nfix, const double *fixed_vals, const double *f, double *u_out,
                int mem_space, sfem_solve_stats *stats, const double *u0) {
    auto t0 = std::chrono::steady_clock::now();
    const int b = m->b;
    const int64_t n = K->n;
    nd = m->nN * b;
    spmv_grid = (unsigned)sfem_cdiv(m->nslices * 32 > 0 ? m->nslices * 32 : 1, SPMV_T);
    upd_grid = (unsigned)sfem_cdiv(m->nN, UPD_T);
    vec_grid = (unsigned)sfem_cdiv(nd, 256);
    const long long launches0 = ctx->launches;

    int64_t *dfix = nullptr;
    double *dvals = nullptr, *fg = nullptr, *fi = nullptr, *x64 = nullptr, *ug = nullptr;
    SFEM_TRY(alloc(&fixed, nd, "fixed mask"));
    SFEM_TRY(alloc(&gfixed, n, "global fixed mask"));
    SFEM_TRY(alloc(&ud, nd, "q_d"));
    SFEM_TRY(alloc(&bvec, nd, "rhs"));
    SFEM_TRY(alloc(&x64, nd, "x"));
    SFEM_TRY(alloc(&ug, n, "u"));
    SFEM_TRY(alloc(&S, 1, "CG scalars"));
    SFEM_TRY(alloc(&partial, 2 * (int64_t)std::max(spmv_grid, std::max(upd_grid, vec_grid)),
                   "partials"));
    SFEM_TRY(alloc(&dfix, nfix, "fixed dofs"));
    SFEM_TRY(alloc(&dvals, nfix, "fixed values"));
    SFEM_TRY(sfem_copy_in(ctx, dfix, fixed_dofs, sizeof(int64_t) * nfix, mem_space));
    SFEM_TRY(sfem_copy_in(ctx, dvals, fixed_vals, sizeof(double) * nfix, mem_space));
    SFEM_CUDA(ctx, cudaMemsetAsync(ud, 0, sizeof(double) * nd, ctx->stream));
    SFEM_CUDA(ctx, cudaMemsetAsync(x64, 0, sizeof(double) * nd, ctx->stream));
    SFEM_CUDA(ctx, cudaMemsetAsync(gfixed, 0, n > 0 ? n : 1, ctx->stream));
    k_mask_inactive<<<vec_grid, 256, 0, ctx->stream>>>(m->rowlen, m->nN, b, fixed);
    SFEM_LAUNCHED(ctx);
    if (nfix > 0) {
        k_fix<<<(unsigned)sfem_cdiv(nfix, 256), 256, 0, ctx->stream>>>(dfix, dvals, nfix, n, m->g2i, fixed, ud, gfixed,
                                                                       ctx->d_err);
        SFEM_LAUNCHED(ctx);
    }
    if (n > 0) {
        k_check_empty<<<(unsigned)sfem_cdiv(n, 256), 256, 0, ctx->stream>>>(n, m->g2i, gfixed, ctx->d_err);
        SFEM_LAUNCHED(ctx);
    }
    if (f) {
        SFEM_TRY(alloc(&fg, n, "f"));
        SFEM_TRY(alloc(&fi, nd, "f internal"));
        SFEM_TRY(sfem_copy_in(ctx, fg, f, sizeof(double) * n, mem_space));
        SFEM_CUDA(ctx, cudaMemsetAsync(fi, 0, sizeof(double) * nd, ctx->stream));
        k_gather_global<<<(unsigned)sfem_cdiv(n, 256), 256, 0, ctx->stream>>>(fg, n, m->g2i, fi);
        SFEM_LAUNCHED(ctx);
    }
    SFEM_TRY(sfem_check_device(ctx, "Dirichlet set-up"));
    // lift: b = f - K q_d on the free DOFs (q64 of the mixed path reuses x64 as scratch here)
    {
        unsigned char *nofix = nullptr;
        SFEM_TRY(alloc(&nofix, nd, "no mask"));
        SFEM_CUDA(ctx, cudaMemsetAsync(nofix, 0, nd, ctx->stream));
        unsigned char *keep = fixed;
        fixed = nofix;
        auto lift = [&](auto kern) {
            kern<<<spmv_grid, SPMV_T, 0, ctx->stream>>>(m->sliceptr, m->col, K->val, m->nN, m->nslices, ud, x64, fixed,
                                                        S, partial);
            SFEM_LAUNCHED(ctx);
        };
        if (b == 1) lift(k_spmv<double, 1, 4>);
        else if (b == 2) lift(k_spmv<double, 2, 4>);
        else lift(k_spmv<double, 3, 4>);
        fixed = keep;
        k_rhs<<<vec_grid, 256, 0, ctx->stream>>>(nd, fi, x64, fixed, bvec);
        SFEM_LAUNCHED(ctx);
        SFEM_CUDA(ctx, cudaMemsetAsync(x64, 0, sizeof(double) * nd, ctx->stream));
    }
    // ||b||^2 and the stopping threshold
    CgScalars hs;
    memset(&hs, 0, sizeof(hs));
    hs.maxit = opts.maxit > 0 ? opts.maxit : 1000000;
    SFEM_CUDA(ctx, cudaMemcpyAsync(S, &hs, sizeof(hs), cudaMemcpyHostToDevice, ctx->stream));
    {
        // rr of b via k_init on a throwaway z/p: reuse the generic reduction
        double *tz = nullptr, *tp = nullptr, *ones = nullptr;
        SFEM_TRY(alloc(&tz, nd, "tmp"));
        SFEM_TRY(alloc(&tp, nd, "tmp"));
        SFEM_TRY(alloc(&ones, nd, "tmp"));
        SFEM_CUDA(ctx, cudaMemsetAsync(ones, 0, sizeof(double) * nd, ctx->stream));
        if (b == 1) k_init<double, 1, 0><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, bvec, tz, tp, ones, S, partial);
        else if (b == 2) k_init<double, 2, 0><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, bvec, tz, tp, ones, S, partial);
        else k_init<double, 3, 0><<<upd_grid, UPD_T, 0, ctx->stream>>>(m->nN, bvec, tz, tp, ones, S, partial);
        SFEM_LAUNCHED(ctx);
        SFEM_TRY(read_scalars(&hs));
    }
    const double bb = hs.rr;
    // warm start: x = x0 on the free DOFs, r0 = b - K x0
    r0vec = bvec;
    double rr0 = bb;
    if (u0) {
        double *ug0 = nullptr, *kx = nullptr;
        SFEM_TRY(alloc(&ug0, n, "initial guess"));
        SFEM_TRY(alloc(&kx, nd, "K x0"));
        SFEM_TRY(alloc(&r0vec, nd, "initial residual"));
        SFEM_TRY(sfem_copy_in(ctx, ug0, u0, sizeof(double) * n, mem_space));
        k_gather_global<<<(unsigned)sfem_cdiv(n > 0 ? n : 1, 256), 256, 0, ctx->stream>>>(ug0, n, m->g2i, x64);
        k_zero_fixed<<<vec_grid, 256, 0, ctx->stream>>>(nd, fixed, x64);
        ctx->launches += 2;
        if (b == 1) launch_spmv<double, 1>(K->val, x64, kx, false);
        else if (b == 2) launch_spmv<double, 2>(K->val, x64, kx, false);
        else launch_spmv<double, 3>(K->val, x64, kx, false);
        k_rhs<<<vec_grid, 256, 0, ctx->stream>>>(nd, bvec, kx, fixed, r0vec);
        k_true_residual<<<vec_grid, UPD_T, 0, ctx->stream>>>(nd, bvec, kx, fixed, S, partial);
        ctx->launches += 2;
        SFEM_TRY(read_scalars(&hs));
        rr0 = hs.rr;
    }
    int64_t n_free = 0;
    {
        std::vector<unsigned char> hf(nd);
        SFEM_CUDA(ctx, cudaMemcpyAsync(hf.data(), fixed, nd, cudaMemcpyDeviceToHost, ctx->stream));
        SFEM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (unsigned char c : hf) n_free += c ? 0 : 1;
    }
    hs.bb = bb;
    hs.tol2 = opts.rtol * opts.rtol * bb;
    hs.delta2 = opts.reliable_delta * opts.reliable_delta;
    hs.rr = rr0;
    hs.rr_ref = rr0;
    hs.it = 0;
    hs.done = bb > 0.0 && n_free > 0 && rr0 > hs.tol2 ? 0 : 1;
    if (hs.done) relres = bb > 0.0 ? sqrt(rr0 / bb) : 0.0;
    hs.status = SFEM_OK;
    SFEM_CUDA(ctx, cudaMemcpyAsync(S, &hs, sizeof(hs), cudaMemcpyHostToDevice, ctx->stream));
    if (!hs.done) {
        if (b == 1) SFEM_TRY(solve_b<1>(x64));
        else if (b == 2) SFEM_TRY(solve_b<2>(x64));
        else SFEM_TRY(solve_b<3>(x64));
    }
    // output: u = q_d + C q_f in global numbering
    k_scatter_out<<<(unsigned)sfem_cdiv(n > 0 ? n : 1, 256), 256, 0, ctx->stream>>>(n, m->g2i, ud, x64, ug);
    SFEM_LAUNCHED(ctx);
    if (nfix > 0) {
        k_fixed_out<<<(unsigned)sfem_cdiv(nfix, 256), 256, 0, ctx->stream>>>(dfix, dvals, nfix, m->g2i, ug);
        SFEM_LAUNCHED(ctx);
    }
    SFEM_TRY(sfem_copy_out(ctx, u_out, ug, sizeof(double) * n, mem_space));
    SFEM_TRY(sfem_check_device(ctx, "solve"));
    auto t1 = std::chrono::steady_clock::now();
    if (stats) {
        stats->status = hs.done && iterations == 0 ? SFEM_OK : status;
        stats->iterations = iterations;
        stats->reliable_updates = reliable;
        stats->relres = relres;
        stats->ms_total = std::chrono::duration<double, std::milli>(t1 - t0).count();
        stats->ms_spmv = ms_spmv;
        stats->spmv_launches = spmv_timed;
        stats->kernel_launches = (int)(ctx->launches - launches0);
        stats->n_free = n_free;
    }
    const int st = hs.done && iterations == 0 ? SFEM_OK : status;
    if (st == SFEM_NOT_CONVERGED)
        return sfem_set_error(ctx, st, "CG reached maxit=%d at relative residual %.3e", opts.maxit, relres);
    if (st == SFEM_SINGULAR) return sfem_set_error(ctx, st, "CG breakdown: K_free is singular or indefinite");
    return st;
}

}  // namespace

extern "C" void sfem_solve_opts_default(sfem_solve_opts *o) {
    if (!o) return;
    o->precision = SFEM_FP64;
    o->precond = SFEM_PC_JACOBI;
    o->rtol = 1e-10;
    o->maxit = 100000;
    o->check_every = 32;
    o->reliable_delta = 0.1;
    o->profile = 0;
    o->fp32_storage = SFEM_FP32_UPPER;
}

extern "C" int sfem_solve_dirichlet(sfem_ctx *ctx, sfem_matrix *K, const int64_t *fixed_dofs, int64_t nfix,
                                    const double *fixed_vals, const double *f, double *u_out, int mem_space,
                                    const sfem_solve_opts *opts, sfem_solve_stats *stats) {
    SfemRange range_("sfem solve");
    if (!ctx || !K || !u_out) return SFEM_BAD_ARG;
    if (nfix < 0 || (nfix > 0 && (!fixed_dofs || !fixed_vals))) return sfem_set_error(ctx, SFEM_BAD_ARG, "bad fixed DOF list");
    cudaSetDevice(ctx->device);
    sfem_solve_opts o;
    sfem_solve_opts_default(&o);
    if (opts) o = *opts;
    if (!(o.rtol >= 0.0) || o.maxit < 0 || (o.precision != SFEM_FP64 && o.precision != SFEM_MIXED) ||
        o.precond < SFEM_PC_JACOBI || o.precond > SFEM_PC_MULTIGRID || !(o.reliable_delta > 0.0) ||
        (o.fp32_storage != SFEM_FP32_UPPER && o.fp32_storage != SFEM_FP32_FULL) ||
        !(o.reliable_delta < 1.0))
        return sfem_set_error(ctx, SFEM_BAD_ARG, "bad solve options");
    if (stats) memset(stats, 0, sizeof(*stats));
    Solver s(ctx, K, o);
    return s.run(fixed_dofs, nfix, fixed_vals, f, u_out, mem_space, stats);
}

namespace {

// x0 = sum_j c[j] * u_j over up to three earlier solutions
__global__ void k_combine3(int64_t n, const double *__restrict__ u0, const double *__restrict__ u1,
                           const double *__restrict__ u2, double c0, double c1, double c2, double *__restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = c0 * u0[i];
    if (u1) v += c1 * u1[i];
    if (u2) v += c2 * u2[i];
    x[i] = v;
}

// Affine weights (sum 1) of the k earlier prescribed-value vectors G[0..k)
// that best reproduce g in the least-squares sense; the displacement is an
// affine function of the prescribed values, so the same weights applied to
// the earlier solutions give the new one exactly when g lies in their span.
int affine_weights(const std::vector<const double *> &G, const double *g, int64_t nfix, double *c) {
    const int k = (int)G.size();
    if (k == 1) {
        c[0] = 1.0;
        return 1;
    }
    // unknowns c_1..c_{k-1}, c_0 = 1 - sum; minimise |sum_j c_j (G_j - G_0) - (g - G_0)|
    double A[2][2] = {{0, 0}, {0, 0}}, r[2] = {0, 0};
    for (int64_t t = 0; t < nfix; ++t) {
        double d[2];
        for (int j = 1; j < k; ++j) d[j - 1] = G[j][t] - G[0][t];
        const double tt = g[t] - G[0][t];
        for (int a = 0; a < k - 1; ++a) {
            r[a] += d[a] * tt;
            for (int b = 0; b < k - 1; ++b) A[a][b] += d[a] * d[b];
        }
    }
    double x[2] = {0, 0};
    if (k == 2) {
        if (!(A[0][0] > 0.0)) return affine_weights({G[0]}, g, nfix, c);
        x[0] = r[0] / A[0][0];
    } else {
        const double det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
        const double scale = A[0][0] * A[1][1];
        if (!(scale > 0.0) || !(fabs(det) > 1e-12 * scale)) return affine_weights({G[0], G[1]}, g, nfix, c);
        x[0] = (r[0] * A[1][1] - r[1] * A[0][1]) / det;
        x[1] = (A[0][0] * r[1] - A[1][0] * r[0]) / det;
    }
    c[0] = 1.0;
    for (int j = 1; j < k; ++j) {
        c[j] = x[j - 1];
        c[0] -= x[j - 1];
    }
    return k;
}

}  // namespace

extern "C" int sfem_solve_increments(sfem_ctx *ctx, sfem_matrix *K, const int64_t *fixed_dofs, int64_t nfix,
                                     const double *fixed_vals, int64_t nsteps, const double *f, double *u_out,
                                     int mem_space, const sfem_solve_opts *opts, int warm_start,
                                     sfem_solve_stats *stats) {
    if (!ctx || !K || !u_out || nsteps < 0) return SFEM_BAD_ARG;
    if (nfix < 0 || (nfix > 0 && (!fixed_dofs || !fixed_vals)))
        return sfem_set_error(ctx, SFEM_BAD_ARG, "bad fixed DOF list");
    if (nsteps == 0) return SFEM_OK;
    cudaSetDevice(ctx->device);
    sfem_solve_opts o;
    sfem_solve_opts_default(&o);
    if (opts) o = *opts;
    SFEM_TRY(sfem_check_ptr(ctx, fixed_dofs, mem_space));
    SFEM_TRY(sfem_check_ptr(ctx, fixed_vals, mem_space));
    SFEM_TRY(sfem_check_ptr(ctx, f, mem_space));
    SFEM_TRY(sfem_check_ptr(ctx, u_out, mem_space));
    const int64_t n = K->n;
    // the prescribed values of every step: on the host for the warm-start
    // weights, on the device for the solves
    std::vector<double> hvals((size_t)(nfix * nsteps));
    if (nfix > 0)
        SFEM_CUDA(ctx, cudaMemcpy(hvals.data(), fixed_vals, sizeof(double) * nfix * nsteps, cudaMemcpyDefault));
    int64_t *dfix = nullptr;
    double *dvals = nullptr, *df = nullptr, *ring = nullptr, *x0 = nullptr;
    int st = SFEM_OK;
    do {
        if ((st = sfem_dalloc(ctx, (void **)&dfix, sizeof(int64_t) * (nfix ? nfix : 1), "fixed dofs"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&dvals, sizeof(double) * (nfix * nsteps ? nfix * nsteps : 1),
                              "fixed values")))
            break;
        if ((st = sfem_dalloc(ctx, (void **)&ring, sizeof(double) * 3 * (n ? n : 1), "earlier solutions"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&x0, sizeof(double) * (n ? n : 1), "initial guess"))) break;
        if ((st = sfem_copy_in(ctx, dfix, fixed_dofs, sizeof(int64_t) * nfix, mem_space))) break;
        if ((st = sfem_copy_in(ctx, dvals, hvals.data(), sizeof(double) * nfix * nsteps, SFEM_MEM_HOST))) break;
        if (f) {
            if ((st = sfem_dalloc(ctx, (void **)&df, sizeof(double) * (n ? n : 1), "f"))) break;
            if ((st = sfem_copy_in(ctx, df, f, sizeof(double) * n, mem_space))) break;
        }
        for (int64_t s = 0; s < nsteps && st == SFEM_OK; ++s) {
            const double *guess = nullptr;
            const int64_t kprev = std::min<int64_t>(s, 3);
            if (warm_start && kprev > 0) {
                std::vector<const double *> G;
                const double *U[3] = {nullptr, nullptr, nullptr};
                for (int64_t j = 0; j < kprev; ++j) {  // most recent first
                    G.push_back(hvals.data() + (s - 1 - j) * nfix);
                    U[j] = ring + ((s - 1 - j) % 3) * n;
                }
                double c[3] = {0, 0, 0};
                const int used = affine_weights(G, hvals.data() + s * nfix, nfix, c);
                k_combine3<<<(unsigned)sfem_cdiv(n > 0 ? n : 1, 256), 256, 0, ctx->stream>>>(
                    n, U[0], used > 1 ? U[1] : nullptr, used > 2 ? U[2] : nullptr, c[0], c[1], c[2], x0);
                SFEM_LAUNCHED(ctx);
                guess = x0;
            }
            double *us = ring + (s % 3) * n;
            sfem_solve_stats one;
            memset(&one, 0, sizeof(one));
            {
                Solver solver(ctx, K, o);
                st = solver.run(dfix, nfix, dvals + s * nfix, df, us, SFEM_MEM_DEVICE, &one, guess);
            }
            if (stats) stats[s] = one;
            if (st != SFEM_OK) break;
            st = sfem_copy_out(ctx, u_out + s * n, us, sizeof(double) * n, mem_space);
        }
        if (st == SFEM_OK) st = sfem_check_device(ctx, "load increments");
    } while (0);
    void *bufs[] = {dfix, dvals, df, ring, x0};
    for (void *p : bufs) sfem_dfree(ctx, p);
    return st;
}
