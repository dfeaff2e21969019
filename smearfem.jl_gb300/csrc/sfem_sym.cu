// Upper-triangle ("symmetric") FP32 copy of K for the mixed-precision solver.
//
// K is assembled bitwise symmetric (block(r,c) == block(c,r)^T), so the FP32
// inner CG only needs, per node row r,
//   upper part: the blocks (r, c) with c >= r, values stored, sliced-ELL:
//       colU[slabU*32 + lane], valU in the lane-contiguous block layout
//       (v32_at: each lane's block is one float4 + float4 + float for b = 3)
//   lower part: for every neighbour c < r, where block (c, r) sits in c's
//       upper part, as int2 {slabU*32 + lane of that block, c}:
//       lo[slabL*32 + lane]   ({-1, 0} = padding).  Both are in one 8-byte
//       load, so the value and x loads issue together (no dependent lookup).
// y_r = sum_{c>=r} A_rc x_c + sum_{c<r} A_cr^T x_c, computed by one lane per
// row in a fixed order, so the result is deterministic.  Per 27-neighbour row
// this reads 14 value blocks instead of 27: 612 B instead of 1,080 B in FP32.
#include <limits.h>

#include "sfem_internal.cuh"

namespace {

__device__ __forceinline__ int row_kdiag(const int *__restrict__ col, int64_t slab0, int lane, int len, int r) {
    int k = 0;
    while (k < len && col[(slab0 + k) * 32 + lane] < r) ++k;
    return k;
}

__global__ void k_sym_len(const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                          const int *__restrict__ rowlen, int64_t nN, int *__restrict__ lenU,
                          int *__restrict__ lenL) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nN) return;
    const int len = rowlen[r];
    const int kd = row_kdiag(col, sliceptr[r >> 5], (int)(r & 31), len, (int)r);
    lenU[r] = len - kd;
    lenL[r] = kd;
}

__global__ void k_sym_width(const int *__restrict__ lenU, const int *__restrict__ lenL, int64_t nN, int64_t nslices,
                            int64_t *__restrict__ wU, int64_t *__restrict__ wL) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = t >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;  // whole warps
    const int64_t r = s * 32 + lane;
    int u = r < nN ? lenU[r] : 0, l = r < nN ? lenL[r] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        u = max(u, __shfl_xor_sync(0xffffffffu, u, o));
        l = max(l, __shfl_xor_sync(0xffffffffu, l, o));
    }
    if (lane == 0) {
        wU[s] = u;
        wL[s] = l;
    }
}

// Upper part: columns (when colU != nullptr) and FP32 values from the FP64 K.
// kdiag: each row's diagonal position (k_sym_len's lenL) when it is at hand,
// else it is searched.
template <int B>
__global__ void k_sym_fill_upper(const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                                 const double *__restrict__ val, const int *__restrict__ rowlen, int64_t nN,
                                 int64_t nslices, const int64_t *__restrict__ sptrU, int *__restrict__ colU,
                                 float *__restrict__ valU, const int *__restrict__ kdiag) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = t >> 5;
    const int lane = (int)(t & 31);
    if (s >= nslices) return;
    const int64_t r = s * 32 + lane;
    const int64_t slab0 = sliceptr[s], u0 = sptrU[s], wU = sptrU[s + 1] - u0;
    const int len = r < nN ? rowlen[r] : 0;
    const int kd = r < nN ? (kdiag ? kdiag[r] : row_kdiag(col, slab0, lane, len, (int)r)) : 0;
    for (int64_t k = 0; k < wU; ++k) {
        const int64_t su = u0 + k;
        const bool live = k < len - kd;
        if (colU) colU[su * 32 + lane] = live ? col[(slab0 + kd + k) * 32 + lane] : (r < nN ? (int)r : 0);
#pragma unroll
        for (int e = 0; e < B * B; ++e)
            valU[v32_at<B>(su, lane, e)] = live ? (float)val[((slab0 + kd + k) * B * B + e) * 32 + lane] : 0.0f;
    }
}

// Lower part: for neighbour c < r, the position of block (c, r) in valU.
template <int B>
__global__ void k_sym_fill_lower(const int64_t *__restrict__ sliceptr, const int *__restrict__ col,
                                 const int *__restrict__ rowlen, int64_t nN, int64_t nslices,
                                 const int64_t *__restrict__ sptrU, const int64_t *__restrict__ sptrL,
                                 int2 *__restrict__ lo, int *__restrict__ bad, const int *__restrict__ kdiag) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = t >> 5;
    const int lane = (int)(t & 31);
    if (s >= nslices) return;
    const int64_t r = s * 32 + lane;
    const int64_t slab0 = sliceptr[s], l0 = sptrL[s], wL = sptrL[s + 1] - l0;
    const int kd = r < nN ? kdiag[r] : 0;
    for (int64_t k = 0; k < wL; ++k) {
        int2 ent = make_int2(-1, 0);
        if (k < kd) {
            const int c = col[(slab0 + k) * 32 + lane];
            const int64_t cs0 = sliceptr[c >> 5];
            const int cl = c & 31, clen = rowlen[c];
            const int ckd = kdiag[c];
            int lo_i = ckd, hi_i = clen - 1, pos = -1;  // r > c lies in c's upper part
            while (lo_i <= hi_i) {
                const int mid = (lo_i + hi_i) >> 1;
                const int v = col[(cs0 + mid) * 32 + cl];
                if (v == r) {
                    pos = mid;
                    break;
                }
                if (v < r) lo_i = mid + 1;
                else hi_i = mid - 1;
            }
            const int64_t off = (sptrU[c >> 5] + (pos - ckd)) * 32 + cl;  // slab and lane of block (c, r)
            if (pos < 0 || off > (int64_t)INT_MAX) {
                atomicExch(bad, 1);
            } else {
                ent = make_int2((int)off, c);
            }
        }
        lo[(l0 + k) * 32 + lane] = ent;
    }
}

template <int B>
void launch_fill_upper(sfem_ctx *ctx, const sfem_matrix *K, bool cols, const int *kdiag = nullptr) {
    const sfem_mesh *m = K->mesh;
    const unsigned grid = (unsigned)sfem_cdiv(m->nslices * 32 > 0 ? m->nslices * 32 : 1, 128);
    k_sym_fill_upper<B><<<grid, 128, 0, ctx->stream>>>(m->sliceptr, m->col, K->val, m->rowlen, m->nN, m->nslices,
                                                       K->sptrU, cols ? K->colU : nullptr, K->valU, kdiag);
    SFEM_LAUNCHED(ctx);
}

}  // namespace

void sfem_sym_free(sfem_ctx *ctx, sfem_matrix *K) {
    void *bufs[] = {K->sptrU, K->sptrL, K->colU, K->lo, K->valU};
    for (void *p : bufs) sfem_dfree(ctx, p);
    K->sptrU = K->sptrL = nullptr;
    K->colU = nullptr;
    K->lo = nullptr;
    K->valU = nullptr;
    K->sym_state = 0;
}

int sfem_sym_refresh_values(sfem_ctx *ctx, sfem_matrix *K) {
    if (K->sym_state != 1) return SFEM_OK;
    const int b = K->mesh->b;
    if (b == 1) launch_fill_upper<1>(ctx, K, false);
    else if (b == 2) launch_fill_upper<2>(ctx, K, false);
    else launch_fill_upper<3>(ctx, K, false);
    return sfem_cuda_status(ctx, cudaGetLastError(), "symmetric value refresh");
}

int sfem_sym_build(sfem_ctx *ctx, sfem_matrix *K) {
    if (K->sym_state != 0) return SFEM_OK;
    sfem_mesh *m = K->mesh;
    const int64_t nN = m->nN, nsl = m->nslices;
    const int b = m->b;
    if (m->nslabs * 32 * (int64_t)b * b > (int64_t)INT_MAX) {
        K->sym_state = -1;  // int32 value offsets would overflow: the full FP32 SpMV is used instead
        return SFEM_OK;
    }
    int *lenU = nullptr, *lenL = nullptr, *bad = nullptr;
    int64_t *wU = nullptr, *wL = nullptr;
    int st = SFEM_OK;
    do {
        if ((st = sfem_dalloc(ctx, (void **)&lenU, sizeof(int) * nN, "sym lenU"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&lenL, sizeof(int) * nN, "sym lenL"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&wU, sizeof(int64_t) * nsl, "sym wU"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&wL, sizeof(int64_t) * nsl, "sym wL"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&bad, sizeof(int), "sym flag"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&K->sptrU, sizeof(int64_t) * (nsl + 1), "sym sptrU"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&K->sptrL, sizeof(int64_t) * (nsl + 1), "sym sptrL"))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream), "memset"))) break;
        k_sym_len<<<(unsigned)sfem_cdiv(nN, 256), 256, 0, ctx->stream>>>(m->sliceptr, m->col, m->rowlen, nN, lenU, lenL);
        SFEM_LAUNCHED(ctx);
        k_sym_width<<<(unsigned)sfem_cdiv(nsl * 32, 256), 256, 0, ctx->stream>>>(lenU, lenL, nN, nsl, wU, wL);
        SFEM_LAUNCHED(ctx);
        if ((st = sfem_scan_i64(ctx, wU, K->sptrU, nsl))) break;
        if ((st = sfem_scan_i64(ctx, wL, K->sptrL, nsl))) break;
        int64_t *h = (int64_t *)ctx->h_small;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(h, K->sptrU + nsl, 8, cudaMemcpyDeviceToHost, ctx->stream),
                                   "memcpy")))
            break;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(h + 1, K->sptrL + nsl, 8, cudaMemcpyDeviceToHost, ctx->stream),
                                   "memcpy")))
            break;
        if ((st = sfem_check_device(ctx, "symmetric pattern"))) break;
        K->nslabsU = h[0];
        K->nslabsL = h[1];
        if ((st = sfem_dalloc(ctx, (void **)&K->colU, sizeof(int) * (K->nslabsU * 32 + 1), "sym colU"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&K->lo, sizeof(int2) * (K->nslabsL * 32 + 1), "sym lower"))) break;
        if ((st = sfem_dalloc(ctx, (void **)&K->valU, sizeof(float) * (K->nslabsU * 32 * b * b + 1), "sym values")))
            break;
        K->sym_state = 1;
        if (b == 1) launch_fill_upper<1>(ctx, K, true, lenL);
        else if (b == 2) launch_fill_upper<2>(ctx, K, true, lenL);
        else launch_fill_upper<3>(ctx, K, true, lenL);
        {
            const unsigned g = (unsigned)sfem_cdiv(nsl * 32 > 0 ? nsl * 32 : 1, 128);
            if (b == 1)
                k_sym_fill_lower<1><<<g, 128, 0, ctx->stream>>>(m->sliceptr, m->col, m->rowlen, nN, nsl, K->sptrU,
                                                               K->sptrL, K->lo, bad, lenL);
            else if (b == 2)
                k_sym_fill_lower<2><<<g, 128, 0, ctx->stream>>>(m->sliceptr, m->col, m->rowlen, nN, nsl, K->sptrU,
                                                               K->sptrL, K->lo, bad, lenL);
            else
                k_sym_fill_lower<3><<<g, 128, 0, ctx->stream>>>(m->sliceptr, m->col, m->rowlen, nN, nsl, K->sptrU,
                                                               K->sptrL, K->lo, bad, lenL);
            SFEM_LAUNCHED(ctx);
        }
        int *hb = (int *)ctx->h_small;
        if ((st = sfem_cuda_status(ctx, cudaMemcpyAsync(hb, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
                                   "memcpy")))
            break;
        if ((st = sfem_check_device(ctx, "symmetric fill"))) break;
        if (*hb) {  // a lower entry was not found or did not fit: use the full FP32 copy
            sfem_sym_free(ctx, K);
            K->sym_state = -1;
        }
    } while (0);
    sfem_dfree(ctx, lenU);
    sfem_dfree(ctx, lenL);
    sfem_dfree(ctx, wU);
    sfem_dfree(ctx, wL);
    sfem_dfree(ctx, bad);
    if (st != SFEM_OK) {
        sfem_sym_free(ctx, K);
        K->sym_state = -1;
    }
    return st;
}
