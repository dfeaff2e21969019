// Context, error reporting, copies, device scans and the host-side helpers
// gaussian_quadrature / basis_function of the C ABI.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "sfem_internal.cuh"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

int sfem_set_error(sfem_ctx *ctx, int code, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return code;
}

int sfem_cuda_status(sfem_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return SFEM_OK;
    cudaGetLastError();  // clear non-sticky errors
    return sfem_set_error(ctx, e == cudaErrorMemoryAllocation ? SFEM_OOM : SFEM_CUDA_ERROR,
                          "%s: %s", what, cudaGetErrorString(e));
}

static const char *status_name(int code) {
    switch (code) {
        case SFEM_OK: return "ok";
        case SFEM_BAD_ARG: return "bad argument";
        case SFEM_BAD_INDEX: return "index out of range";
        case SFEM_SINGULAR_JACOBIAN: return "singular element Jacobian (det J == 0)";
        case SFEM_OOM: return "out of device memory";
        case SFEM_NOT_CONVERGED: return "not converged";
        case SFEM_CUDA_ERROR: return "CUDA error";
        case SFEM_SINGULAR: return "singular system";
        case SFEM_UNSUPPORTED: return "unsupported";
    }
    return "unknown";
}

int sfem_check_device(sfem_ctx *ctx, const char *where) {
    SFEM_CUDA(ctx, cudaGetLastError());
    SFEM_CUDA(ctx, cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(DevErr), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    SFEM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    DevErr e = *ctx->h_err;
    if (e.code != 0) {
        SFEM_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(DevErr), ctx->stream));
        SFEM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return sfem_set_error(ctx, e.code, "%s: %s at index %lld (aux %d)", where,
                              status_name(e.code), e.index, e.aux);
    }
    return SFEM_OK;
}

// ---------------------------------------------------------------------------
// memory
// ---------------------------------------------------------------------------

int sfem_dalloc(sfem_ctx *ctx, void **p, size_t bytes, const char *what) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return sfem_set_error(ctx, SFEM_OOM, "allocating %zu bytes for %s: %s", bytes, what,
                              cudaGetErrorString(e));
    }
    return SFEM_OK;
}

void sfem_dfree(sfem_ctx *ctx, void *p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

int sfem_check_ptr(sfem_ctx *ctx, const void *p, int mem_space) {
    if (!p) return SFEM_OK;
    if (mem_space != SFEM_MEM_HOST && mem_space != SFEM_MEM_DEVICE)
        return sfem_set_error(ctx, SFEM_BAD_ARG, "mem_space must be SFEM_MEM_HOST or SFEM_MEM_DEVICE");
    if (mem_space == SFEM_MEM_DEVICE) {
        cudaPointerAttributes a;
        cudaError_t e = cudaPointerGetAttributes(&a, p);
        if (e != cudaSuccess || (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return sfem_set_error(ctx, SFEM_BAD_ARG, "pointer %p is not device memory", p);
        }
    }
    return SFEM_OK;
}

// Inputs are always copied into library-owned device buffers, so no kernel
// ever dereferences a caller pointer.
int sfem_copy_in(sfem_ctx *ctx, void *dst, const void *src, size_t bytes, int mem_space) {
    if (bytes == 0) return SFEM_OK;
    SFEM_TRY(sfem_check_ptr(ctx, src, mem_space));
    SFEM_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream));
    return SFEM_OK;
}

int sfem_copy_out(sfem_ctx *ctx, void *dst, const void *src, size_t bytes, int mem_space) {
    if (bytes == 0) return SFEM_OK;
    SFEM_TRY(sfem_check_ptr(ctx, dst, mem_space));
    SFEM_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream));
    return SFEM_OK;
}

// ---------------------------------------------------------------------------
// exclusive scan (int32/int64 -> int64, total appended)
// ---------------------------------------------------------------------------

namespace {
constexpr int SCAN_T = 512;
constexpr int SCAN_I = 8;
constexpr int SCAN_TILE = SCAN_T * SCAN_I;

template <typename Tin>
__global__ void __launch_bounds__(SCAN_T) k_scan_tile(const Tin *__restrict__ in, int64_t *__restrict__ out,
                                                      int64_t n, int64_t *__restrict__ tile_sums) {
    __shared__ int64_t warp_tot[SCAN_T / 32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t v[SCAN_I];
    int64_t tsum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_I; ++i) {
        int64_t idx = base + (int64_t)threadIdx.x * SCAN_I + i;
        v[i] = idx < n ? (int64_t)in[idx] : 0;
        tsum += v[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < SCAN_T / 32 ? warp_tot[lane] : 0;
        int64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < SCAN_T / 32) warp_tot[lane] = wi - w;  // exclusive warp offsets
        if (lane == SCAN_T / 32 - 1 && tile_sums) tile_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    int64_t run = warp_tot[warp] + incl - tsum;
#pragma unroll
    for (int i = 0; i < SCAN_I; ++i) {
        int64_t idx = base + (int64_t)threadIdx.x * SCAN_I + i;
        if (idx < n) out[idx] = run;
        run += v[i];
    }
}

__global__ void k_scan_add(int64_t *__restrict__ out, int64_t n, const int64_t *__restrict__ offs) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n) out[idx] += offs[idx / SCAN_TILE];
}

__global__ void k_scan_total(const int64_t *__restrict__ out, const int64_t *__restrict__ in_last_src,
                             int64_t n, int64_t *__restrict__ dst, int is32, const void *in) {
    // out[n] = out[n-1] + in[n-1]
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int64_t last = n > 0 ? (is32 ? (int64_t)((const int *)in)[n - 1] : ((const int64_t *)in)[n - 1]) : 0;
        dst[0] = n > 0 ? out[n - 1] + last : 0;
    }
    (void)in_last_src;
}

template <typename Tin>
int scan_impl(sfem_ctx *ctx, const Tin *in, int64_t *out, int64_t n, int is32) {
    if (n > 0) {
        int64_t tiles = sfem_cdiv(n, SCAN_TILE);
        if (tiles == 1) {
            k_scan_tile<Tin><<<1, SCAN_T, 0, ctx->stream>>>(in, out, n, nullptr);
            SFEM_LAUNCHED(ctx);
        } else {
            int64_t *sums = nullptr, *offs = nullptr;
            SFEM_TRY(sfem_dalloc(ctx, (void **)&sums, sizeof(int64_t) * tiles, "scan tile sums"));
            SFEM_TRY(sfem_dalloc(ctx, (void **)&offs, sizeof(int64_t) * (tiles + 1), "scan offsets"));
            k_scan_tile<Tin><<<(unsigned)tiles, SCAN_T, 0, ctx->stream>>>(in, out, n, sums);
            SFEM_LAUNCHED(ctx);
            SFEM_TRY(scan_impl<int64_t>(ctx, sums, offs, tiles, 0));
            k_scan_add<<<(unsigned)sfem_cdiv(n, 256), 256, 0, ctx->stream>>>(out, n, offs);
            SFEM_LAUNCHED(ctx);
            sfem_dfree(ctx, sums);
            sfem_dfree(ctx, offs);
        }
    }
    k_scan_total<<<1, 32, 0, ctx->stream>>>(out, nullptr, n, out + n, is32, in);
    SFEM_LAUNCHED(ctx);
    return sfem_cuda_status(ctx, cudaGetLastError(), "scan");
}
}  // namespace

int sfem_scan_i32(sfem_ctx *ctx, const int *in, int64_t *out, int64_t n) {
    return scan_impl<int>(ctx, in, out, n, 1);
}
int sfem_scan_i64(sfem_ctx *ctx, const int64_t *in, int64_t *out, int64_t n) {
    return scan_impl<int64_t>(ctx, in, out, n, 0);
}

// ---------------------------------------------------------------------------
// C ABI: context
// ---------------------------------------------------------------------------

extern "C" int sfem_ctx_create(int device, sfem_ctx **out) {
    if (!out) return SFEM_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return SFEM_CUDA_ERROR;
    }
    if (device < 0 || device >= ndev) return SFEM_BAD_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SFEM_CUDA_ERROR;
    sfem_ctx *c = new sfem_ctx();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_err, sizeof(DevErr)) != cudaSuccess ||
        cudaMallocHost(&c->h_err, sizeof(DevErr)) != cudaSuccess ||
        cudaMallocHost(&c->h_small, 4096) != cudaSuccess ||
        cudaMemset(c->d_err, 0, sizeof(DevErr)) != cudaSuccess) {
        cudaGetLastError();
        sfem_ctx_destroy(c);
        return SFEM_CUDA_ERROR;
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (c->num_sms < 1) c->num_sms = 1;
    // Keep freed pool memory for reuse by this process (large per-solve buffers).
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    cudaGetLastError();
    *out = c;
    return SFEM_OK;
}

extern "C" int sfem_ctx_destroy(sfem_ctx *ctx) {
    if (!ctx) return SFEM_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    cudaGetLastError();
    delete ctx;
    return SFEM_OK;
}

extern "C" const char *sfem_last_error(const sfem_ctx *ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" int sfem_ctx_synchronize(sfem_ctx *ctx) {
    if (!ctx) return SFEM_BAD_ARG;
    return sfem_cuda_status(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
}

extern "C" const char *sfem_version(void) { return SFEM_VERSION; }

extern "C" void *sfem_ctx_stream(sfem_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int64_t sfem_ctx_kernel_launches(const sfem_ctx *ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------------------
// C ABI: host helpers, src/fem.jl:21-31 and :48-114 (same expressions)
// ---------------------------------------------------------------------------

extern "C" int sfem_gaussian_quadrature(double a, double b, int nGaussPoints, double *xi, double *w) {
    if (!xi || !w) return SFEM_BAD_ARG;
    if (nGaussPoints == 2) {
        xi[0] = -(b - a) / (2 * sqrt(3.0)) + (b + a) / 2;
        xi[1] = (b - a) / (2 * sqrt(3.0)) + (b + a) / 2;
        w[0] = (b - a) / 2;
        w[1] = (b - a) / 2;
        return SFEM_OK;
    }
    if (nGaussPoints == 3) {
        xi[0] = -(b - a) / (2 * sqrt(5.0 / 3.0)) + (b + a) / 2;
        xi[1] = 0.0;
        xi[2] = (b - a) / (2 * sqrt(5.0 / 3.0)) + (b + a) / 2;
        w[0] = (b - a) / 2 * 5 / 9;
        w[1] = (b - a) / 2 * 8 / 9;
        w[2] = (b - a) / 2 * 5 / 9;
        return SFEM_OK;
    }
    return SFEM_BAD_ARG;
}

extern "C" int sfem_basis_function(int ndim, int function_class, double x, double y, double z,
                                   double *N, double *dN) {
    if (!N || !dN) return SFEM_BAD_ARG;
    if (function_class == SFEM_Q1 && ndim == 3) {
        const double n[8] = {(1 - x) * (1 - y) * (1 - z) / 8, (1 + x) * (1 - y) * (1 - z) / 8,
                             (1 + x) * (1 + y) * (1 - z) / 8, (1 - x) * (1 + y) * (1 - z) / 8,
                             (1 - x) * (1 - y) * (1 + z) / 8, (1 + x) * (1 - y) * (1 + z) / 8,
                             (1 + x) * (1 + y) * (1 + z) / 8, (1 - x) * (1 + y) * (1 + z) / 8};
        const double dx[8] = {-(1 - y) * (1 - z) / 8, (1 - y) * (1 - z) / 8, (1 + y) * (1 - z) / 8,
                              -(1 + y) * (1 - z) / 8, -(1 - y) * (1 + z) / 8, (1 - y) * (1 + z) / 8,
                              (1 + y) * (1 + z) / 8, -(1 + y) * (1 + z) / 8};
        const double dy[8] = {-(1 - x) * (1 - z) / 8, -(1 + x) * (1 - z) / 8, (1 + x) * (1 - z) / 8,
                              (1 - x) * (1 - z) / 8, -(1 - x) * (1 + z) / 8, -(1 + x) * (1 + z) / 8,
                              (1 + x) * (1 + z) / 8, (1 - x) * (1 + z) / 8};
        const double dz[8] = {-(1 - x) * (1 - y) / 8, -(1 + x) * (1 - y) / 8, -(1 + x) * (1 + y) / 8,
                              -(1 - x) * (1 + y) / 8, (1 - x) * (1 - y) / 8, (1 + x) * (1 - y) / 8,
                              (1 + x) * (1 + y) / 8, (1 - x) * (1 + y) / 8};
        for (int a = 0; a < 8; ++a) {
            N[a] = n[a];
            dN[a] = dx[a];
            dN[8 + a] = dy[a];
            dN[16 + a] = dz[a];
        }
        return SFEM_OK;
    }
    if (function_class == SFEM_Q1 && ndim == 2) {
        const double n[4] = {(1 - x) * (1 - y) / 4, (x + 1) * (1 - y) / 4, (1 + x) * (y + 1) / 4,
                             (1 - x) * (1 + y) / 4};
        const double dx[4] = {-(1 - y) / 4, (1 - y) / 4, (y + 1) / 4, -(1 + y) / 4};
        const double dy[4] = {-(1 - x) / 4, -(x + 1) / 4, (1 + x) / 4, (1 - x) / 4};
        for (int a = 0; a < 4; ++a) {
            N[a] = n[a];
            dN[a] = dx[a];
            dN[4 + a] = dy[a];
        }
        return SFEM_OK;
    }
    if (function_class == SFEM_Q1 && ndim == 1) {
        N[0] = 0.5 - 0.5 * x;
        N[1] = 0.5 + 0.5 * x;
        dN[0] = -0.5;
        dN[1] = 0.5;
        return SFEM_OK;
    }
    if (function_class == SFEM_Q2 && ndim == 2) {
        const double n[9] = {(1 - x) * x * (1 - y) * y / 4,
                             -x * (1 + x) * (1 - y) * y / 4,
                             x * (1 + x) * y * (1 + y) / 4,
                             -(1 - x) * x * y * (1 + y) / 4,
                             -(1 - x) * (1 + x) * (1 - y) * y / 2,
                             x * (1 + x) * (1 - y) * (1 + y) / 2,
                             (1 - x) * (1 + x) * y * (1 + y) / 2,
                             -(1 - x) * x * (1 - y) * (1 + y) / 2,
                             (1 - x) * (1 + x) * (1 - y) * (1 + y)};
        const double dx[9] = {(1 - 2 * x) * (1 - y) * y / 4,
                              -(1 + 2 * x) * (1 - y) * y / 4,
                              (1 + 2 * x) * y * (1 + y) / 4,
                              -(1 - 2 * x) * y * (1 + y) / 4,
                              x * (1 - y) * y,
                              (1 + 2 * x) * (1 - y) * (1 + y) / 2,
                              -x * y * (1 + y),
                              -(1 - 2 * x) * (1 - y) * (1 + y) / 2,
                              -2 * x * (1 - y) * (1 + y)};
        const double dy[9] = {(1 - x) * x * (1 - 2 * y) / 4,
                              -x * (1 + x) * (1 - 2 * y) / 4,
                              x * (1 + x) * (1 + 2 * y) / 4,
                              -(1 - x) * x * (1 + 2 * y) / 4,
                              -(1 - x) * (1 + x) * (1 - 2 * y) / 2,
                              -x * (1 + x) * y,
                              (1 - x) * (1 + x) * (1 + 2 * y) / 2,
                              (1 - x) * x * y,
                              -(1 - x) * (1 + x) * 2 * y};
        for (int a = 0; a < 9; ++a) {
            N[a] = n[a];
            dN[a] = dx[a];
            dN[9 + a] = dy[a];
        }
        return SFEM_OK;
    }
    return SFEM_BAD_ARG;
}
