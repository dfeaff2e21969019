// The reference's structured mesh and its cylinder mapping, generated on the
// GPU so a driver can build its inputs where they are used:
//   sfem_meshgrid        examples/vector3D.jl:10-130 (nodes x fastest, then y,
//                        then z; Q1 connectivity; interleaved ID; the top and
//                        bottom surface quads, or edges in 2D)
//   sfem_inflate_sphere  src/PostProcess.jl:30-44
// Coordinates follow the rounding of a linspace: step = (x1 - x0) / ne,
// x_i = i * step + x0 with the last point set to x1 exactly, each operation
// rounded on its own (no fused multiply-add), so the boundary planes hold
// their nodes exactly -- the reference's boundary selection compares
// coordinates with ==.
#include "sfem_internal.cuh"

namespace {

__device__ __forceinline__ double grid_coord(double a, double b, int64_t ne, int64_t i) {
    if (i == ne) return b;
    const double step = __ddiv_rn(__dadd_rn(b, -a), (double)ne);
    return __dadd_rn(__dmul_rn((double)i, step), a);
}

__global__ void k_grid_nodes(int ndim, int64_t ne, double x0, double x1, double y0, double y1, double z0, double z1,
                             int64_t nN, double *__restrict__ X, int64_t *__restrict__ ID) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    const int64_t n1 = ne + 1;
    const int64_t i = m % n1, j = (m / n1) % n1, k = m / (n1 * n1);
    if (X) {
        X[m * ndim + 0] = grid_coord(x0, x1, ne, i);
        X[m * ndim + 1] = grid_coord(y0, y1, ne, j);
        if (ndim == 3) X[m * ndim + 2] = grid_coord(z0, z1, ne, k);
    }
    if (ID)
        for (int l = 0; l < ndim; ++l) ID[m + l * nN] = ndim * m + l + 1;  // ID[m, l], column-major
}

// Element n (0-based, x fastest) and its surface entries; all arrays
// column-major with 1-based node numbers, as the reference's Julia matrices.
__global__ void k_grid_elems(int ndim, int64_t ne, int64_t *__restrict__ IEN, int64_t *__restrict__ top,
                             int64_t *__restrict__ btm) {
    const int64_t nEl = ndim == 2 ? ne * ne : ne * ne * ne;
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nEl) return;
    const int64_t n1 = ne + 1, p = n1 * n1;
    const int64_t i = n % ne, j = (n / ne) % ne, k = n / (ne * ne);
    int64_t c[8];
    if (ndim == 2) {
        c[0] = j * n1 + i + 1;
        c[1] = j * n1 + i + 2;
        c[2] = (j + 1) * n1 + i + 2;
        c[3] = (j + 1) * n1 + i + 1;
        const int64_t nf = ne;
        if (IEN)
            for (int a = 0; a < 4; ++a) IEN[n + a * nEl] = c[a];
        if (j == 0) {  // `if j == 1` (bottom) ... `elseif j == ne` (top): ne = 1 fills only the bottom
            if (btm) {
                btm[i + 0 * nf] = c[0];
                btm[i + 1 * nf] = c[1];
            }
        } else if (j == ne - 1) {
            if (top) {
                top[i + 0 * nf] = c[3];
                top[i + 1 * nf] = c[2];
            }
        }
        return;
    }
    const int64_t base = k * p + j * n1 + i + 1;
    c[0] = base;
    c[1] = base + 1;
    c[2] = base + n1 + 1;
    c[3] = base + n1;
    c[4] = base + p;
    c[5] = base + p + 1;
    c[6] = base + p + n1 + 1;
    c[7] = base + p + n1;
    if (IEN)
        for (int a = 0; a < 8; ++a) IEN[n + a * nEl] = c[a];
    const int64_t nf = ne * ne, f = j * ne + i;
    if (k == 0) {
        if (btm)
            for (int a = 0; a < 4; ++a) btm[f + a * nf] = c[a];
    } else if (k == ne - 1) {
        if (top)
            for (int a = 0; a < 4; ++a) top[f + a * nf] = c[4 + a];
    }
}

__global__ void k_inflate(double *__restrict__ X, int ndim, int64_t nN, double xc, double yc) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    double *p = X + m * ndim;
    const double dx = __dadd_rn(p[0], -xc), dy = __dadd_rn(p[1], -yc);
    const double scale = fmax(fabs(dx), fabs(dy));
    if (scale == 0.0) {  // Julia's `scale ≈ 0.` (rtol sqrt(eps), atol 0) holds only for exact 0
        p[0] = 0.0;
        p[1] = 0.0;
        return;
    }
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    p[0] = __ddiv_rn(__dmul_rn(scale, dx), r);
    p[1] = __ddiv_rn(__dmul_rn(scale, dy), r);
}

unsigned grid_for(int64_t n) { return (unsigned)sfem_cdiv(n > 0 ? n : 1, 256); }

}  // namespace

extern "C" int sfem_meshgrid(sfem_ctx *ctx, double x0, double x1, double y0, double y1, double z0, double z1,
                             int64_t ne, int ndim, double *NodeList, int64_t *IEN, int64_t *ID, int64_t *IEN_top,
                             int64_t *IEN_btm, int mem_space) {
    if (!ctx) return SFEM_BAD_ARG;
    if ((ndim != 2 && ndim != 3) || ne < 1)
        return sfem_set_error(ctx, SFEM_BAD_ARG, "meshgrid needs ndim 2 or 3 and ne >= 1");
    const int64_t n1 = ne + 1;
    const int64_t nN = ndim == 2 ? n1 * n1 : n1 * n1 * n1;
    const int64_t nEl = ndim == 2 ? ne * ne : ne * ne * ne;
    const int64_t nF = ndim == 2 ? ne : ne * ne, nenF = ndim == 2 ? 2 : 4;
    if (nN > (int64_t)1 << 31) return sfem_set_error(ctx, SFEM_BAD_ARG, "mesh too large for int32 node ids");
    void *outs[5] = {NodeList, IEN, ID, IEN_top, IEN_btm};
    for (void *p : outs) SFEM_TRY(sfem_check_ptr(ctx, p, mem_space));
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        cudaGetLastError();
        return sfem_set_error(ctx, SFEM_CUDA_ERROR, "cudaSetDevice(%d) failed", ctx->device);
    }
    const bool dev = mem_space == SFEM_MEM_DEVICE;
    double *X = dev ? NodeList : nullptr;
    int64_t *ien = dev ? IEN : nullptr, *id = dev ? ID : nullptr, *top = dev ? IEN_top : nullptr,
            *btm = dev ? IEN_btm : nullptr;
    int st = SFEM_OK;
    do {
        if (!dev) {  // staging buffers for host outputs
            if (NodeList && (st = sfem_dalloc(ctx, (void **)&X, sizeof(double) * ndim * nN, "grid nodes"))) break;
            if (IEN && (st = sfem_dalloc(ctx, (void **)&ien, sizeof(int64_t) * (1 << ndim) * nEl, "grid IEN"))) break;
            if (ID && (st = sfem_dalloc(ctx, (void **)&id, sizeof(int64_t) * ndim * nN, "grid ID"))) break;
            if (IEN_top && (st = sfem_dalloc(ctx, (void **)&top, sizeof(int64_t) * nenF * nF, "grid top"))) break;
            if (IEN_btm && (st = sfem_dalloc(ctx, (void **)&btm, sizeof(int64_t) * nenF * nF, "grid bottom"))) break;
        }
        // the reference's zeros() start: a surface list may stay unfilled (ne = 1 has no top)
        if (top && (st = sfem_cuda_status(ctx, cudaMemsetAsync(top, 0, sizeof(int64_t) * nenF * nF, ctx->stream),
                                          "memset")))
            break;
        if (btm && (st = sfem_cuda_status(ctx, cudaMemsetAsync(btm, 0, sizeof(int64_t) * nenF * nF, ctx->stream),
                                          "memset")))
            break;
        if (X || id) {
            k_grid_nodes<<<grid_for(nN), 256, 0, ctx->stream>>>(ndim, ne, x0, x1, y0, y1, z0, z1, nN, X, id);
            SFEM_LAUNCHED(ctx);
        }
        if (ien || top || btm) {
            k_grid_elems<<<grid_for(nEl), 256, 0, ctx->stream>>>(ndim, ne, ien, top, btm);
            SFEM_LAUNCHED(ctx);
        }
        if (!dev) {
            if (NodeList && (st = sfem_copy_out(ctx, NodeList, X, sizeof(double) * ndim * nN, mem_space))) break;
            if (IEN && (st = sfem_copy_out(ctx, IEN, ien, sizeof(int64_t) * (1 << ndim) * nEl, mem_space))) break;
            if (ID && (st = sfem_copy_out(ctx, ID, id, sizeof(int64_t) * ndim * nN, mem_space))) break;
            if (IEN_top && (st = sfem_copy_out(ctx, IEN_top, top, sizeof(int64_t) * nenF * nF, mem_space))) break;
            if (IEN_btm && (st = sfem_copy_out(ctx, IEN_btm, btm, sizeof(int64_t) * nenF * nF, mem_space))) break;
        }
        st = sfem_check_device(ctx, "meshgrid");
    } while (0);
    if (!dev) {
        void *bufs[] = {X, ien, id, top, btm};
        for (void *p : bufs) sfem_dfree(ctx, p);
    }
    return st;
}

extern "C" int sfem_inflate_sphere(sfem_ctx *ctx, double *NodeList, int ndim, int64_t nNodes, double x0, double x1,
                                   double y0, double y1, int mem_space) {
    if (!ctx || (!NodeList && nNodes > 0) || nNodes < 0 || ndim < 2) return SFEM_BAD_ARG;
    SFEM_TRY(sfem_check_ptr(ctx, NodeList, mem_space));
    if (nNodes == 0) return SFEM_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        cudaGetLastError();
        return sfem_set_error(ctx, SFEM_CUDA_ERROR, "cudaSetDevice(%d) failed", ctx->device);
    }
    const double xc = 0.5 * (x0 + x1), yc = 0.5 * (y0 + y1);
    double *X = NodeList;
    if (mem_space != SFEM_MEM_DEVICE) {
        SFEM_TRY(sfem_dalloc(ctx, (void **)&X, sizeof(double) * ndim * nNodes, "inflate nodes"));
        int st = sfem_copy_in(ctx, X, NodeList, sizeof(double) * ndim * nNodes, mem_space);
        if (st == SFEM_OK) {
            k_inflate<<<grid_for(nNodes), 256, 0, ctx->stream>>>(X, ndim, nNodes, xc, yc);
            SFEM_LAUNCHED(ctx);
            st = sfem_copy_out(ctx, NodeList, X, sizeof(double) * ndim * nNodes, mem_space);
        }
        if (st == SFEM_OK) st = sfem_check_device(ctx, "inflate_sphere");
        sfem_dfree(ctx, X);
        return st;
    }
    k_inflate<<<grid_for(nNodes), 256, 0, ctx->stream>>>(X, ndim, nNodes, xc, yc);
    SFEM_LAUNCHED(ctx);
    return sfem_check_device(ctx, "inflate_sphere");
}
