// Re-assembly of an existing matrix without any device allocation.
//
// Who needs this: callers that cannot call cudaMalloc/cudaFree at the point
// where they re-assemble K.  Examples are a host process whose device memory
// is owned by another allocator under a hard budget (a framework's caching
// allocator, or a memory-capped serving process), a latency-bound loop
// (load increments, material updates) where cudaFree's implicit device-wide
// synchronisation would stall other streams, and deployments that forbid
// dynamic allocation after start-up.  They build the mesh, pattern and
// matrix once (those calls do allocate), and afterwards refresh K's values
// for new material data through this entry point, which only launches
// kernels and copies into memory that already exists.
//
// The element-stiffness scratch that sfem_assemble takes from the stream-
// ordered pool lives here in a file-scope device array instead, together
// with the copies of Young/nu.  Its size is fixed at build time
// (SFEM_NOALLOC_SCRATCH_DOUBLES, 64 MiB); meshes that need more are rejected.
#include "sfem_internal.cuh"

// 8 Mi doubles = 64 MiB on every GPU that loads the library, held until exit.
#define SFEM_NOALLOC_SCRATCH_DOUBLES (8ull << 20)

static __device__ __align__(256) double g_noalloc_scratch[SFEM_NOALLOC_SCRATCH_DOUBLES];

namespace {

// In host code `g_noalloc_scratch` names a host-side stand-in, not device
// memory, so its device address is looked up with the device current.  The
// first lookup on a device may load the module (do it before any stream
// capture); later lookups allocate nothing and are repeated on every call,
// so a context rebuilt after cudaDeviceReset gets the array's new address.
int scratch_for_device(sfem_ctx *ctx, double **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return sfem_set_error(ctx, SFEM_CUDA_ERROR, "cudaGetSymbolAddress(no-alloc scratch): %s",
                              cudaGetErrorString(e));
    }
    *out = (double *)p;
    return SFEM_OK;
}

__global__ void k_refresh_fp32(int64_t n, const double *__restrict__ v, float *__restrict__ v32) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v32[i] = (float)v[i];
}

}  // namespace

extern "C" int sfem_reassemble_noalloc(sfem_ctx *ctx, sfem_matrix *K, const double *Young, int64_t nYoung,
                                       const double *nu, int64_t nNu, int mem_space) {
    if (!ctx || !K || !K->mesh) return SFEM_BAD_ARG;
    sfem_mesh *m = K->mesh;
    if (m->ctx != ctx) return sfem_set_error(ctx, SFEM_BAD_ARG, "matrix belongs to another context");
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        cudaGetLastError();
        return sfem_set_error(ctx, SFEM_CUDA_ERROR, "cudaSetDevice(%d) failed", ctx->device);
    }
    const int b = m->b;
    const bool vec = b > 1;
    if (vec) {
        if (!Young || !nu) return sfem_set_error(ctx, SFEM_BAD_ARG, "Young and nu are required for elasticity");
        if ((nYoung != 1 && nYoung != m->nEl) || (nNu != 1 && nNu != m->nEl))
            return sfem_set_error(ctx, SFEM_BAD_ARG, "Young/nu must have length 1 or ne^ndim");
    } else {
        nYoung = nNu = 0;
    }
    const unsigned long long kdoubles = (unsigned long long)sfem_npairs(m->nen) * b * b * (unsigned long long)m->nEl;
    const unsigned long long need = kdoubles + (unsigned long long)nYoung + (unsigned long long)nNu;
    if (need > SFEM_NOALLOC_SCRATCH_DOUBLES) {
        const unsigned long long per_el = (unsigned long long)sfem_npairs(m->nen) * b * b + (nYoung > 1) + (nNu > 1);
        return sfem_set_error(ctx, SFEM_BAD_ARG,
                              "mesh too large for sfem_reassemble_noalloc: needs %llu doubles of scratch, the fixed "
                              "device array holds %llu (64 MiB), i.e. at most %llu elements of this class; use "
                              "sfem_assemble",
                              need, (unsigned long long)SFEM_NOALLOC_SCRATCH_DOUBLES,
                              (unsigned long long)(SFEM_NOALLOC_SCRATCH_DOUBLES - (nYoung == 1) - (nNu == 1)) / per_el);
    }
    double *scratch = nullptr;
    SFEM_TRY(scratch_for_device(ctx, &scratch));
    double *kbuf = scratch;
    double *dE = vec ? scratch + kdoubles : nullptr;
    double *dnu = vec ? dE + nYoung : nullptr;
    if (vec) {
        SFEM_TRY(sfem_copy_in(ctx, dE, Young, sizeof(double) * nYoung, mem_space));
        SFEM_TRY(sfem_copy_in(ctx, dnu, nu, sizeof(double) * nNu, mem_space));
    }
    // Every scratch entry the gather reads is written by the element kernel of
    // this same call, so nothing in the shared array has to be cleared first.
    SFEM_TRY(sfem_element_stiffness(ctx, m, K->plane, dE, nYoung, dnu, nNu, kbuf));
    // Errors of the element kernel (det J = 0, a bad index) are reported
    // before anything is written into K, so K keeps its old values then.
    SFEM_TRY(sfem_check_device(ctx, "no-alloc element stiffness"));
    SFEM_TRY(sfem_gather_blocks(ctx, m, kbuf, K->val, nullptr));
    if (K->val32) {  // keep the FP32 copy used by the mixed solver consistent
        const int64_t nv = m->nslabs * 32 * b * b;
        if (nv > 0) {
            k_refresh_fp32<<<(unsigned)sfem_cdiv(nv, 256), 256, 0, ctx->stream>>>(nv, K->val, K->val32);
            SFEM_LAUNCHED(ctx);
        }
    }
    SFEM_TRY(sfem_sym_refresh_values(ctx, K));  // and its upper-triangle FP32 copy (no allocation)
    return sfem_check_device(ctx, "no-alloc re-assembly");
}
