// Serving: a device-resident request loop with continuous batching.
//
// Host side (one worker thread per server):
//   admission  requests wait in a FIFO until their device footprint fits the
//              HBM budget; the mesh pattern is built once per topology key
//              and cached; the request's inputs and work buffers are placed
//              on the device and its descriptor is written into a ring;
//              publishing bumps a tail counter in mapped host memory.
//   harvest    a completed request (its done flag, written by the GPU into
//              mapped host memory, equals its sequence number) has u copied
//              back, its buffers released, and its waiters woken.
//   kernel     if requests are outstanding and the persistent kernel is not
//              running (it leaves after an idle deadline), it is launched.
// Device side (k_serve, persistent):
//   every group (one CTA, or a thread-block cluster) claims the next
//   published descriptor with a CAS on a device head counter, runs the
//   per-mesh pipeline of sfem_meshsolve.cuh on it, and publishes completion
//   with a system-scope fence and release store.  Requests that arrive while
//   others are on the GPU start as soon as a group is free: their work
//   overlaps on the device.  Polling for work is bounded by an idle deadline;
//   nothing waits on another group.
//
// Request buffers come from the stream-ordered pool and are recycled while
// the kernel keeps running, so after every claim each thread executes a
// system-scope acquire fence: it drops L1 lines that may still hold a
// recycled buffer's old contents.
#include <algorithm>
#include <atomic>
#include <initializer_list>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sfem_meshsolve.cuh"

namespace {

using namespace sfem_dev;

// Element classes one serving kernel handles; a request names its own.
enum ServeClass { CLS_Q1_2D_SCALAR = 0, CLS_Q1_2D_ELASTIC, CLS_Q1_3D_SCALAR, CLS_Q1_3D_ELASTIC, CLS_Q2_2D_SCALAR,
                  NUM_CLASSES };

int serve_class(int ndim, int fclass, int b) {
    if (fclass == SFEM_Q2) return (ndim == 2 && b == 1) ? CLS_Q2_2D_SCALAR : -1;
    if (fclass != SFEM_Q1) return -1;
    if (ndim == 2) return b == 1 ? CLS_Q1_2D_SCALAR : (b == 2 ? CLS_Q1_2D_ELASTIC : -1);
    if (ndim == 3) return b == 1 ? CLS_Q1_3D_SCALAR : (b == 3 ? CLS_Q1_3D_ELASTIC : -1);
    return -1;
}

// Shape-function tables: 2D Q1, 3D Q1, 2D Q2.
struct ServeTables {
    ElemTableB t[3];
};

struct ServeDesc {
    BatchArgs args;
    BatchMesh mesh;
    long long seq;
    int slot;
    int cls;  // ServeClass
};

struct ServeTrace {
    long long t_claim, t_end;  // %globaltimer (ns) at claim and at completion
    int smid, pad;             // SM of the group's first CTA
};

struct ServeCtl {
    const ServeDesc *ring;
    long long cap;
    unsigned long long *head;      // device: next descriptor to claim
    const long long *tail;         // mapped host: descriptors published
    long long *done;               // mapped host: per slot, seq of the last completed request
    const int *stop;               // mapped host: stop request
    long long idle_ns;             // leave after this long without work
    int *exit_reason;              // mapped host: 1 idle, 2 stop
    ServeTrace *trace;             // mapped host: per slot, when and where the request ran
    unsigned long long *state;     // device: idle / started groups and CLOSING (zeroed per launch)
};

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ long long ld_acquire_sys(const long long *p) {
    long long v;
    asm volatile("ld.acquire.sys.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_acquire_sys_i(const int *p) {
    int v;
    asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_sys(long long *p, long long v) {
    asm volatile("st.release.sys.global.s64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// The kernel leaves collectively: a group that has found no work for idle_ns
// counts itself idle, and once every started group is idle one of them sets
// CLOSING; from then on no group takes work and all leave.  (A group leaving
// alone would let the kernel run on with fewer groups, and the host relaunches
// only a kernel that has ended.)  Groups that start after CLOSING leave at
// once, so the resident groups never wait for one that is not resident.
// State word: bits 0-23 idle groups, 24-47 started groups, 63 CLOSING.
constexpr unsigned long long IDLE_ONE = 1ull, STARTED_ONE = 1ull << 24, CLOSING = 1ull << 63;
constexpr unsigned long long COUNT_MASK = (1ull << 24) - 1;

__device__ __forceinline__ bool all_idle(unsigned long long v) {
    return (v & COUNT_MASK) == ((v >> 24) & COUNT_MASK);
}

// Claim the next published descriptor; -1 when the kernel closes for lack of
// work, -2 on stop.  Every wait here ends: the host's stop flag, the work of
// the busy groups (bounded by maxit) and the idle deadline bound it.
__device__ long long claim(const ServeCtl &c) {
    unsigned long long t0 = gtimer();
    unsigned ns = 256;
    bool idle = false;
    for (;;) {
        if (ld_acquire_sys_i(c.stop)) return -2;
        const long long t = ld_acquire_sys(c.tail);
        const unsigned long long h = atomicAdd(c.head, 0ull);
        if ((long long)h < t) {
            if (idle) {  // rejoin the busy groups unless the kernel is closing
                unsigned long long v = atomicAdd(c.state, 0ull);
                for (;;) {
                    if (v & CLOSING) return -1;
                    const unsigned long long w = atomicCAS(c.state, v, v - IDLE_ONE);
                    if (w == v) break;
                    v = w;
                }
                idle = false;
                t0 = gtimer();
            }
            if (atomicCAS(c.head, h, h + 1) == h) return (long long)h;
            continue;  // another group took it: retry at once
        }
        if (!idle) {
            if ((long long)(gtimer() - t0) > c.idle_ns) {
                const unsigned long long v = atomicAdd(c.state, IDLE_ONE) + IDLE_ONE;
                idle = true;
                if (!(v & CLOSING) && all_idle(v)) atomicCAS(c.state, v, v | CLOSING);
            }
        } else {
            const unsigned long long v = atomicAdd(c.state, 0ull);
            if (v & CLOSING) return -1;
            if (all_idle(v)) atomicCAS(c.state, v, v | CLOSING);
        }
        __nanosleep(ns);
        ns = ns < 8192 ? 2 * ns : 8192;
    }
}

// One group (a thread-block cluster) per request; any element class.
template <bool MIXED>
__global__ void __launch_bounds__(512, 1) k_serve(const __grid_constant__ ServeTables tabs, const __grid_constant__ ServeCtl c) {
    __shared__ double red[128];  // two halves, alternating (block_sum2)
    __shared__ double xch[4];
    __shared__ int s_flag;
    __shared__ long long s_idx;
    __shared__ __align__(16) BatchArgs s_args;
    cgrp::cluster_group cl = cgrp::this_cluster();
    const int tid = threadIdx.x;
    long long t_claim = 0;
    bool joined = false;
    for (;;) {
        if (cl.block_rank() == 0 && tid == 0) {
            bool closed = false;
            if (!joined) {  // count this group as started, unless the kernel already closes
                joined = true;
                closed = (atomicAdd(c.state, STARTED_ONE) & CLOSING) != 0;
            }
            s_idx = closed ? -1 : claim(c);
            t_claim = (long long)gtimer();
        }
        cl.sync();
        const long long idx = *cl.map_shared_rank(&s_idx, 0);
        cl.sync();
        if (idx < 0) {
            if (cl.block_rank() == 0 && tid == 0 && c.exit_reason) *c.exit_reason = idx == -2 ? 2 : 1;
            break;
        }
        asm volatile("fence.acq_rel.sys;" ::: "memory");  // see the freshly uploaded request, not stale L1 lines
        const ServeDesc *d = c.ring + (idx % c.cap);
        static_assert(sizeof(BatchArgs) % 8 == 0, "BatchArgs is copied in 8-byte words");
        const long long *src = (const long long *)&d->args;
        long long *dst = (long long *)&s_args;
        for (int w = tid; w < (int)(sizeof(BatchArgs) / 8); w += blockDim.x) dst[w] = __ldcg(src + w);
        __syncthreads();
        {  // u starts at zero (DOFs without an equation keep it); written again only after later group syncs
            const int64_t nu = s_args.u_len;
            for (int64_t i = (int64_t)cl.block_rank() * blockDim.x + tid; i < nu; i += (int64_t)cl.num_blocks() * blockDim.x)
                s_args.u_out[i] = 0.0;
        }
        // Unroll choices per class: the two elasticity classes get the wide SpMV
        // (the 2D one with its pipelined 9-slab path, the 3D one as a separate
        // function so that its allocation is not shared with the other classes:
        // measured 17% faster per iteration); the scalar ones stay narrow, which
        // keeps the shared kernel's register allocation nearly free of spills.
        // Requests with a multigrid hierarchy run the pipeline as a call of its own.
        const ClusterGroup G;
        const bool mg = MIXED && s_args.mg != nullptr;
        switch (__ldcg(&d->cls)) {
            case CLS_Q1_2D_SCALAR:
                if (mg) process_mesh_mg<ClusterGroup, 2, 4, 4, 1, true, 4, 0, 1, false>(G, tabs.t[0], s_args, 0, red, xch, &s_flag);
                else process_mesh<ClusterGroup, 2, 4, 4, 1, MIXED, 4, 0, 1>(G, tabs.t[0], s_args, 0, red, xch, &s_flag);
                break;
            case CLS_Q1_2D_ELASTIC:
                if (mg) process_mesh_mg<ClusterGroup, 2, 4, 4, 2, true, 9, 9, 1, false>(G, tabs.t[0], s_args, 0, red, xch, &s_flag);
                else process_mesh<ClusterGroup, 2, 4, 4, 2, MIXED, 9, 9, 1>(G, tabs.t[0], s_args, 0, red, xch, &s_flag);
                break;
            case CLS_Q1_3D_SCALAR:
                if (mg) process_mesh_mg<ClusterGroup, 3, 8, 8, 1, true, 4, 0, 1, false>(G, tabs.t[1], s_args, 0, red, xch, &s_flag);
                else process_mesh<ClusterGroup, 3, 8, 8, 1, MIXED, 4, 0, 1>(G, tabs.t[1], s_args, 0, red, xch, &s_flag);
                break;
            case CLS_Q1_3D_ELASTIC:
                if (mg) process_mesh_mg<ClusterGroup, 3, 8, 8, 3, true, 9, 0, 1, true>(G, tabs.t[1], s_args, 0, red, xch, &s_flag);
                else process_mesh<ClusterGroup, 3, 8, 8, 3, MIXED, 9, 0, 1, true>(G, tabs.t[1], s_args, 0, red, xch, &s_flag);
                break;
            default:
                process_mesh<ClusterGroup, 2, 9, 4, 1, MIXED, 4, 0, 1>(G, tabs.t[2], s_args, 0, red, xch, &s_flag);
                break;
        }
        cl.sync();
        if (cl.block_rank() == 0 && tid == 0) {
            const int slot = __ldcg(&d->slot);
            const long long seq = __ldcg(&d->seq);
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            ServeTrace tr;
            tr.t_claim = t_claim;
            tr.t_end = (long long)gtimer();
            tr.smid = (int)smid;
            tr.pad = 0;
            c.trace[slot] = tr;
            __threadfence_system();  // u, the stats and the trace are visible before the flag
            st_release_sys(c.done + slot, seq);
        }
    }
    cl.sync();  // peers may read this CTA's shared memory until all are done
}

struct Topology {
    sfem_mesh *mesh = nullptr;
    int refs = 0;
    int mg_ne = 0;           // elements per direction of a structured (meshgrid) mesh, else 0
    double *warm = nullptr;  // last solution served on this topology (warm starts)
    bool warm_valid = false;
};

struct Request {
    int64_t id = 0, key = 0;
    std::vector<double> X, E, nu, fvals;
    std::vector<int64_t> IEN, ID, fdofs;
    int64_t nN = 0, nEl = 0;
    int ndim = 0, fclass = 0, b = 0, nen = 0, plane = 0, cls = 0;
    int mg_ne = 0;     // multigrid hierarchy of this many elements per direction (0: none)
    int64_t need = 0;  // device bytes while in flight
    // in flight
    int slot = -1;
    long long seq = -1;
    sfem_mesh *mesh = nullptr;
    std::vector<void *> bufs;
    double *d_u = nullptr;
    int64_t ndof = 0;
    // result
    bool finished = false;
    int status = SFEM_OK;
    std::vector<double> u;
    sfem_batch_stats stats{};
    ServeTrace trace{};
    std::chrono::steady_clock::time_point t_submit, t_publish, t_done;
};

}  // namespace

struct sfem_server {
    sfem_server_config cfg;
    sfem_ctx *ctx = nullptr;               // pattern builds, uploads (ctx->stream)
    cudaStream_t compute = nullptr, copy = nullptr;
    ServeDesc *ring = nullptr;
    int64_t cap = 0;
    unsigned long long *head = nullptr;  // [0] next descriptor to claim, [1] the kernel's group state
    long long *h_tail = nullptr, *h_done = nullptr;  // mapped host memory: host and device addresses
    int *h_stop = nullptr, *h_exit = nullptr;
    sfem_batch_stats *h_stats = nullptr;
    long long *d_tail = nullptr, *d_done = nullptr;
    int *d_stop = nullptr, *d_exit = nullptr;
    sfem_batch_stats *d_stats = nullptr;
    ServeTrace *h_trace = nullptr, *d_trace = nullptr;
    std::vector<char> busy;  // ring position in use (descriptor, done flag, stats)
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::unordered_map<int64_t, Request *> requests;  // every request not yet collected
    std::vector<Request *> inflight;
    std::unordered_map<int64_t, Topology> topo;
    bool quit = false, kernel_running = false;
    int64_t next_id = 1, published = 0, bytes_in_use = 0, budget = 0;
    int64_t n_done = 0, n_launches = 0, peak_inflight = 0, peak_bytes = 0;
    int last_error = SFEM_OK;
    std::string last_msg;
    int grid = 0, cluster = 1;
};

namespace {

int64_t request_bytes(int ndim, int nen, int b, int64_t nN, int64_t nEl, int64_t nfix, int64_t nslabs) {
    const int64_t nd = ((nN + 31) / 32) * 32 * b;
    int64_t bytes = 0;
    bytes += 8 * (int64_t)ndim * nN;                              // X
    bytes += 8 * (nEl + 1) + 8 * 2;                               // E, nu
    bytes += 16 * nfix;                                           // fixed dofs + values
    bytes += 8 * (int64_t)sfem_npairs(nen) * b * b * nEl;         // element stiffness
    bytes += (8 + 4) * nslabs * 32 * b * b;                       // K fp64 + fp32
    bytes += 2 * nd + 8 * 4 * nd + 8 * (6 * nd + nd * b);         // masks, FP64 vectors, CG vectors + minv
    bytes += 8 * b * nN * 2;                                      // u, initial guess (warm starts)
    return bytes;
}

// Dynamic shared memory of process_mesh for one class at `threads` per CTA.
template <int NDIM, int NEN, int NGP>
size_t class_smem(int threads) {
    constexpr int GS = NEN * NDIM + 1;
    const int ngroups = (threads / 32) / NGP;
    return sizeof(double) * (size_t)ngroups * (NGP * 32 * GS + NGP * 32);
}

template <bool MIXED>
int launch_serve(sfem_server *s, const ServeCtl &c) {
    const int threads = s->cfg.threads;
    const size_t smem = std::max({class_smem<2, 4, 4>(threads), class_smem<3, 8, 8>(threads), class_smem<2, 9, 4>(threads)});
    auto kern = k_serve<MIXED>;
    sfem_ctx *ctx = s->ctx;
    SFEM_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr[1];
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s->compute;
    // always launched as clusters (of one CTA when cluster == 1): the kernel syncs and
    // exchanges partial sums through cluster barriers and distributed shared memory
    int csize = s->cfg.cluster, nclusters = 0;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    for (;;) {
        attr[0].val.clusterDim.x = csize;
        cfg.gridDim = dim3(csize * ctx->num_sms, 1, 1);
        if (cudaOccupancyMaxActiveClusters(&nclusters, (void *)kern, &cfg) == cudaSuccess && nclusters >= 1) break;
        cudaGetLastError();
        if (csize == 1) return sfem_set_error(ctx, SFEM_UNSUPPORTED, "serving kernel does not fit");
        csize /= 2;
    }
    // this server's share of the GPU
    const double frac = s->cfg.sm_fraction > 0.0 && s->cfg.sm_fraction <= 1.0 ? s->cfg.sm_fraction : 1.0;
    const int groups = std::max(1, (int)(nclusters * frac));
    cfg.gridDim = dim3((unsigned)(groups * csize), 1, 1);
    s->grid = groups * csize;
    s->cluster = csize;
    ServeTables tabs;
    tabs.t[0] = make_table_b(2, SFEM_Q1);
    tabs.t[1] = make_table_b(3, SFEM_Q1);
    tabs.t[2] = make_table_b(2, SFEM_Q2);
    SFEM_CUDA(ctx, cudaLaunchKernelEx(&cfg, kern, tabs, c));
    SFEM_LAUNCHED(ctx);
    return SFEM_OK;
}

int start_kernel(sfem_server *s) {
    ServeCtl c;
    c.ring = s->ring;
    c.cap = s->cap;
    c.head = s->head;
    c.tail = s->d_tail;
    c.done = s->d_done;
    c.stop = s->d_stop;
    c.idle_ns = (long long)(s->cfg.idle_exit_ms * 1e6);
    c.exit_reason = s->d_exit;
    c.trace = s->d_trace;
    c.state = s->head + 1;
    // the previous launch has ended (stream order): start with no groups counted
    if (cudaMemsetAsync(c.state, 0, sizeof(unsigned long long), s->compute) != cudaSuccess)
        return sfem_set_error(s->ctx, SFEM_CUDA_ERROR, "resetting the serving kernel state");
    *s->h_exit = 0;
    const int st = s->cfg.solve.precision == SFEM_MIXED ? launch_serve<true>(s, c) : launch_serve<false>(s, c);
    if (st == SFEM_OK) {
        s->kernel_running = true;
        s->n_launches++;
    }
    return st;
}

void release_request_buffers(sfem_server *s, Request *r) {
    for (void *p : r->bufs) sfem_dfree(s->ctx, p);
    r->bufs.clear();
    if (r->mesh) {  // set only once the request holds its pattern (own, or a counted reference)
        if (r->key == 0) {
            sfem_mesh_release(r->mesh);
        } else {
            auto it = s->topo.find(r->key);
            if (it != s->topo.end()) it->second.refs--;
        }
    }
    r->mesh = nullptr;
}

// Place one request on the device and publish it (worker thread, mutex not held).
int place_request(sfem_server *s, Request *r) {
    SfemRange range_("sfem serve place");
    sfem_ctx *ctx = s->ctx;
    const int b = r->b, nd_ = r->ndim;
    sfem_mesh *m = nullptr;
    if (r->key != 0) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->topo.find(r->key);
            if (it != s->topo.end()) m = it->second.mesh;
        }
        if (!m) {  // first request of this topology: build its pattern (only the worker inserts)
            if (r->IEN.empty()) return sfem_set_error(ctx, SFEM_BAD_ARG, "new topology without IEN");
            SFEM_TRY(sfem_mesh_create_nel(ctx, nd_, r->fclass, b, r->nEl, r->X.data(), r->nN,
                                          r->IEN.data(), r->nEl, r->nen, b > 1 ? r->ID.data() : nullptr,
                                          SFEM_MEM_HOST, &m));
            int st = sfem_pattern_build(ctx, m, nullptr, nullptr);
            if (st != SFEM_OK) {
                sfem_mesh_release(m);
                return st;
            }
            std::lock_guard<std::mutex> lk(s->mu);
            s->topo[r->key].mesh = m;
        }
        if (m->nN != r->nN || m->nEl != r->nEl || m->ndim != r->ndim || m->nen != r->nen || m->b != r->b)
            return sfem_set_error(ctx, SFEM_BAD_ARG, "topology key %lld reused with a different mesh",
                                  (long long)r->key);
        std::lock_guard<std::mutex> lk(s->mu);
        s->topo[r->key].refs++;
        r->mesh = m;
    } else {
        SFEM_TRY(sfem_mesh_create_nel(ctx, nd_, r->fclass, b, r->nEl, r->X.data(), r->nN, r->IEN.data(),
                                      r->nEl, r->nen, b > 1 ? r->ID.data() : nullptr, SFEM_MEM_HOST, &m));
        r->mesh = m;  // released with the request
        SFEM_TRY(sfem_pattern_build(ctx, m, nullptr, nullptr));
    }
    const int64_t nN = m->nN, nEl = m->nEl, nfix = (int64_t)r->fdofs.size();
    const int64_t nd = m->nN * b;  // nN is a multiple of 32 only in batches; pad vectors to whole slices here
    const int64_t ndp = m->nslices * 32 * b;
    const int64_t nv = m->nslabs * 32 * b * b;
    const int64_t nk = (int64_t)sfem_npairs(m->nen) * b * b * nEl;
    (void)nd;
    auto alloc = [&](void **p, size_t bytes, const char *what) -> int {
        SFEM_TRY(sfem_dalloc(ctx, p, bytes, what));
        r->bufs.push_back(*p);
        return SFEM_OK;
    };
    double *X, *E, *NU, *fv, *kbuf, *val64, *ud, *b64, *x64, *q64, *u;
    float *val32;
    int64_t *fd;
    unsigned char *fixed, *gfixed;
    void *vecT;
    SFEM_TRY(alloc((void **)&X, sizeof(double) * nd_ * nN, "request X"));
    SFEM_TRY(alloc((void **)&E, sizeof(double) * r->E.size(), "request E"));
    SFEM_TRY(alloc((void **)&NU, sizeof(double) * r->nu.size(), "request nu"));
    SFEM_TRY(alloc((void **)&fd, sizeof(int64_t) * (nfix + 1), "request fixed dofs"));
    SFEM_TRY(alloc((void **)&fv, sizeof(double) * (nfix + 1), "request fixed values"));
    SFEM_TRY(alloc((void **)&kbuf, sizeof(double) * (nk + 1), "request element stiffness"));
    SFEM_TRY(alloc((void **)&val64, sizeof(double) * (nv + 1), "request K"));
    SFEM_TRY(alloc((void **)&val32, sizeof(float) * (nv + 1), "request K fp32"));
    SFEM_TRY(alloc((void **)&fixed, ndp + 1, "request mask"));
    SFEM_TRY(alloc((void **)&gfixed, b * nN + 1, "request global mask"));
    SFEM_TRY(alloc((void **)&ud, sizeof(double) * ndp, "request q_d"));
    SFEM_TRY(alloc((void **)&b64, sizeof(double) * ndp, "request rhs"));
    SFEM_TRY(alloc((void **)&x64, sizeof(double) * ndp, "request x"));
    SFEM_TRY(alloc((void **)&q64, sizeof(double) * ndp, "request q"));
    SFEM_TRY(alloc(&vecT, sizeof(double) * (6 * ndp + ndp * b), "request CG vectors"));
    SFEM_TRY(alloc((void **)&u, sizeof(double) * (b * nN + 1), "request u"));
    MgMesh *mg = nullptr;
    if (r->mg_ne > 0) {  // multigrid hierarchy: the record, then its arrays
        const int64_t mgb = mg_layout(nd_, b, r->mg_ne, ndp, nullptr, nullptr);
        SFEM_TRY(alloc((void **)&mg, (size_t)mgb, "request multigrid"));
        MgMesh rec;
        mg_layout(nd_, b, r->mg_ne, ndp, (char *)mg, &rec);
        SFEM_CUDA(ctx, cudaMemcpyAsync(mg, &rec, sizeof(rec), cudaMemcpyHostToDevice, ctx->stream));
    }
    double *u0 = nullptr;
    if (s->cfg.warm_start && r->key != 0) {  // a private copy: the topology's buffer moves on
        const double *w = nullptr;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->topo.find(r->key);
            if (it != s->topo.end() && it->second.warm_valid) w = it->second.warm;
        }
        if (w) {
            SFEM_TRY(alloc((void **)&u0, sizeof(double) * (b * nN), "request initial guess"));
            SFEM_CUDA(ctx, cudaMemcpyAsync(u0, w, sizeof(double) * b * nN, cudaMemcpyDeviceToDevice, ctx->stream));
        }
    }
    SFEM_TRY(sfem_copy_in(ctx, X, r->X.data(), sizeof(double) * nd_ * nN, SFEM_MEM_HOST));
    SFEM_TRY(sfem_copy_in(ctx, E, r->E.data(), sizeof(double) * r->E.size(), SFEM_MEM_HOST));
    SFEM_TRY(sfem_copy_in(ctx, NU, r->nu.data(), sizeof(double) * r->nu.size(), SFEM_MEM_HOST));
    SFEM_TRY(sfem_copy_in(ctx, fd, r->fdofs.data(), sizeof(int64_t) * nfix, SFEM_MEM_HOST));
    SFEM_TRY(sfem_copy_in(ctx, fv, r->fvals.data(), sizeof(double) * nfix, SFEM_MEM_HOST));
    r->d_u = u;  // zeroed by the kernel: no memset kernel that would wait for free SMs
    r->ndof = b * nN;
    // descriptor
    const int slot = r->slot;
    ServeDesc d;
    memset(&d, 0, sizeof(d));
    d.mesh.node0 = 0;
    d.mesh.nnode = nN;
    d.mesh.slice0 = 0;
    d.mesh.slice1 = m->nslices;
    d.mesh.elem0 = 0;
    d.mesh.elem1 = nEl;
    d.mesh.dof0 = 0;
    d.mesh.ndof = b * nN;
    d.mesh.fix0 = 0;
    d.mesh.fix1 = nfix;
    BatchArgs &a = d.args;
    a.meshes = &s->ring[slot].mesh;
    a.nmesh = 1;
    a.nmesh_all = 1;
    a.X = X;
    a.ien = m->ien;
    a.nEl = nEl;
    a.n2e_ptr = m->n2e_ptr;
    a.n2e = m->n2e;
    a.rowlen = m->rowlen;
    a.sliceptr = m->sliceptr;
    a.col = m->col;
    a.g2i = m->g2i;
    a.id = m->id;
    a.nN = nN;
    a.n_global = m->n_global;
    a.E = E;
    a.nE = (int64_t)r->E.size();
    a.nu = NU;
    a.nNu = (int64_t)r->nu.size();
    a.plane = r->plane;
    a.fix_dofs = fd;
    a.fix_vals = fv;
    a.kbuf = kbuf;
    a.val64 = val64;
    a.val32 = val32;
    a.fixed = fixed;
    a.gfixed = gfixed;
    a.ud = ud;
    a.b64 = b64;
    a.x64 = x64;
    a.q64 = q64;
    a.vecT = vecT;
    a.nd = ndp;
    a.u_out = u;
    a.u_len = b * nN;
    a.u_init = u0;
    a.rtol = s->cfg.solve.rtol;
    a.delta2 = s->cfg.solve.reliable_delta * s->cfg.solve.reliable_delta;
    a.maxit = s->cfg.solve.maxit > 0 ? s->cfg.solve.maxit : 1000000;
    a.block_jacobi = s->cfg.solve.precond != SFEM_PC_JACOBI ? 1 : 0;
    a.mg = mg;
    a.stats = s->d_stats + slot;  // mapped host memory
    a.err = ctx->d_err;
    d.seq = r->seq;
    d.slot = slot;
    d.cls = r->cls;
    SFEM_CUDA(ctx, cudaMemcpyAsync(&s->ring[slot], &d, sizeof(d), cudaMemcpyHostToDevice, ctx->stream));
    SFEM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SFEM_OK;
}

void worker_loop(sfem_server *s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        bool did = false;
        // ---- admission
        // Request seq lives at ring position seq % cap (the kernel claims
        // sequence numbers and finds the descriptor there); a position is
        // reused only after its previous request has been harvested.
        while (!s->pending.empty() && !s->busy[s->published % s->cap]) {
            Request *r = s->pending.front();
            if (!s->inflight.empty() && s->bytes_in_use + r->need > s->budget) break;  // wait for memory
            s->pending.pop_front();
            r->slot = (int)(s->published % s->cap);
            s->busy[r->slot] = 1;
            r->seq = s->published;
            lk.unlock();
            int st = place_request(s, r);
            lk.lock();
            if (st != SFEM_OK) {
                release_request_buffers(s, r);
                r->status = st;
                r->finished = true;
                r->t_done = std::chrono::steady_clock::now();
                s->busy[r->slot] = 0;  // not published: the next request takes this position and sequence
                s->last_error = st;
                s->last_msg = s->ctx->last_error;
                s->cv_done.notify_all();
                did = true;
                continue;
            }
            s->h_done[r->slot] = -1;
            s->bytes_in_use += r->need;
            s->peak_bytes = std::max(s->peak_bytes, s->bytes_in_use);
            s->inflight.push_back(r);
            s->peak_inflight = std::max<int64_t>(s->peak_inflight, (int64_t)s->inflight.size());
            s->published++;
            r->t_publish = std::chrono::steady_clock::now();
            __atomic_store_n(s->h_tail, (long long)s->published, __ATOMIC_RELEASE);
            did = true;
        }
        // ---- persistent kernel
        if (s->kernel_running && cudaStreamQuery(s->compute) != cudaErrorNotReady) {
            cudaGetLastError();
            s->kernel_running = false;
        }
        if (!s->kernel_running && !s->inflight.empty()) {  // also while quitting: in-flight work finishes
            const int st = start_kernel(s);
            if (st != SFEM_OK) {  // the GPU cannot run them: fail what is on the ring
                s->last_error = st;
                s->last_msg = s->ctx->last_error;
                for (Request *r : s->inflight) {
                    release_request_buffers(s, r);
                    s->bytes_in_use -= r->need;
                    s->busy[r->slot] = 0;
                    r->status = st;
                    r->finished = true;
                    r->t_done = std::chrono::steady_clock::now();
                }
                s->inflight.clear();
                s->cv_done.notify_all();
                did = true;
            }
        }
        // ---- harvest
        for (size_t i = 0; i < s->inflight.size();) {
            Request *r = s->inflight[i];
            const long long v = __atomic_load_n(&s->h_done[r->slot], __ATOMIC_ACQUIRE);
            if (v != r->seq) {
                ++i;
                continue;
            }
            r->u.resize(r->ndof);
            lk.unlock();
            cudaMemcpyAsync(r->u.data(), r->d_u, sizeof(double) * r->ndof, cudaMemcpyDeviceToHost, s->copy);
            cudaStreamSynchronize(s->copy);
            lk.lock();
            r->stats = s->h_stats[r->slot];
            r->trace = s->h_trace[r->slot];
            if (s->cfg.warm_start && r->key != 0 && r->stats.status == SFEM_OK) {
                Topology &t = s->topo[r->key];
                if (!t.warm && sfem_dalloc(s->ctx, (void **)&t.warm, sizeof(double) * r->ndof, "warm start") != SFEM_OK)
                    t.warm = nullptr;
                if (t.warm && cudaMemcpyAsync(t.warm, r->d_u, sizeof(double) * r->ndof, cudaMemcpyDeviceToDevice,
                                              s->ctx->stream) == cudaSuccess)
                    t.warm_valid = true;
                cudaGetLastError();
            }
            r->status = r->stats.status;
            release_request_buffers(s, r);
            s->bytes_in_use -= r->need;
            s->busy[r->slot] = 0;
            r->finished = true;
            r->t_done = std::chrono::steady_clock::now();
            s->n_done++;
            s->inflight[i] = s->inflight.back();
            s->inflight.pop_back();
            s->cv_done.notify_all();
            did = true;
        }
        if (s->quit && s->inflight.empty()) break;
        if (!did) {
            if (s->inflight.empty() && s->pending.empty()) {
                s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
            } else {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(50));
                lk.lock();
            }
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" void sfem_server_config_default(sfem_server_config *c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->cluster = 4;
    c->threads = 512;
    c->sm_fraction = 0.9;  // leave SMs for the pattern builds of new topologies
    c->hbm_budget_fraction = 0.5;
    c->hbm_budget_bytes = 0;
    c->max_inflight = 1024;
    c->idle_exit_ms = 20.0;
    sfem_solve_opts_default(&c->solve);
    c->solve.precision = SFEM_MIXED;
    c->solve.precond = SFEM_PC_BLOCK_JACOBI;
    c->solve.rtol = 1e-8;
}

extern "C" int sfem_server_create(int device, const sfem_server_config *cfg, sfem_server **out) {
    if (!out) return SFEM_BAD_ARG;
    *out = nullptr;
    sfem_server_config c;
    sfem_server_config_default(&c);
    if (cfg) c = *cfg;
    if ((c.cluster != 1 && c.cluster != 2 && c.cluster != 4 && c.cluster != 8) ||
        (c.threads != 256 && c.threads != 512) || c.max_inflight < 1 || !(c.idle_exit_ms > 0.0) ||
        c.solve.precond < SFEM_PC_JACOBI || c.solve.precond > SFEM_PC_MULTIGRID)
        return SFEM_BAD_ARG;
    sfem_server *s = new sfem_server();
    s->cfg = c;
    int st = sfem_ctx_create(device, &s->ctx);
    if (st != SFEM_OK) {
        delete s;
        return st;
    }
    sfem_ctx *ctx = s->ctx;
    do {
        if ((st = sfem_cuda_status(ctx, cudaStreamCreateWithFlags(&s->compute, cudaStreamNonBlocking), "stream")))
            break;
        if ((st = sfem_cuda_status(ctx, cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking), "stream"))) break;
        s->cap = c.max_inflight;
        if ((st = sfem_cuda_status(ctx, cudaMalloc(&s->ring, sizeof(ServeDesc) * s->cap), "ring"))) break;
        if ((st = sfem_cuda_status(ctx, cudaMalloc(&s->head, 2 * sizeof(unsigned long long)), "head"))) break;
        if ((st = sfem_cuda_status(ctx, cudaMemset(s->head, 0, 2 * sizeof(unsigned long long)), "head"))) break;
        if ((st = sfem_cuda_status(ctx, cudaHostAlloc((void **)&s->h_tail, 64, cudaHostAllocMapped), "tail"))) break;
        if ((st = sfem_cuda_status(ctx, cudaHostAlloc((void **)&s->h_stop, 64, cudaHostAllocMapped), "stop"))) break;
        if ((st = sfem_cuda_status(ctx, cudaHostAlloc((void **)&s->h_exit, 64, cudaHostAllocMapped), "exit"))) break;
        if ((st = sfem_cuda_status(ctx, cudaHostAlloc((void **)&s->h_done, sizeof(long long) * s->cap,
                                                      cudaHostAllocMapped), "done")))
            break;
        if ((st = sfem_cuda_status(ctx, cudaHostAlloc((void **)&s->h_stats, sizeof(sfem_batch_stats) * s->cap,
                                                      cudaHostAllocMapped), "stats")))
            break;
        if ((st = sfem_cuda_status(ctx, cudaHostAlloc((void **)&s->h_trace, sizeof(ServeTrace) * s->cap,
                                                      cudaHostAllocMapped), "trace")))
            break;
        if ((st = sfem_cuda_status(ctx, cudaHostGetDevicePointer((void **)&s->d_trace, s->h_trace, 0), "trace")) ||
            (st = sfem_cuda_status(ctx, cudaHostGetDevicePointer((void **)&s->d_tail, s->h_tail, 0), "tail")) ||
            (st = sfem_cuda_status(ctx, cudaHostGetDevicePointer((void **)&s->d_stop, s->h_stop, 0), "stop")) ||
            (st = sfem_cuda_status(ctx, cudaHostGetDevicePointer((void **)&s->d_exit, s->h_exit, 0), "exit")) ||
            (st = sfem_cuda_status(ctx, cudaHostGetDevicePointer((void **)&s->d_done, s->h_done, 0), "done")) ||
            (st = sfem_cuda_status(ctx, cudaHostGetDevicePointer((void **)&s->d_stats, s->h_stats, 0), "stats")))
            break;
        *s->h_tail = 0;
        *s->h_stop = 0;
        *s->h_exit = 0;
        for (int64_t i = 0; i < s->cap; ++i) s->h_done[i] = -1;
        s->busy.assign(s->cap, 0);
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        s->budget = c.hbm_budget_bytes > 0 ? c.hbm_budget_bytes : (int64_t)(fr * c.hbm_budget_fraction);
        s->worker = std::thread(worker_loop, s);
    } while (0);
    if (st != SFEM_OK) {
        sfem_server_destroy(s);
        return st;
    }
    *out = s;
    return SFEM_OK;
}

extern "C" int sfem_server_submit(sfem_server *s, int ndim, int function_class, int nDof, int plane,
                                  int64_t topology_key, const double *NodeList, int64_t nNodes, const int64_t *IEN,
                                  int64_t nEl, const int64_t *ID, const double *Young, int64_t nYoung,
                                  const double *nu, int64_t nNu, const int64_t *fixed_dofs, int64_t nfix,
                                  const double *fixed_vals, int64_t *request_id) {
    if (!s || !request_id || !NodeList || nNodes < 1 || nEl < 1 || nfix < 0) return SFEM_BAD_ARG;
    const int cls = serve_class(ndim, function_class, nDof);
    if (cls < 0 || (plane != SFEM_PLANE_STRESS && plane != SFEM_PLANE_STRAIN)) return SFEM_BAD_ARG;
    const int b = nDof, nen = function_class == SFEM_Q2 ? 9 : (1 << ndim);
    if (b > 1 && (!Young || !nu || (nYoung != 1 && nYoung != nEl) || nNu != 1)) return SFEM_BAD_ARG;
    if (nfix > 0 && (!fixed_dofs || !fixed_vals)) return SFEM_BAD_ARG;
    Request *r = new Request();
    r->key = topology_key;
    r->nN = nNodes;
    r->nEl = nEl;
    r->ndim = ndim;
    r->fclass = function_class;
    r->b = b;
    r->nen = nen;
    r->plane = plane;
    r->cls = cls;
    r->X.assign(NodeList, NodeList + (int64_t)ndim * nNodes);
    bool cached;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        // a key seen before: its first request carries the connectivity
        cached = topology_key != 0 && s->topo.count(topology_key) != 0;
        if (cached) r->mg_ne = s->topo[topology_key].mg_ne;
    }
    const bool want_mg = s->cfg.solve.precond == SFEM_PC_MULTIGRID && s->cfg.solve.precision == SFEM_MIXED;
    if (!cached) {
        if (!IEN || (b > 1 && !ID)) {
            delete r;
            return SFEM_BAD_ARG;
        }
        r->IEN.assign(IEN, IEN + nEl * nen);
        if (b > 1) r->ID.assign(ID, ID + nNodes * b);
        if (want_mg) {
            const int ne = mg_structured_ne(ndim, function_class, nen, nNodes, nEl, IEN, nEl);
            r->mg_ne = mg_levels(ne) >= 2 ? ne : 0;
        }
    }
    if (b > 1) {
        r->E.assign(Young, Young + nYoung);
        r->nu.assign(nu, nu + nNu);
    } else {
        r->E.assign(1, 1.0);
        r->nu.assign(1, 0.3);
    }
    r->fdofs.assign(fixed_dofs, fixed_dofs + nfix);
    r->fvals.assign(fixed_vals, fixed_vals + nfix);
    // footprint estimate from the structured-neighbour bound (27 / 25 / 9 node blocks per row)
    const int64_t width = ndim == 3 ? 27 : (nen == 9 ? 25 : 9);
    r->need = request_bytes(ndim, nen, b, nNodes, nEl, nfix, ((nNodes + 31) / 32) * width);
    if (r->mg_ne > 0) r->need += mg_layout(ndim, b, r->mg_ne, ((nNodes + 31) / 32) * 32 * b, nullptr, nullptr);
    r->t_submit = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (topology_key != 0 && !cached) s->topo[topology_key].mg_ne = r->mg_ne;  // placed in submission order
    r->id = s->next_id++;
    s->requests[r->id] = r;
    s->pending.push_back(r);
    *request_id = r->id;
    s->cv_work.notify_all();
    return SFEM_OK;
}

extern "C" int sfem_server_wait(sfem_server *s, int64_t request_id, double timeout_ms, double *u_out, int64_t u_len,
                                sfem_server_result *res) {
    if (!s) return SFEM_BAD_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return SFEM_BAD_ARG;
    Request *r = it->second;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds((int64_t)(timeout_ms * 1e3));
    while (!r->finished) {
        if (timeout_ms >= 0 && s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !r->finished)
            return SFEM_TIMEOUT;  // not finished within the timeout; the request stays queued
        if (timeout_ms < 0) s->cv_done.wait(lk);
    }
    if (res) {
        memset(res, 0, sizeof(*res));
        res->status = r->status;
        res->iterations = r->stats.iterations;
        res->refreshes = r->stats.refreshes;
        res->relres = r->stats.relres;
        res->gpu_ms = r->stats.ms;
        res->queue_ms = std::chrono::duration<double, std::milli>(r->t_publish - r->t_submit).count();
        res->total_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        res->ndof = r->ndof;
        res->t_claim_ms = r->trace.t_claim * 1e-6;
        res->t_end_ms = r->trace.t_end * 1e-6;
        res->smid = r->trace.smid;
    }
    if (u_out && u_len > 0) memcpy(u_out, r->u.data(), sizeof(double) * std::min<int64_t>(u_len, (int64_t)r->u.size()));
    s->requests.erase(it);
    delete r;
    return SFEM_OK;
}

extern "C" int sfem_server_info(sfem_server *s, sfem_server_totals *t) {
    if (!s || !t) return SFEM_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(t, 0, sizeof(*t));
    t->completed = s->n_done;
    t->pending = (int64_t)s->pending.size();
    t->inflight = (int64_t)s->inflight.size();
    t->peak_inflight = s->peak_inflight;
    t->kernel_launches = s->n_launches;
    t->bytes_in_use = s->bytes_in_use;
    t->peak_bytes = s->peak_bytes;
    t->budget_bytes = s->budget;
    t->grid = s->grid;
    t->cluster = s->cluster;
    t->topologies = (int64_t)s->topo.size();
    t->last_error = s->last_error;
    return SFEM_OK;
}

extern "C" int sfem_server_destroy(sfem_server *s) {
    if (!s) return SFEM_OK;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            // drop what has not reached the GPU; what is on it finishes
            while (!s->pending.empty()) {
                Request *r = s->pending.front();
                s->pending.pop_front();
                r->finished = true;
                r->status = SFEM_TIMEOUT;  // never reached the GPU
            }
            s->quit = true;
            s->cv_work.notify_all();
            s->cv_done.notify_all();
        }
        s->worker.join();
    }
    if (s->h_stop) *(volatile int *)s->h_stop = 1;
    if (s->compute) cudaStreamSynchronize(s->compute);
    for (auto &kv : s->requests) delete kv.second;
    for (auto &kv : s->topo) {
        if (kv.second.warm) sfem_dfree(s->ctx, kv.second.warm);
        if (kv.second.mesh) sfem_mesh_release(kv.second.mesh);
    }
    if (s->ring) cudaFree(s->ring);
    if (s->head) cudaFree(s->head);
    if (s->h_tail) cudaFreeHost(s->h_tail);
    if (s->h_stop) cudaFreeHost(s->h_stop);
    if (s->h_exit) cudaFreeHost(s->h_exit);
    if (s->h_done) cudaFreeHost(s->h_done);
    if (s->h_stats) cudaFreeHost(s->h_stats);
    if (s->h_trace) cudaFreeHost(s->h_trace);
    if (s->compute) cudaStreamDestroy(s->compute);
    if (s->copy) cudaStreamDestroy(s->copy);
    if (s->ctx) sfem_ctx_destroy(s->ctx);
    delete s;
    return SFEM_OK;
}
