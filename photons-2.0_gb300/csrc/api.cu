// Force-pass context, stage orchestration and the photons_* C ABI.
//
// A pass (photons_force_pass) runs, on one stream:
//   upload -> tree build -> leaf offsets -> dual-tree walk -> P2P
//   -> [P2M, M2M, M2L, L2L, L2P when any M2L task exists] -> gather/download
// The reference-named entry points (legacy.cu) reuse the same stages.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <vector>

#include "photons_fmm.h"
#include "api_internal.cuh"
#include "p2p.cuh"
#include "split_kernel_coeffs.h"

// ------------------------------------------------------------------
// errors
// ------------------------------------------------------------------
static thread_local int g_status = 0;
static thread_local char g_msg[512] = {0};

int ph_set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    g_status = code;
    return code;
}

int ph_set_cuda_error(cudaError_t e, const char *what, const char *file, int line)
{
    const char *base = strrchr(file, '/');
    return ph_set_error(PH_ERR_CUDA, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), base ? base + 1 : file,
                        line);
}

extern "C" int photons_gpu_status(void) { return g_status; }
extern "C" unsigned long long photons_launch_count(void) { return ph::g_launches.load(std::memory_order_relaxed); }
extern "C" const char *photons_gpu_error(void) { return g_msg; }
extern "C" void photons_gpu_clear_error(void)
{
    g_status = 0;
    g_msg[0] = 0;
}

// Pinned host memory for the host-buffer pass: the pass's copies then run
// at the host link's rate (on GB300, 211 GB/s in and 193 GB/s out for any
// size; some pinning routes of large buffers copied at a tenth of that).
extern "C" void *photons_host_alloc(size_t bytes)
{
    photons_gpu_clear_error();
    void *p = nullptr;
    if (bytes == 0) bytes = 1;
    const cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ph_set_error(PH_ERR_NOMEM, "pinned host allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return nullptr;
    }
    return p;
}

extern "C" void photons_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}

namespace ph {
std::atomic<unsigned long long> g_launches{0};
thread_local unsigned long long *t_capture_tally = nullptr;

int device_sm_count()
{
    static int v = 0;
    if (!v) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        if (v <= 0) v = 1;
    }
    return v;
}
}  // namespace ph

// ------------------------------------------------------------------
// buffers
// ------------------------------------------------------------------
template <class T>
static int dalloc(T *&p, size_t n)
{
    if (p) cudaFree(p);
    p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)&p, n * sizeof(T));
    if (e != cudaSuccess) {
        p = nullptr;
        cudaGetLastError();
        return ph_set_error(PH_ERR_NOMEM, "device allocation of %zu bytes failed: %s", n * sizeof(T),
                            cudaGetErrorString(e));
    }
    return 0;
}

template <class T>
static void dfree(T *&p)
{
    if (p) cudaFree(p);
    p = nullptr;
}


#define CHUNK_ELEMS 1024
#define MAX_DEPTH_CAP PH_MAX_DEPTH_CAP

// Each grow below first marks its capacity empty and bumps the epoch, then
// sets the capacity only after every allocation succeeded: a failed
// cudaMalloc leaves null buffers that the next pass reallocates, never a
// recorded capacity over a freed buffer (or a captured graph that uses one).
static int alloc_particles(photons_ctx *c, int n)
{
    if (n <= c->cap_n) return 0;
    ph::BuildBufs &b = c->b;
    c->cap_n = b.cap_n = 0;
    c->epoch++;
    PH_TRY(dalloc(b.x, n)); PH_TRY(dalloc(b.y, n)); PH_TRY(dalloc(b.z, n));
    PH_TRY(dalloc(b.perm, n)); PH_TRY(dalloc(b.smallpos, n)); PH_TRY(dalloc(b.bigpos, n));
    PH_TRY(dalloc(c->pos4, n));
    PH_TRY(dalloc(c->ax, n)); PH_TRY(dalloc(c->ay, n)); PH_TRY(dalloc(c->az, n));
    PH_TRY(dalloc(c->io, (size_t)3 * n));
    c->epoch++;
    b.cap_n = n;
    c->cap_n = n;
    return 0;
}

static int alloc_tree(photons_ctx *c, int n, int cap)
{
    int chunks = n / CHUNK_ELEMS + cap + 2;
    ph::BuildBufs &b = c->b;
    if (cap > b.cap_nodes) {
        b.cap_nodes = b.cap_leaves = 0;
        c->t.cap_u = c->cap_u = c->mu_cap_leaves = 0;
        b.scan_scratch_elems = 0;
        c->epoch++;
        PH_TRY(dalloc(b.tn_start, cap)); PH_TRY(dalloc(b.tn_len, cap)); PH_TRY(dalloc(b.tn_depth, cap));
        PH_TRY(dalloc(b.tn_parent, cap)); PH_TRY(dalloc(b.tn_child0, cap)); PH_TRY(dalloc(b.tn_child1, cap));
        PH_TRY(dalloc(b.tn_mode, cap)); PH_TRY(dalloc(b.tn_S, cap)); PH_TRY(dalloc(b.tn_box, (size_t)6 * cap));
        PH_TRY(dalloc(b.tn_split, cap)); PH_TRY(dalloc(b.tn_nch, cap)); PH_TRY(dalloc(b.tn_chunk_base, cap));
        PH_TRY(dalloc(b.tn_nodeflag, cap)); PH_TRY(dalloc(b.tn_leafflag, cap)); PH_TRY(dalloc(b.tn_nodebase, cap));
        PH_TRY(dalloc(b.tn_leafbase, cap)); PH_TRY(dalloc(b.tn_sub_nodes, cap)); PH_TRY(dalloc(b.tn_sub_leaves, cap));
        PH_TRY(dalloc(b.tn_pre, cap)); PH_TRY(dalloc(b.tn_lbase, cap));
        PH_TRY(dalloc(b.tl_start, cap)); PH_TRY(dalloc(b.tl_len, cap)); PH_TRY(dalloc(b.tl_depth, cap));
        PH_TRY(dalloc(b.tl_parent, cap)); PH_TRY(dalloc(b.tl_final, cap)); PH_TRY(dalloc(b.tl_box, (size_t)6 * cap));
        PH_TRY(dalloc(b.tn_boxid, cap)); PH_TRY(dalloc(b.tl_boxid, cap));
        PH_TRY(dalloc(b.tn_subroot, cap)); PH_TRY(dalloc(b.tl_subroot, cap));
        const size_t scratch = ph::scan_scratch_elems(cap > chunks ? cap : chunks) + 8;
        PH_TRY(dalloc(b.scan_scratch, scratch));
        b.scan_scratch_elems = scratch;
        PH_TRY(dalloc(b.cnt, ph::BC_NCOUNTERS));
        PH_TRY(dalloc(b.lvl_begin, MAX_DEPTH_CAP + 2)); PH_TRY(dalloc(b.lvl_count, MAX_DEPTH_CAP + 2));
        PH_TRY(dalloc(b.leaf_begin, MAX_DEPTH_CAP + 2)); PH_TRY(dalloc(b.leaf_count, MAX_DEPTH_CAP + 2));
        c->epoch++;
        b.cap_nodes = cap;
        b.cap_leaves = cap;
    }
    // unified tree: leaves and nodes (2N/MAXLEAF each at most) and, in a
    // rank's domain pass, the nodes of the trees it receives
    const int cu = 2 * cap + 2 + c->imp_reserve_u;
    if (cu > c->cap_u) {
        ph::TreeBufs &t = c->t;
        c->t.cap_u = c->cap_u = c->mu_cap_leaves = 0;
        c->epoch++;
        PH_TRY(dalloc(t.ipart, cu)); PH_TRY(dalloc(t.npart, cu)); PH_TRY(dalloc(t.depth, cu));
        PH_TRY(dalloc(t.parent, cu)); PH_TRY(dalloc(t.son0, cu)); PH_TRY(dalloc(t.son1, cu));
        PH_TRY(dalloc(t.cx, cu)); PH_TRY(dalloc(t.cy, cu)); PH_TRY(dalloc(t.cz, cu));
        PH_TRY(dalloc(t.wx, cu)); PH_TRY(dalloc(t.wy, cu)); PH_TRY(dalloc(t.wz, cu));
        PH_TRY(dalloc(t.wsum, cu)); PH_TRY(dalloc(t.split, cu));
        PH_TRY(dalloc(t.depth_list, cu));
        PH_TRY(dalloc(t.depth_off, MAX_DEPTH_CAP + 2));
        PH_TRY(dalloc(t.depth_cnt, MAX_DEPTH_CAP + 2));
        t.max_depth_cap = MAX_DEPTH_CAP;
        t.depth_nblk = 0;
        const int nblk = ph::depth_sort_blocks(cu);
        PH_TRY(dalloc(t.depth_blk, (size_t)2 * MAX_DEPTH_CAP * nblk));
        t.depth_nblk = nblk;
        const size_t need = ph::scan_scratch_elems(MAX_DEPTH_CAP * nblk) + 8;
        if (need > b.scan_scratch_elems) {
            b.scan_scratch_elems = 0;
            PH_TRY(dalloc(b.scan_scratch, need));
            b.scan_scratch_elems = need;
        }
        t.cap_u = cu;
        // per-unified walk bookkeeping and expansions
        ph::WalkBufs &w = c->w;
        PH_TRY(dalloc(w.pd_off, cu)); PH_TRY(dalloc(w.pd_cnt, cu));
        PH_TRY(dalloc(w.p2p_off, cu)); PH_TRY(dalloc(w.p2p_cnt, cu));
        PH_TRY(dalloc(w.m2l_off, cu)); PH_TRY(dalloc(w.m2l_cnt, cu));
        PH_TRY(dalloc(t.chi, cu)); PH_TRY(dalloc(t.clo, cu)); PH_TRY(dalloc(t.w32, cu)); PH_TRY(dalloc(t.son2, cu));
        PH_TRY(dalloc(t.boxid, cu));
        PH_TRY(dalloc(c->mu_sorted, cu)); PH_TRY(dalloc(c->mu_nrecv, cu)); PH_TRY(dalloc(c->mu_nev, cu));
        PH_TRY(dalloc(c->mu_size, cu)); PH_TRY(dalloc(c->mu_rbase, cu));
        PH_TRY(dalloc(c->mu_scan, ph::scan_scratch_elems(cu) + 8));
        if (!c->mu_total || !c->mu_over) { PH_TRY(dalloc(c->mu_total, 1)); PH_TRY(dalloc(c->mu_over, 1)); }
        c->mu_cap_leaves = cu;
        PH_TRY(dalloc(c->M, (size_t)cu * PH_NMULTI));
        PH_TRY(dalloc(c->L, (size_t)cu * PH_NMULTI));
        PH_TRY(dalloc(c->M32, (size_t)cu * PH_NMULTI));
        c->cap_u = cu;
    }
    if (chunks > b.cap_chunks) {
        b.cap_chunks = 0;
        c->epoch++;
        PH_TRY(dalloc(b.ch_partial, chunks)); PH_TRY(dalloc(b.ch_cnt, chunks)); PH_TRY(dalloc(b.ch_small_base, chunks));
        PH_TRY(dalloc(b.ch_node, chunks)); PH_TRY(dalloc(b.ch_swap, chunks));
        c->epoch++;
        b.cap_chunks = chunks;
        size_t need = ph::scan_scratch_elems(cap > chunks ? cap : chunks) + 8;
        if (need > b.scan_scratch_elems) {
            b.scan_scratch_elems = 0;
            PH_TRY(dalloc(b.scan_scratch, need));
            b.scan_scratch_elems = need;
        }
    }
    return 0;
}

static int alloc_walk(photons_ctx *c, long long p2p_cap, long long pd_cap, long long m2l_cap, int stack_cap,
                      int stage_cap)
{
    ph::WalkBufs &w = c->w;
    if (!w.ctr) { PH_TRY(dalloc(w.ctr, ph::WC_N)); c->epoch++; }
    if (!c->far_gate) { PH_TRY(dalloc(c->far_gate, 2)); c->epoch++; }
    if (!c->work_counter) { PH_TRY(dalloc(c->work_counter, 4)); c->epoch++; }
    if (p2p_cap > w.p2p_cap) {
        w.p2p_cap = 0;
        c->epoch++;
        PH_TRY(dalloc(w.p2p_pool, p2p_cap));
        w.p2p_cap = p2p_cap;
        c->epoch++;
    }
    if (pd_cap > w.pd_cap) {
        w.pd_cap = 0;
        c->epoch++;
        PH_TRY(dalloc(w.pd_pool[0], pd_cap));
        PH_TRY(dalloc(w.pd_pool[1], pd_cap));
        w.pd_cap = pd_cap;
        c->epoch++;
    }
    if (m2l_cap > w.m2l_cap) {
        w.m2l_cap = 0;
        c->epoch++;
        PH_TRY(dalloc(w.m2l_pool, m2l_cap));
        w.m2l_cap = m2l_cap;
    }
    // resident 256-thread walk blocks per SM: 2 (no register spills) or 3
    const char *wb = getenv("PHOTONS_WALK_BLOCKS");
    int nwarps = ph::device_sm_count() * ((wb && atoi(wb) == 3) ? 3 : 2) * 8;
    if (stack_cap > w.stack_cap || stage_cap > w.stage_cap || nwarps != w.nwarps) {
        if (stack_cap < w.stack_cap) stack_cap = w.stack_cap;
        if (stage_cap < w.stage_cap) stage_cap = w.stage_cap;
        w.stack_cap = w.stage_cap = w.nwarps = 0;
        c->epoch++;
        PH_TRY(dalloc(w.scratch, (size_t)nwarps * (stack_cap + 3 * (size_t)stage_cap)));
        c->epoch++;
        w.stack_cap = stack_cap;
        w.stage_cap = stage_cap;
        w.nwarps = nwarps;
    }
    return 0;
}

static void free_all(photons_ctx *c)
{
    ph::BuildBufs &b = c->b;
    void *ptrs[] = {b.x, b.y, b.z, b.perm, b.smallpos, b.bigpos, b.tn_start, b.tn_len, b.tn_depth, b.tn_parent,
                    b.tn_child0, b.tn_child1, b.tn_mode, b.tn_S, b.tn_box, b.tn_split, b.tn_nch, b.tn_chunk_base,
                    b.tn_nodeflag, b.tn_leafflag, b.tn_nodebase, b.tn_leafbase, b.tn_sub_nodes, b.tn_sub_leaves,
                    b.tn_pre, b.tn_lbase, b.tl_start, b.tl_len, b.tl_depth, b.tl_parent, b.tl_final, b.tl_box,
                    b.ch_partial, b.ch_cnt, b.ch_small_base, b.ch_node, b.cnt, b.scan_scratch, c->t.ipart, c->t.npart,
                    c->t.depth, c->t.parent, c->t.son0, c->t.son1, c->t.cx, c->t.cy, c->t.cz, c->t.wx, c->t.wy,
                    c->t.wz, c->t.wsum, c->t.split, c->t.depth_list, c->t.depth_off, c->w.pd_pool[0],
                    c->w.pd_pool[1], c->w.pd_off, c->w.pd_cnt, c->w.p2p_pool, c->w.p2p_off, c->w.p2p_cnt,
                    c->w.m2l_pool, c->w.m2l_off, c->w.m2l_cnt, c->w.scratch, c->w.ctr, c->pos4, c->ax, c->ay,
                    c->az, c->M, c->L, c->io, c->work_counter, c->t.chi, c->t.clo, c->t.w32, c->t.son2, c->M32,
                    b.lvl_begin, b.lvl_count, b.leaf_begin, b.leaf_count, c->t.depth_cnt, b.tn_boxid, b.tl_boxid,
                    c->t.boxid, b.boxes, c->far_gate, c->mu_sorted, c->mu_nrecv, c->mu_slot, c->mu_over,
                    c->mu_size, c->mu_rbase, c->mu_total, c->mu_scan, c->mu_buf, c->mu_ev, c->mu_nev, c->mu_pq,
                    b.tn_subroot, b.tl_subroot, b.ch_swap, c->t.depth_blk};
    for (void *p : ptrs)
        if (p) cudaFree(p);
}

// ------------------------------------------------------------------
// small kernels
// ------------------------------------------------------------------
namespace {

// a copy between device memory and pinned host memory that the device
// addresses directly (over the host link); 16-byte elements where both
// pointers allow, else 8-byte ones
__global__ void k_copy_host(const double *__restrict__ src, double *__restrict__ dst, size_t count)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x, t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
        const double2 *s2 = reinterpret_cast<const double2 *>(src);
        double2 *d2 = reinterpret_cast<double2 *>(dst);
        const size_t n2 = count / 2;
        size_t i = t;
        for (; i + 3 * stride < n2; i += 4 * stride) {
            const double2 a = s2[i], b = s2[i + stride], c = s2[i + 2 * stride], d = s2[i + 3 * stride];
            d2[i] = a; d2[i + stride] = b; d2[i + 2 * stride] = c; d2[i + 3 * stride] = d;
        }
        for (; i < n2; i += stride) d2[i] = s2[i];
        if (t == 0 && (count & 1)) dst[count - 1] = src[count - 1];
    } else {
        for (size_t i = t; i < count; i += stride) dst[i] = src[i];
    }
}

// the pass's counters into the host-side report (one block)
__global__ void k_pass_report(const int *cnt, const unsigned long long *wc, const int *depth_off, int ndepth_off,
                              const long long *mu_total, const int *mu_over, PassReport *out)
{
    const int t = threadIdx.x;
    if (t < ph::BC_NCOUNTERS) out->cnt[t] = cnt[t];
    if (t < ph::WC_N) out->wc[t] = wc[t];
    for (int i = t; i < ndepth_off; i += blockDim.x) out->depth_off[i] = depth_off[i];
    if (t == 0) {
        out->mu_need = mu_total ? *mu_total : 0;
        out->mu_over = mu_over ? *mu_over : 0;
        out->ndepth_off = ndepth_off;
    }
}

__global__ void k_gather_out(const int *perm, const double *ax, const double *ay, const double *az, int n, double *out,
                             int tree_order)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int o = tree_order ? i : perm[i];
        out[3 * o] = ax[i];
        out[3 * o + 1] = ay[i];
        out[3 * o + 2] = az[i];
    }
}

}  // namespace

// The device address of a host buffer of `bytes` bytes when the whole range
// is pinned host memory mapped for this device (cudaHostAlloc, or host
// memory registered with the runtime), else null.
static const void *mapped_host(const void *p, size_t bytes)
{
    if (!p || !bytes) return nullptr;
    cudaPointerAttributes a0, a1;
    const char *q = static_cast<const char *>(p);
    if (cudaPointerGetAttributes(&a0, q) != cudaSuccess || cudaPointerGetAttributes(&a1, q + bytes - 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
        return nullptr;
    if (static_cast<const char *>(a1.devicePointer) - static_cast<const char *>(a0.devicePointer) != (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a0.devicePointer;
}

// Host <-> device copies of a pass's positions and accelerations.  Pinned
// host buffers that the device addresses are copied by a kernel over the
// host link, at the copy engines' rate (211 / 193 GB/s at 256^3); the copy
// engines' own copies stall for tens of milliseconds a few times a second
// for minutes after another process has freed large device allocations,
// and the kernel's do not.  Other host memory goes through cudaMemcpyAsync.
static int ph_copy_host(photons_ctx *c, double *dst, const double *src, size_t count, bool to_device)
{
    const size_t bytes = sizeof(double) * count;
    const void *m = mapped_host(to_device ? static_cast<const void *>(src) : static_cast<const void *>(dst), bytes);
    if (!m) {
        PH_CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                                      c->stream));
        return 0;
    }
    const double *s = to_device ? static_cast<const double *>(m) : src;
    double *d = to_device ? dst : static_cast<double *>(const_cast<void *>(m));
    ph::note_launch(), k_copy_host<<<ph::device_sm_count() * 4, 512, 0, c->stream>>>(s, d, count);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// the context's pinned host report and a box staging area of >= nbox entries
static int ensure_host_link(photons_ctx *c, int nbox)
{
    void *d = nullptr;
    if (!c->ev_hlink) PH_CUDA_CHECK(cudaEventCreateWithFlags(&c->ev_hlink, cudaEventDisableTiming));
    if (!c->rep) {
        PH_CUDA_CHECK(cudaHostAlloc(reinterpret_cast<void **>(&c->rep), sizeof(PassReport),
                                    cudaHostAllocPortable | cudaHostAllocMapped));
        PH_CUDA_CHECK(cudaHostGetDevicePointer(&d, c->rep, 0));
        c->rep_dev = static_cast<PassReport *>(d);
    }
    if (c->hbox_cap < nbox) {
        PH_CUDA_CHECK(cudaEventSynchronize(c->ev_hlink));
        if (c->hbox) cudaFreeHost(c->hbox);
        c->hbox = nullptr;
        c->hbox_dev = nullptr;
        c->hbox_cap = 0;
        PH_CUDA_CHECK(cudaHostAlloc(reinterpret_cast<void **>(&c->hbox), sizeof(BoxParams) * (size_t)nbox,
                                    cudaHostAllocPortable | cudaHostAllocMapped));
        PH_CUDA_CHECK(cudaHostGetDevicePointer(&d, c->hbox, 0));
        c->hbox_dev = static_cast<BoxParams *>(d);
        c->hbox_cap = nbox;
    }
    return 0;
}

// the pass's counters into c->rep (read them after the stream has finished)
static int ph_enqueue_report(photons_ctx *c, int ndepth_off)
{
    PH_TRY(ensure_host_link(c, 1));
    ph::note_launch(), k_pass_report<<<1, 256, 0, c->stream>>>(c->b.cnt, c->w.ctr, c->t.depth_off, ndepth_off,
                                                                c->mu_total, c->mu_over, c->rep_dev);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// enqueue the report, wait for the stream, and read it: build counters,
// walk counters (into c->ws), depth offsets (levels + 2, into c->info) and
// the mutual kernel's reaction need and flag
static int ph_read_report(photons_ctx *c, int levels, int *h, long long *mu_need, int *mu_over)
{
    PH_TRY(ph_enqueue_report(c, levels + 2));
    PH_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    const PassReport *r = c->rep;
    memcpy(h, r->cnt, sizeof(int) * ph::BC_NCOUNTERS);
    memcpy(c->ws.c, r->wc, sizeof(c->ws.c));
    c->info.depth_off.assign(r->depth_off, r->depth_off + levels + 2);
    *mu_need = r->mu_need;
    *mu_over = r->mu_over;
    return 0;
}

// FP32 P2P kernel: 2 mutual pairs (the default; used for MAXLEAF 48-64),
// 0 packed one-way pairs, 1 scalar (PHOTONS_P2P_KERNEL=mutual|packed|scalar)
static int p2p_variant()
{
    const char *v = getenv("PHOTONS_P2P_KERNEL");
    if (v && !strcmp(v, "scalar")) return 1;
    if (v && !strcmp(v, "packed")) return 0;
    return 2;
}

// Test hook for the time limit of the bulk-staging waits: with
// PHOTONS_TEST_STAGE_SHORTFALL=1 each bulk copy's mbarrier is armed for 16
// bytes more than the copy brings, so every staging wait runs out (after
// two seconds) and the pass fails with an error; the context stays usable.
static int stage_shortfall()
{
    const char *v = getenv("PHOTONS_TEST_STAGE_SHORTFALL");
    return v && !strcmp(v, "1") ? 16 : 0;
}

// floats per reaction value: an FP64 pass keeps doubles in the float buffer
static long long mu_per_value(int precision) { return precision == PHOTONS_FP64 ? 2 : 1; }

// the reaction buffer of the mutual kernel (floats); grown from the last
// pass's need, which the device reports when it did not fit
// A reaction buffer that was too small made the pass evaluate every pair
// one way (correct, but not the mutual kernel's rounding); size it and
// report that the pass should be repeated, so results never depend on
// whether an earlier pass had already grown the buffer.
static bool mutual_feedback(photons_ctx *c, int over, long long need, int precision)
{
    if (!(over & 1) || need <= c->mu_buf_cap / mu_per_value(precision)) return false;
    c->hint_mubuf = need + need / 16 + 4096;
    return true;
}

// bit 1 of the mutual kernel's flag: a source-staging bulk copy did not
// land within the kernel's time limit, and the warps that waited stopped
static int mutual_status(int over)
{
    if (over & 2) return ph_set_error(PH_ERR_CUDA, "P2P source staging: a bulk copy did not complete in time");
    return 0;
}

// Mutual pairs from leaf size 48.  At leaf 32 they win on near-uniform
// input (256^3 Zel'dovich: 55 vs 69 ms) but lose on halos (128^3 NFW: 47 vs
// 30 ms: leaves of 22 particles fill 32 target slots, and 65 % of the
// entries sit in lists longer than the sort handles, evaluated one way);
// below 32 they lose everywhere.  On halo-dominated input the one-way
// kernel can win at 48-64 too (128^3 NFW leaf 48: 35 against 39 ms);
// PHOTONS_F_ONE_WAY selects it, and the leaf-size autotuner times both.
#ifndef MU_MIN_LEAF
#define MU_MIN_LEAF 48
#endif
// FP64 passes use mutual pairs at every leaf size: the pair force is ~70
// FP64 operations, so evaluating each symmetric pair once halves the pass
// whatever the pairing costs.
static bool uses_mutual(const photons_ctx *c, int precision)
{
    if (c->mu_off || (c->pass_flags & PHOTONS_F_ONE_WAY)) return false;
    if (precision == PHOTONS_FP64) return true;
    return p2p_variant() == 2 && c->pp.maxleaf >= MU_MIN_LEAF && c->pp.maxleaf <= 64;
}

// buffers of the mutual kernel, only for passes that run it: per-entry
// slots and packed entries (the P2P pool's capacity) and the reaction slots
static int alloc_mutual(photons_ctx *c, int precision)
{
    if (!uses_mutual(c, precision)) return 0;
    // first guess: about half of a leaf's ~110-250 list entries received, 3
    // floats per particle and entry (256^3 leaf 64 needs ~180 per particle);
    // a pass that needs more repeats once with the measured size
    long long want = (c->hint_mubuf ? c->hint_mubuf : (long long)c->n * 192 + 4096) * mu_per_value(precision);
    // the reaction slots take ~700 bytes per particle: where they would not
    // leave 1 GB of the device free, this context evaluates every pair one way
    size_t grow = 0, free_b = 0, total_b = 0;
    if (c->w.p2p_cap > c->mu_slot_cap) grow += (size_t)(c->w.p2p_cap - c->mu_slot_cap) * (2 * sizeof(int) + sizeof(int2));
    if (want > c->mu_buf_cap) grow += (size_t)(want - c->mu_buf_cap) * sizeof(float);
    if (grow && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && grow + ((size_t)1 << 30) > free_b) {
        c->mu_off = true;
        c->epoch++;
        return 0;
    }
    if (c->w.p2p_cap > c->mu_slot_cap) {
        c->mu_slot_cap = 0;
        c->epoch++;
        PH_TRY(dalloc(c->mu_slot, (size_t)c->w.p2p_cap));
        PH_TRY(dalloc(c->mu_ev, (size_t)c->w.p2p_cap));
        PH_TRY(dalloc(c->mu_pq, (size_t)c->w.p2p_cap));
        c->mu_slot_cap = c->w.p2p_cap;
        c->epoch++;
    }
    if (want > c->mu_buf_cap) {
        c->mu_buf_cap = 0;
        c->epoch++;
        PH_TRY(dalloc(c->mu_buf, (size_t)want));
        c->mu_buf_cap = want;
        c->epoch++;
    }
    return 0;
}

// ------------------------------------------------------------------
// stages
// ------------------------------------------------------------------
int ph_validate(const photons_params *p, int n)
{
    if (!p) return ph_set_error(PH_ERR_ARG, "null parameters");
    if (n < 1) return ph_set_error(PH_ERR_ARG, "particle count %d < 1", n);
    if (p->maxleaf < 1 || p->maxleaf > PH_MAX_LEAF)
        return ph_set_error(PH_ERR_ARG, "MAXLEAF %d outside [1, %d]", p->maxleaf, PH_MAX_LEAF);
    if (n <= p->maxleaf)
        return ph_set_error(PH_ERR_SMALL, "N=%d <= MAXLEAF=%d: the reference's image walk treats the root as a leaf "
                                          "and reads undefined bodies", n, p->maxleaf);
    if (!(p->boxsize > 0) || !(p->rs > 0) || !(p->rcut > 0) || !(p->eps >= 0) || !(p->theta >= 0) ||
        !std::isfinite(p->mass))
        return ph_set_error(PH_ERR_ARG, "invalid force parameters");
    if (p->precision != PHOTONS_FP32_SPLIT && p->precision != PHOTONS_FP64)
        return ph_set_error(PH_ERR_ARG, "unknown precision %d", p->precision);
    if (PHOTONS_F_SHAPE_OF(p->flags) >= PHOTONS_P2P_SHAPES)
        return ph_set_error(PH_ERR_ARG, "unknown P2P kernel shape %d", PHOTONS_F_SHAPE_OF(p->flags));
    // leaves + nodes are addressed with 27-bit ids in the lists: 2 x (2N/MAXLEAF) + 2 < 2^27
    if (2.0 * (2.0 * n / p->maxleaf) + 2.0 >= (double)PH_MAX_UNIFIED)
        return ph_set_error(PH_ERR_ARG, "N=%d with MAXLEAF=%d exceeds the 2^27 tree-id space", n, p->maxleaf);
    return 0;
}

// events inside a captured pass become event-record nodes of the graph
static int ph_record(photons_ctx *c, int ev)
{
    PH_CUDA_CHECK(cudaEventRecordWithFlags(c->ev[ev], c->stream,
                                           c->capturing ? cudaEventRecordExternal : cudaEventRecordDefault));
    return 0;
}

// node levels to launch for a context's first pass: mean splits roughly
// halve the count per level; clustered sets go deeper (PH_FLAG_DEPTH grows
// it).  PHOTONS_TREE_LEVELS sets the starting count instead.
static int estimate_levels(int n, int maxleaf)
{
    const char *e = getenv("PHOTONS_TREE_LEVELS");
    if (e && atoi(e) > 0) return atoi(e) < MAX_DEPTH_CAP - 1 ? atoi(e) : MAX_DEPTH_CAP - 1;
    int lv = 1;
    while (lv < 60 && (double)n / std::ldexp(1.0, lv) > (double)maxleaf) lv++;
    lv += 8;
    return lv < MAX_DEPTH_CAP - 1 ? lv : MAX_DEPTH_CAP - 1;
}

// levels of wide nodes (more than CHUNK_ELEMS particles) to launch: the
// last build's need with a margin, else an estimate from N; never above the
// depth bound
static int tree_top(const photons_ctx *c, int n, int levels)
{
    int top = c->hint_top;
    if (top <= 0) {
        top = 1;
        while (top < 60 && (double)n / std::ldexp(1.0, top) > (double)CHUNK_ELEMS) top++;
        top += 2;
    }
    return top < levels ? top : levels;
}

// validation, capacities and parameters of a pass over n particles
// the reference's 2N/MAXLEAF node and leaf capacity of one box (src/fmm.c:203-209)
static int box_cap(int n, int maxleaf)
{
    int cap = (int)(2.0 * ((double)n) / ((double)maxleaf));
    if (cap > n) cap = n + 1;
    if (cap < 1) cap = 1;
    return cap;
}

// the per-box constants every kernel reads (host side of BoxParams)
static BoxParams box_params(const photons_params *p, int first, int count)
{
    BoxParams B;
    memset(&B, 0, sizeof B);
    B.boxsize = p->boxsize;
    B.rs = p->rs;
    B.rcut = p->rcut;
    B.eps = p->eps;
    B.mass = p->mass;
    B.rcut2 = p->rcut * p->rcut;
    B.Lhi = (float)p->boxsize;
    B.Llo = (float)(p->boxsize - (double)B.Lhi);
    B.c2f = (float)(p->rcut * p->rcut);
    PassParams pp{};
    pp.boxsize = p->boxsize; pp.theta = p->theta; pp.rs = p->rs; pp.rcut = p->rcut; pp.eps = p->eps;
    pp.mass = p->mass; pp.maxleaf = p->maxleaf;
    const ph::SplitConsts k = ph::make_split_consts(pp);
    B.sig = k.sig;
    B.e2s = k.e2s;
    B.pias = k.pias;
    B.cs = k.cs;
    const double sig = ph::split_sig(pp);
    B.acc_scale = p->mass * sig * sig;
    const double ia = 0.5 / p->rs;
    B.far_a = (float)ia;
    B.far_pa = (float)(SPLIT_P * ia);
    B.first = first;
    B.count = count;
    B.root = -1;
    return B;
}

// Validation, capacities, the box table and the pass-wide parameters of a
// pass over nbox boxes (counts[b] particles each, concatenated).  Boxes may
// differ in side, rs, rcut, softening and mass; theta, MAXLEAF, precision,
// image mask and flags are those of the pass.
static int ph_prepare_boxes(photons_ctx *c, int nbox, const photons_params *p, const int *counts)
{
    if (nbox < 1 || !p || !counts) return ph_set_error(PH_ERR_ARG, "bad box list");
    long long n = 0, cap = 0;
    for (int b = 0; b < nbox; b++) {
        if (p[b].theta != p[0].theta || p[b].maxleaf != p[0].maxleaf || p[b].precision != p[0].precision ||
            p[b].image_mask != p[0].image_mask || p[b].flags != p[0].flags)
            return ph_set_error(PH_ERR_ARG, "box %d: theta, MAXLEAF, precision, image mask and flags must match "
                                            "those of box 0", b);
        PH_TRY(ph_validate(&p[b], counts[b]));
        n += counts[b];
        cap += box_cap(counts[b], p[b].maxleaf);
    }
    if (n > INT32_MAX / 3) return ph_set_error(PH_ERR_ARG, "%lld particles in one pass exceed the supported count", n);
    photons_params all = p[0];
    PH_TRY(ph_validate(&all, (int)n));  // the 27-bit id space over all boxes
    if (c->dom_set && nbox != 1) return ph_set_error(PH_ERR_ARG, "a rank's domain pass covers one box");
    PH_TRY(alloc_particles(c, (int)n + (c->dom_set ? c->imp_reserve_body : 0)));
    PH_TRY(alloc_tree(c, (int)n, (int)cap));
    if (nbox > c->cap_box) {
        c->cap_box = 0;
        c->epoch++;
        PH_TRY(dalloc(c->b.boxes, nbox));
        c->cap_box = nbox;
        c->epoch++;
    }
    c->h_boxes.resize(nbox);
    int first = 0;
    for (int b = 0; b < nbox; b++) {
        c->h_boxes[b] = box_params(&p[b], first, counts[b]);
        first += counts[b];
    }
    c->pp.axis0 = 0;
    if (c->dom_set) {
        // a rank's domain: the root's box and first split axis
        BoxParams &B = c->h_boxes[0];
        B.domain = 1;
        for (int d = 0; d < 3; d++) { B.dom_lo[d] = c->dom.lo[d]; B.dom_hi[d] = c->dom.hi[d]; }
        c->pp.axis0 = c->dom.axis;
    }
    c->b.nbox = nbox;
    c->b.rule_cap = (int)cap;
    c->pp.boxsize = p->boxsize;
    c->pp.theta = p->theta;
    c->pp.rs = p->rs;
    c->pp.rcut = p->rcut;
    c->pp.eps = p->eps;
    c->pp.mass = p->mass;
    c->pp.maxleaf = p->maxleaf;
    c->pp.images = 1;
    c->pass_flags = p->flags;
    c->n = (int)n;
    c->info.nleaf_cap = c->info.nnode_cap = (int)cap;
    c->have_tree = c->have_lists = c->have_multipoles = false;
    return 0;
}

// the box table for this pass (before the build; the build writes the roots)
// the box table, staged in pinned host memory and copied by a kernel (the
// staging is rewritten only after the last kernel that read it has run)
static int ph_upload_boxes(photons_ctx *c)
{
    const int nbox = (int)c->h_boxes.size();
    PH_TRY(ensure_host_link(c, nbox));
    PH_CUDA_CHECK(cudaEventSynchronize(c->ev_hlink));
    memcpy(c->hbox, c->h_boxes.data(), sizeof(BoxParams) * (size_t)nbox);
    static_assert(sizeof(BoxParams) % sizeof(double) == 0, "box table copied as doubles");
    ph::note_launch(), k_copy_host<<<1, 256, 0, c->stream>>>(reinterpret_cast<const double *>(c->hbox_dev),
                                                              reinterpret_cast<double *>(c->b.boxes),
                                                              sizeof(BoxParams) * (size_t)nbox / sizeof(double));
    PH_CUDA_CHECK(cudaGetLastError());
    PH_CUDA_CHECK(cudaEventRecord(c->ev_hlink, c->stream));
    return 0;
}

// tree build from device positions src (enqueue only)
static int ph_enqueue_tree(photons_ctx *c, const double *src, int levels)
{
    cudaStream_t st = c->stream;
    PH_TRY(ph::launch_init_particles(c->b, src, c->n, st));
    PH_TRY(ph::build_tree(c->b, c->t, c->pp, levels, tree_top(c, c->n, levels), st));
    PH_TRY(ph::launch_geom32(c->t, c->b.cnt, st));
    PH_TRY(ph::launch_leaf_offsets(c->b, c->t, c->pos4, st));
    c->ndepth = levels + 1;
    return ph_record(c, EV_TREE);
}

// build flags after the stream has finished: capacity overflow is an error
// of the reference's rule; PH_FLAG_TOP asks for more levels of wide nodes,
// PH_FLAG_DEPTH for a deeper bound (*grow: the bound to build again with)
static int ph_check_build(photons_ctx *c, int flags, int levels, int *grow)
{
    *grow = 0;
    if (flags & PH_FLAG_LEAF_CAPACITY)
        return ph_set_error(PH_ERR_CAPACITY, "leaf capacity 2N/MAXLEAF=%d exceeded by the mean-split tree", c->b.rule_cap);
    if (flags & PH_FLAG_NODE_CAPACITY)
        return ph_set_error(PH_ERR_CAPACITY, "node capacity 2N/MAXLEAF=%d exceeded by the mean-split tree", c->b.rule_cap);
    if (flags & (PH_FLAG_DEPTH | PH_FLAG_TOP)) {
        const int top = tree_top(c, c->n, levels);
        if (flags & PH_FLAG_TOP) c->hint_top = top * 2 > top + 4 ? top * 2 : top + 4;
        if (!(flags & PH_FLAG_DEPTH) && top < levels) {
            *grow = levels;
            return 0;
        }
        if (levels >= MAX_DEPTH_CAP - 1) return ph_set_error(PH_ERR_DEPTH, "tree deeper than %d levels", MAX_DEPTH_CAP - 1);
        *grow = levels * 2 < MAX_DEPTH_CAP - 1 ? levels * 2 : MAX_DEPTH_CAP - 1;
    }
    return 0;
}

static void ph_tree_info_from(photons_ctx *c, const int *h, int levels)
{
    c->info.nleaf = h[ph::BC_LEAVES];
    c->info.nnode = h[ph::BC_NODES];
    c->info.depth = h[ph::BC_DEPTH];
    c->info.levels = h[ph::BC_NLEVELS];
    c->info.flags = h[ph::BC_FLAGS];
    // keep the launch counts while they cover the tree with a small margin,
    // so repeated passes over similar trees reuse one captured graph: the
    // depth bound over the deepest depth, the levels of wide nodes over the
    // recorded levels (the last of them holds subtree roots only)
    const int lv = c->info.depth;
    if (levels < lv + 1 || levels > lv + 6) c->hint_levels = lv + 3;
    else c->hint_levels = levels;
    const int need = c->info.levels > 2 ? c->info.levels - 1 : 1, top = tree_top(c, c->n, levels);
    if (top < need || top > need + 4) c->hint_top = need + 2;
    else c->hint_top = top;
}

static int ph_stage_build_boxes(photons_ctx *c, int nbox, const photons_params *p, const int *counts,
                                const double *pos, int device_io)
{
    PH_TRY(ph_prepare_boxes(c, nbox, p, counts));
    const int n = c->n;
    cudaStream_t st = c->stream;
    PH_TRY(ph_upload_boxes(c));
    const double *src = pos;
    PH_TRY(ph_record(c, EV_START));
    if (!device_io) {
        PH_TRY(ph_copy_host(c, c->io, pos, (size_t)3 * n, true));
        src = c->io;
    }
    PH_TRY(ph_record(c, EV_UPLOADED));
    int levels = c->hint_levels ? c->hint_levels : estimate_levels(n, p->maxleaf);
    for (;;) {
        PH_TRY(ph_enqueue_tree(c, src, levels));
        PH_CUDA_CHECK(cudaStreamSynchronize(st));
        ph::TreeInfo info = c->info;
        PH_TRY(ph::read_tree_info(c->b, c->t, levels, info));
        int grow = 0;
        PH_TRY(ph_check_build(c, info.flags, levels, &grow));
        if (grow) { levels = grow; continue; }
        c->info.depth_off = info.depth_off;
        int h[ph::BC_NCOUNTERS] = {0};
        h[ph::BC_LEAVES] = info.nleaf;
        h[ph::BC_NODES] = info.nnode;
        h[ph::BC_DEPTH] = info.depth;
        h[ph::BC_NLEVELS] = info.levels;
        h[ph::BC_FLAGS] = info.flags;
        ph_tree_info_from(c, h, levels);
        c->ndepth = info.depth + 1;
        break;
    }
    c->have_tree = true;
    return 0;
}

int ph_stage_build(photons_ctx *c, const photons_params *p, int n, const double *pos, int device_io)
{
    return ph_stage_build_boxes(c, 1, p, &n, pos, device_io);
}

// list-pool sizes after an overflowed walk
static void grow_walk_caps(photons_ctx *c, unsigned long long fl, long long &p2p_cap, long long &pd_cap,
                           long long &m2l_cap, int &stack_cap, int &stage_cap)
{
    const unsigned long long *w = c->ws.c;
    if (fl & PH_FLAG_POOL_OVERFLOW) {
        long long need = (long long)w[ph::WC_P2P_FILL];
        if (need > c->w.p2p_cap) p2p_cap = need + need / 8 + 4096;
        need = (long long)w[ph::WC_PD_MAX];
        long long cur = (long long)w[ph::WC_PD_FILL0];
        if ((long long)w[ph::WC_PD_FILL1] > cur) cur = (long long)w[ph::WC_PD_FILL1];
        if (cur > need) need = cur;
        if (need > c->w.pd_cap) pd_cap = need + need / 8 + 4096;
        need = (long long)w[ph::WC_M2L_FILL];
        if (need > c->w.m2l_cap) m2l_cap = need + need / 8 + 4096;
    }
    if (fl & PH_FLAG_STACK_OVERFLOW) stack_cap = c->w.stack_cap * 4;
    if (fl & PH_FLAG_STAGE_OVERFLOW) {
        long long need = (long long)w[ph::WC_MAX_STAGE];
        stage_cap = (int)(need > 2LL * c->w.stage_cap ? need + 1024 : 2LL * c->w.stage_cap);
    }
}

static void walk_caps(photons_ctx *c, long long &p2p_cap, long long &pd_cap, long long &m2l_cap, int &stack_cap,
                      int &stage_cap)
{
    const long long n = c->n;
    // first-pass guesses: entries per particle fall as leaves grow (about
    // 130 list entries per target leaf at leaf 16-64); an overflow grows them
    const long long per = c->pp.maxleaf > 16 ? c->pp.maxleaf : 16;
    p2p_cap = c->hint_p2p ? c->hint_p2p : n * 32 * 16 / per + 4096;
    pd_cap = c->hint_pd ? c->hint_pd : n * 16 * 16 / per + 4096;
    m2l_cap = c->hint_m2l ? c->hint_m2l : n * 2 + 4096;
    stack_cap = c->w.stack_cap ? c->w.stack_cap : 4096;
    stage_cap = c->w.stage_cap ? c->w.stage_cap : 16384;
}

static void keep_walk_hints(photons_ctx *c, long long p2p_cap, long long pd_cap, long long m2l_cap)
{
    c->hint_p2p = p2p_cap;
    c->hint_pd = pd_cap;
    c->hint_m2l = m2l_cap;
}

int ph_stage_walk(photons_ctx *c, unsigned mask)
{
    if (!c->have_tree) return ph_set_error(PH_ERR_STATE, "no tree: run the build first");
    long long p2p_cap, pd_cap, m2l_cap;
    int stack_cap, stage_cap;
    walk_caps(c, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap);
    for (int attempt = 0; attempt < 6; attempt++) {
        PH_TRY(alloc_walk(c, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap));
        PH_TRY(ph::walk_lists(c->w, c->t, c->b.cnt, c->b.boxes, c->ndepth, c->pp, mask, c->stream, c->walk_imp));
        PH_CUDA_CHECK(cudaMemcpyAsync(c->ws.c, c->w.ctr, sizeof(c->ws.c), cudaMemcpyDeviceToHost, c->stream));
        PH_CUDA_CHECK(cudaStreamSynchronize(c->stream));
        unsigned long long fl = c->ws.c[ph::WC_FLAGS];
        if (!fl) {
            c->have_lists = true;
            c->mask = mask;
            keep_walk_hints(c, p2p_cap, pd_cap, m2l_cap);  // a repeated pass allocates once
            return ph_record(c, EV_WALK);
        }
        grow_walk_caps(c, fl, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap);
    }
    return ph_set_error(PH_ERR_CAPACITY, "interaction lists did not fit after repeated growth");
}

int ph_stage_p2p(photons_ctx *c, int precision, int zero)
{
    cudaStream_t st = c->stream;
    PH_TRY(alloc_mutual(c, precision));
    PH_CUDA_CHECK(cudaMemsetAsync(c->mu_over, 0, sizeof(int), st));
    PH_CUDA_CHECK(cudaMemsetAsync(c->mu_total, 0, sizeof(long long), st));
    const int n = c->n;
    if (zero) {
        PH_CUDA_CHECK(cudaMemsetAsync(c->ax, 0, sizeof(double) * n, st));
        PH_CUDA_CHECK(cudaMemsetAsync(c->ay, 0, sizeof(double) * n, st));
        PH_CUDA_CHECK(cudaMemsetAsync(c->az, 0, sizeof(double) * n, st));
    }
    ph::P2PArgs a;
    memset(&a, 0, sizeof a);
    a.ipart = c->t.ipart; a.npart = c->t.npart;
    a.cx = c->t.cx; a.cy = c->t.cy; a.cz = c->t.cz;
    a.tree_cnt = c->b.cnt;
    a.walk_flags = c->w.ctr + ph::WC_FLAGS;
    a.boxid = c->t.boxid;
    a.boxes = c->b.boxes;
    a.nbox = c->b.nbox;
    a.p2p_pool = c->w.p2p_pool; a.p2p_off = c->w.p2p_off; a.p2p_cnt = c->w.p2p_cnt;
    a.pos4 = c->pos4;
    a.chi = c->t.chi;
    a.clo = c->t.clo;
    a.px = c->b.x; a.py = c->b.y; a.pz = c->b.z;
    a.ax = c->ax; a.ay = c->ay; a.az = c->az;
    a.work_counter = c->work_counter;
    a.boxsize = c->pp.boxsize; a.eps = c->pp.eps; a.mass = c->pp.mass; a.rs = c->pp.rs;
    a.k = ph::make_split_consts(c->pp);
    a.variant = p2p_variant();
    a.shape = PHOTONS_F_SHAPE_OF(c->pass_flags);
    a.bulk = (c->pass_flags & PHOTONS_F_P2P_BULK) ? 1 : 0;
    a.stage_extra = stage_shortfall();
    PH_TRY(ph_record(c, EV_P2P_BEGIN));
    if (uses_mutual(c, precision)) {
        ph::MutualBufs m;
        m.pool = c->w.p2p_pool;
        m.sorted = c->mu_sorted; m.nrecv = c->mu_nrecv; m.size = c->mu_size; m.rbase = c->mu_rbase;
        m.total = c->mu_total; m.scan_scratch = c->mu_scan; m.slot = c->mu_slot; m.over = c->mu_over;
        m.ev = c->mu_ev; m.nev = c->mu_nev; m.maxleaf = c->pp.maxleaf; m.pq = c->mu_pq;
        m.buf = c->mu_buf; m.buf_cap = c->mu_buf_cap / mu_per_value(precision); m.cap_leaves = c->mu_cap_leaves;
        PH_TRY(ph::launch_p2p_mutual(a, m, precision == PHOTONS_FP64, st));
    } else {
        if (a.variant == 2) a.variant = 0;
        PH_TRY(ph::launch_p2p(a, precision == PHOTONS_FP64, st));
    }
    return ph_record(c, EV_P2P);
}

static ph::MultipoleArgs multipole_args(photons_ctx *c)
{
    ph::MultipoleArgs a;
    memset(&a, 0, sizeof a);
    a.px = c->b.x; a.py = c->b.y; a.pz = c->b.z;
    a.ipart = c->t.ipart; a.npart = c->t.npart; a.son0 = c->t.son0; a.son1 = c->t.son1; a.parent = c->t.parent;
    a.cx = c->t.cx; a.cy = c->t.cy; a.cz = c->t.cz;
    a.tree_cnt = c->b.cnt;
    a.walk_flags = c->w.ctr + ph::WC_FLAGS;
    a.ndepth = c->ndepth;
    a.depth_list = c->t.depth_list;
    a.depth_off = c->t.depth_off;
    a.m2l_pool = c->w.m2l_pool; a.m2l_off = c->w.m2l_off; a.m2l_cnt = c->w.m2l_cnt;
    a.M = c->M; a.L = c->L;
    a.chi = c->t.chi; a.clo = c->t.clo; a.pos4 = c->pos4;
    a.ax = c->ax; a.ay = c->ay; a.az = c->az;
    a.boxid = c->t.boxid;
    a.boxes = c->b.boxes;
    a.work = c->work_counter + 1;
    a.gate_m = c->capturing ? c->far_gate : nullptr;
    a.gate_l = c->capturing ? c->far_gate + 1 : nullptr;
    return a;
}

int ph_stage_multipoles(photons_ctx *c)
{
    ph::MultipoleArgs a = multipole_args(c);
    PH_TRY(ph::run_p2m_m2m(a, c->stream));
    c->have_multipoles = true;
    return 0;
}

int ph_stage_m2l(photons_ctx *c, int precision)
{
    ph::MultipoleArgs a = multipole_args(c);
    if (precision == PHOTONS_FP32_SPLIT) return ph::run_m2l_f32(a, c->M32, c->stream);
    return ph::run_m2l(a, c->stream);
}

int ph_stage_downward(photons_ctx *c, int precision)
{
    ph::MultipoleArgs a = multipole_args(c);
    if (precision == PHOTONS_FP32_SPLIT) return ph::run_downward_f32(a, c->stream);
    return ph::run_downward(a, c->stream);
}

// accelerations from tree order into dst (input order unless tree_order)
static int ph_enqueue_gather(photons_ctx *c, double *dst, int tree_order)
{
    int blocks = ph::device_sm_count() * 8;
    ph::note_launch(), k_gather_out<<<blocks, 256, 0, c->stream>>>(c->b.perm, c->ax, c->ay, c->az, c->n, dst,
                                                                    tree_order);
    PH_CUDA_CHECK(cudaGetLastError());
    return ph_record(c, EV_GATHERED);
}

int ph_stage_output(photons_ctx *c, double *acc, int device_io, int tree_order)
{
    PH_TRY(ph_enqueue_gather(c, device_io ? acc : c->io, tree_order));
    if (!device_io) PH_TRY(ph_copy_host(c, acc, c->io, (size_t)3 * c->n, false));
    return ph_record(c, EV_END);
}

// ------------------------------------------------------------------
// the whole pass as one CUDA graph
// ------------------------------------------------------------------
static PassKey pass_key(photons_ctx *c, const photons_params *p, int n, const double *pos, double *acc, int dio,
                        int levels, unsigned mask)
{
    PassKey k;
    memset(&k, 0, sizeof k);
    k.n = n; k.nbox = c->b.nbox; k.levels = levels; k.top = tree_top(c, n, levels); k.maxleaf = p->maxleaf; k.precision = p->precision; k.flags = p->flags;
    k.dio = dio; k.variant = p2p_variant(); k.nwarps = c->w.nwarps; k.mask = mask;
    k.stage_extra = stage_shortfall();
    k.boxsize = p->boxsize; k.theta = p->theta; k.rs = p->rs; k.rcut = p->rcut; k.eps = p->eps; k.mass = p->mass;
    k.pos = dio ? (const void *)pos : nullptr;
    k.acc = dio ? (const void *)acc : nullptr;
    k.stream = c->stream;
    k.epoch = c->epoch;
    return k;
}

// device part of a pass: positions already in src, accelerations to dst
static int ph_enqueue_pass(photons_ctx *c, const photons_params *p, const double *src, double *dst, int levels,
                           unsigned mask)
{
    PH_TRY(ph_enqueue_tree(c, src, levels));
    PH_TRY(ph::walk_lists(c->w, c->t, c->b.cnt, c->b.boxes, c->ndepth, c->pp, mask, c->stream));
    PH_TRY(ph_record(c, EV_WALK));
    PH_TRY(ph_stage_p2p(c, p->precision, 1));
    const bool far = !(p->flags & PHOTONS_F_NO_FARFIELD);
    // the far field runs only if the walk made an M2L task (decided on the
    // device); multipoles also when the caller keeps them
    if (far || (p->flags & PHOTONS_F_MULTIPOLES))
        PH_TRY(ph::launch_far_gate(c->w.ctr, (p->flags & PHOTONS_F_MULTIPOLES) ? 1 : 0, c->far_gate, c->stream));
    if (far) {
        PH_TRY(ph_stage_multipoles(c));
        PH_TRY(ph_stage_m2l(c, p->precision));
        PH_TRY(ph_stage_downward(c, p->precision));
    } else if (p->flags & PHOTONS_F_MULTIPOLES) {
        PH_TRY(ph_stage_multipoles(c));
    }
    PH_TRY(ph_record(c, EV_FAR));
    return ph_enqueue_gather(c, dst, p->flags & PHOTONS_F_TREE_ORDER);
}

static void drop_graph(photons_ctx *c)
{
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    c->have_key = false;
}

static int capture_pass(photons_ctx *c, const photons_params *p, const double *src, double *dst, int levels,
                        unsigned mask)
{
    drop_graph(c);
    cudaStream_t st = c->stream;
    PH_CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    // kernels are counted when the graph runs, not when it is captured
    unsigned long long tally = 0;
    ph::t_capture_tally = &tally;
    int rc = ph_enqueue_pass(c, p, src, dst, levels, mask);
    ph::t_capture_tally = nullptr;
    c->graph_kernels = tally;
    c->capturing = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (!rc && e != cudaSuccess) rc = ph_set_cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    if (!rc) {
        e = cudaGraphInstantiate(&c->gexec, g, 0);
        if (e != cudaSuccess) {
            c->gexec = nullptr;
            rc = ph_set_cuda_error(e, "cudaGraphInstantiate", __FILE__, __LINE__);
        }
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
}

// The per-box constants live in the device box table, uploaded before each
// launch, so a captured graph serves any boxes with the same count and sizes.
static int force_pass_graph(photons_ctx *c, int nbox, const photons_params *p, const int *counts, const double *pos,
                            double *acc, int dio, unsigned mask)
{
    PH_TRY(ph_prepare_boxes(c, nbox, p, counts));
    const int n = c->n;
    cudaStream_t st = c->stream;
    int levels = c->hint_levels ? c->hint_levels : estimate_levels(n, p->maxleaf);
    long long p2p_cap, pd_cap, m2l_cap;
    int stack_cap, stage_cap;
    walk_caps(c, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap);
    const double *src = dio ? pos : c->io;
    double *dst = dio ? acc : c->io;
    for (int attempt = 0; attempt < 16; attempt++) {
        PH_TRY(alloc_walk(c, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap));
        PH_TRY(alloc_mutual(c, p->precision));
        PassKey k = pass_key(c, p, n, pos, acc, dio, levels, mask);
        if (!c->gexec || !c->have_key || memcmp(&k, &c->key, sizeof k) != 0) {
            PH_TRY(capture_pass(c, p, src, dst, levels, mask));
            c->key = k;
            c->have_key = true;
        }
        PH_CUDA_CHECK(cudaEventRecord(c->ev[EV_START], st));
        PH_TRY(ph_upload_boxes(c));
        if (!dio) PH_TRY(ph_copy_host(c, c->io, pos, (size_t)3 * n, true));
        PH_CUDA_CHECK(cudaEventRecord(c->ev[EV_UPLOADED], st));
        PH_CUDA_CHECK(cudaGraphLaunch(c->gexec, st));
        ph::g_launches += c->graph_kernels;
        if (!dio) PH_TRY(ph_copy_host(c, acc, c->io, (size_t)3 * n, false));
        PH_CUDA_CHECK(cudaEventRecord(c->ev[EV_END], st));
        int h[ph::BC_NCOUNTERS];
        long long mu_need = 0;
        int mu_over = 0;
        PH_TRY(ph_read_report(c, levels, h, &mu_need, &mu_over));
        int grow = 0;
        PH_TRY(ph_check_build(c, h[ph::BC_FLAGS], levels, &grow));
        if (grow) { levels = grow; continue; }
        ph_tree_info_from(c, h, levels);
        c->have_tree = true;
        unsigned long long fl = c->ws.c[ph::WC_FLAGS];
        if (fl) {
            grow_walk_caps(c, fl, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap);
            continue;
        }
        PH_TRY(mutual_status(mu_over));
        // the reaction total means something only once tree and lists are complete
        if (mutual_feedback(c, mu_over, mu_need, p->precision)) continue;
        c->info.depth_off.resize(c->info.depth + 2);
        c->have_lists = true;
        c->mask = mask;
        const bool any_m2l = c->ws.c[ph::WC_M2L_LOCAL] + c->ws.c[ph::WC_M2L_IMAGE] > 0;
        c->have_multipoles = (!(p->flags & PHOTONS_F_NO_FARFIELD) && any_m2l) || (p->flags & PHOTONS_F_MULTIPOLES);
        keep_walk_hints(c, p2p_cap, pd_cap, m2l_cap);
        return 0;
    }
    return ph_set_error(PH_ERR_CAPACITY, "force pass did not fit after repeated growth");
}

// ------------------------------------------------------------------
// one kick-drift-kick step as one captured graph
// ------------------------------------------------------------------
namespace {

// 1 when the pass just run did not fit (tree capacity, depth or levels,
// walk pools, or a reaction buffer too small for its mutual pairs): the
// captured step's second kick then leaves the velocities alone
__global__ void k_pass_failed(const int *tree_cnt, const unsigned long long *walk_ctr, const int *mu_over, int *out)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *out = (tree_cnt[ph::BC_FLAGS] & (PH_FLAG_LEAF_CAPACITY | PH_FLAG_NODE_CAPACITY | PH_FLAG_DEPTH | PH_FLAG_TOP)) ||
               walk_ctr[ph::WC_FLAGS] != 0 || *mu_over != 0;
}

}  // namespace

static int capture_kdk(photons_ctx *c, const photons_params *q, int n, double *pos, double *vel, double *acc,
                       int levels, unsigned mask)
{
    if (c->kexec) cudaGraphExecDestroy(c->kexec);
    c->kexec = nullptr;
    c->have_kkey = false;
    cudaStream_t st = c->stream;
    PH_CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    unsigned long long tally = 0;
    ph::t_capture_tally = &tally;
    int rc = ph_enqueue_kick_dev(n, vel, acc, c->kdk_f, nullptr, st);
    if (!rc) rc = ph_enqueue_drift_dev(n, pos, vel, c->kdk_f + 1, q->boxsize, st);
    if (!rc) rc = ph_enqueue_pass(c, q, pos, acc, levels, mask);
    if (!rc) {
        ph::note_launch(), k_pass_failed<<<1, 1, 0, st>>>(c->b.cnt, c->w.ctr, c->mu_over, c->kdk_skip);
        if (cudaGetLastError() != cudaSuccess) rc = ph_set_error(PH_ERR_CUDA, "k_pass_failed launch");
    }
    if (!rc) rc = ph_enqueue_kick_dev(n, vel, acc, c->kdk_f, c->kdk_skip, st);
    ph::t_capture_tally = nullptr;
    c->kdk_kernels = tally;
    c->capturing = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (!rc && e != cudaSuccess) rc = ph_set_cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    if (!rc) {
        e = cudaGraphInstantiate(&c->kexec, g, 0);
        if (e != cudaSuccess) {
            c->kexec = nullptr;
            rc = ph_set_cuda_error(e, "cudaGraphInstantiate", __FILE__, __LINE__);
        }
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
}

// The step runs as one graph (kick, drift, the pass, the second kick) once
// the pass has a captured graph whose key matches this one's: its
// capacities fitted the last pass over these arrays.  Should this pass not
// fit after all (particles moved), the second kick stops itself on the
// device and the caller repeats the pass the usual way, with growth and
// retries, then kicks; the first kick and the drift are never repeated.
int ph_kdk_graph_step(photons_ctx *c, const photons_params *q, int n, double *pos, double *vel, double *acc,
                      double dkh, double dd, int *done)
{
    *done = KDK_NOT_RUN;
    const char *genv = getenv("PHOTONS_GRAPH");
    if ((genv && !strcmp(genv, "0")) || n <= 0 || !pos || !vel || !acc) return 0;
    c->dom_set = false;
    c->walk_imp = ph::WalkImports();
    PH_TRY(ph_prepare_boxes(c, 1, q, &n));
    const unsigned mask = q->image_mask ? q->image_mask : ((1u << PH_NIMG) - 1u);
    const int levels = c->hint_levels ? c->hint_levels : estimate_levels(n, q->maxleaf);
    long long p2p_cap, pd_cap, m2l_cap;
    int stack_cap, stage_cap;
    walk_caps(c, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap);
    PH_TRY(alloc_walk(c, p2p_cap, pd_cap, m2l_cap, stack_cap, stage_cap));
    PH_TRY(alloc_mutual(c, q->precision));
    const PassKey k = pass_key(c, q, n, pos, acc, 1, levels, mask);
    if (!c->gexec || !c->have_key || memcmp(&k, &c->key, sizeof k) != 0) return 0;
    if (!c->kdk_f) { PH_TRY(dalloc(c->kdk_f, 2)); c->have_kkey = false; }
    if (!c->kdk_skip) { PH_TRY(dalloc(c->kdk_skip, 1)); c->have_kkey = false; }
    cudaStream_t st = c->stream;
    if (!c->kexec || !c->have_kkey || memcmp(&k, &c->kkey, sizeof k) != 0 || c->kkey_vel != vel ||
        c->kkey_box != q->boxsize) {
        PH_TRY(capture_kdk(c, q, n, pos, vel, acc, levels, mask));
        c->kkey = k;
        c->kkey_vel = vel;
        c->kkey_box = q->boxsize;
        c->have_kkey = true;
    }
    // the factors through the pinned staging, copied by a kernel
    PH_TRY(ensure_host_link(c, 1));
    PH_CUDA_CHECK(cudaEventSynchronize(c->ev_hlink));
    c->rep->kdk_f[0] = dkh;
    c->rep->kdk_f[1] = dd;
    const double *fdev = reinterpret_cast<const double *>(reinterpret_cast<const char *>(c->rep_dev) +
                                                           offsetof(PassReport, kdk_f));
    ph::note_launch(), k_copy_host<<<1, 32, 0, st>>>(fdev, c->kdk_f, 2);
    PH_CUDA_CHECK(cudaGetLastError());
    PH_CUDA_CHECK(cudaEventRecord(c->ev_hlink, st));
    PH_CUDA_CHECK(cudaEventRecord(c->ev[EV_START], st));
    PH_TRY(ph_upload_boxes(c));
    PH_CUDA_CHECK(cudaEventRecord(c->ev[EV_UPLOADED], st));
    PH_CUDA_CHECK(cudaGraphLaunch(c->kexec, st));
    ph::g_launches += c->kdk_kernels;
    PH_CUDA_CHECK(cudaEventRecord(c->ev[EV_END], st));
    int h[ph::BC_NCOUNTERS];
    long long mu_need = 0;
    int mu_over = 0;
    PH_TRY(ph_read_report(c, levels, h, &mu_need, &mu_over));
    int grow = 0;
    PH_TRY(ph_check_build(c, h[ph::BC_FLAGS], levels, &grow));
    const unsigned long long fl = c->ws.c[ph::WC_FLAGS];
    if (grow || fl) {
        // the caller's pass grows what did not fit (its own checks repeat these)
        *done = KDK_PASS_AGAIN;
        return 0;
    }
    PH_TRY(mutual_status(mu_over));
    if (mu_over) {
        mutual_feedback(c, mu_over, mu_need, q->precision);
        *done = KDK_PASS_AGAIN;
        return 0;
    }
    ph_tree_info_from(c, h, levels);
    c->have_tree = true;
    c->info.depth_off.resize(c->info.depth + 2);
    c->have_lists = true;
    c->mask = mask;
    const bool any_m2l = c->ws.c[ph::WC_M2L_LOCAL] + c->ws.c[ph::WC_M2L_IMAGE] > 0;
    c->have_multipoles = (!(q->flags & PHOTONS_F_NO_FARFIELD) && any_m2l) || (q->flags & PHOTONS_F_MULTIPOLES);
    c->last_flags = q->flags;
    c->precision = q->precision;
    *done = KDK_DONE;
    return 0;
}

// ------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------
extern "C" photons_ctx *photons_create(int device)
{
    photons_gpu_clear_error();
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        ph_set_error(PH_ERR_CUDA, "cannot use CUDA device %d", device);
        return nullptr;
    }
    photons_ctx *c = new photons_ctx();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        ph_set_error(PH_ERR_CUDA, "stream creation failed");
        delete c;
        return nullptr;
    }
    c->stream = c->own_stream;
    for (int i = 0; i < EV_COUNT; i++) cudaEventCreate(&c->ev[i]);
    return c;
}

extern "C" void photons_destroy(photons_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->kexec) cudaGraphExecDestroy(c->kexec);
    cudaFree(c->kdk_f);
    cudaFree(c->kdk_skip);
    if (c->rep) cudaFreeHost(c->rep);
    if (c->hbox) cudaFreeHost(c->hbox);
    if (c->ev_hlink) cudaEventDestroy(c->ev_hlink);
    ph_pm_release(c);
    ph_domain_release(c);
    cudaFree(c->pm_io);
    free_all(c);
    for (int i = 0; i < EV_COUNT; i++) cudaEventDestroy(c->ev[i]);
    cudaStreamDestroy(c->own_stream);
    delete c;
}

extern "C" int photons_set_stream(photons_ctx *c, void *stream)
{
    if (!c) return ph_set_error(PH_ERR_ARG, "null context");
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return 0;
}

static int force_pass_boxes(photons_ctx *c, int nbox, const photons_params *p, const int *counts, const double *pos,
                            double *acc)
{
    photons_gpu_clear_error();
    if (!c) return ph_set_error(PH_ERR_ARG, "null context");
    if (!pos || !acc) return ph_set_error(PH_ERR_ARG, "null particle arrays");
    if (!p || !counts || nbox < 1) return ph_set_error(PH_ERR_ARG, "null parameters");
    cudaSetDevice(c->device);
    // a plain pass covers the whole periodic box (no rank's domain, nothing received)
    c->dom_set = false;
    c->walk_imp = ph::WalkImports();
    const int dio = p->flags & PHOTONS_F_DEVICE_IO;
    const unsigned mask = p->image_mask ? p->image_mask : ((1u << PH_NIMG) - 1u);
    const char *g = getenv("PHOTONS_GRAPH");
    if (!(g && !strcmp(g, "0"))) {
        PH_TRY(force_pass_graph(c, nbox, p, counts, pos, acc, dio, mask));
    } else {
        // stage by stage, with the host checking the build and the walk; a second
        // attempt only when the mutual kernel's reaction buffer had to grow
        for (int attempt = 0; attempt < 2; attempt++) {
            PH_TRY(ph_stage_build_boxes(c, nbox, p, counts, pos, dio));
            PH_TRY(ph_stage_walk(c, mask));
            PH_TRY(ph_stage_p2p(c, p->precision, 1));
            const bool far = !(p->flags & PHOTONS_F_NO_FARFIELD);
            const unsigned long long nm2l = c->ws.c[ph::WC_M2L_LOCAL] + c->ws.c[ph::WC_M2L_IMAGE];
            if (far && (nm2l > 0 || (p->flags & PHOTONS_F_MULTIPOLES))) {
                PH_TRY(ph_stage_multipoles(c));
                PH_TRY(ph_stage_m2l(c, p->precision));
                PH_TRY(ph_stage_downward(c, p->precision));
            } else if (p->flags & PHOTONS_F_MULTIPOLES) {
                PH_TRY(ph_stage_multipoles(c));
            }
            PH_TRY(ph_record(c, EV_FAR));
            PH_TRY(ph_stage_output(c, acc, dio, p->flags & PHOTONS_F_TREE_ORDER));
            PH_CUDA_CHECK(cudaStreamSynchronize(c->stream));
            long long mu_need = 0;
            int mu_over = 0;
            PH_CUDA_CHECK(cudaMemcpy(&mu_need, c->mu_total, sizeof mu_need, cudaMemcpyDeviceToHost));
            PH_CUDA_CHECK(cudaMemcpy(&mu_over, c->mu_over, sizeof mu_over, cudaMemcpyDeviceToHost));
            PH_TRY(mutual_status(mu_over));
            if (!mutual_feedback(c, mu_over, mu_need, p->precision)) break;
        }
    }
    c->last_flags = p->flags;
    c->precision = p->precision;
    return 0;
}

extern "C" int photons_force_pass(photons_ctx *c, const photons_params *p, int n, const double *pos, double *acc)
{
    return force_pass_boxes(c, 1, p, &n, pos, acc);
}

extern "C" int photons_force_pass_boxes(photons_ctx *c, int nbox, const photons_params *params, const int *counts,
                                        const double *pos, double *acc)
{
    return force_pass_boxes(c, nbox, params, counts, pos, acc);
}

extern "C" int photons_get_counters(photons_ctx *c, long long *out, int n)
{
    if (!c || !out) return ph_set_error(PH_ERR_ARG, "null argument");
    const unsigned long long *w = c->ws.c;
    long long v[32] = {0};
    v[0] = (long long)w[ph::WC_P2P_LOCAL];
    v[1] = (long long)w[ph::WC_M2L_LOCAL];
    v[2] = (long long)(w[ph::WC_M2L_LOCAL] + w[ph::WC_M2L_IMAGE]);
    v[3] = (long long)w[ph::WC_PAIRS_IMAGE];
    v[4] = c->info.nleaf_cap;
    v[5] = c->info.nnode_cap;
    v[6] = c->info.nleaf;
    v[7] = c->info.nnode;
    v[8] = c->n;
    v[9] = (long long)c->n + c->info.nleaf_cap;
    v[10] = 0;
    v[11] = (long long)w[ph::WC_P2P_LOCAL];
    v[12] = (long long)w[ph::WC_M2L_LOCAL];
    v[13] = (long long)w[ph::WC_P2P_IMAGE];
    v[14] = (long long)w[ph::WC_M2L_IMAGE];
    int nimg = 0;
    for (int i = 1; i < PH_NIMG; i++) nimg += (c->mask >> i) & 1;
    v[15] = nimg;
    v[16] = (long long)w[ph::WC_PAIRS_LOCAL];
    v[17] = (long long)w[ph::WC_PAIRS_IMAGE];
    v[18] = c->info.depth;
    v[19] = (long long)w[ph::WC_MAX_STACK];
    v[20] = (long long)w[ph::WC_MAX_STAGE];
    v[21] = (long long)std::max(w[ph::WC_PD_MAX], std::max(w[ph::WC_PD_FILL0], w[ph::WC_PD_FILL1]));
    v[22] = (long long)w[ph::WC_P2P_FILL];
    v[23] = (long long)w[ph::WC_M2L_FILL];
    for (int i = 0; i < n && i < 32; i++) out[i] = v[i];
    return 0;
}

extern "C" int photons_get_timings(photons_ctx *c, float *ms, int n)
{
    if (!c || !ms) return ph_set_error(PH_ERR_ARG, "null argument");
    float v[8] = {0};
    cudaEventElapsedTime(&v[0], c->ev[EV_START], c->ev[EV_END]);
    cudaEventElapsedTime(&v[1], c->ev[EV_START], c->ev[EV_UPLOADED]);
    cudaEventElapsedTime(&v[2], c->ev[EV_UPLOADED], c->ev[EV_TREE]);
    cudaEventElapsedTime(&v[3], c->ev[EV_TREE], c->ev[EV_WALK]);
    cudaEventElapsedTime(&v[4], c->ev[EV_P2P_BEGIN], c->ev[EV_P2P]);
    cudaEventElapsedTime(&v[5], c->ev[EV_P2P], c->ev[EV_FAR]);
    cudaEventElapsedTime(&v[6], c->ev[EV_GATHERED], c->ev[EV_END]);
    cudaGetLastError();
    for (int i = 0; i < n && i < 8; i++) ms[i] = v[i];
    return 0;
}

extern "C" int photons_get_perm(photons_ctx *c, int *perm)
{
    if (!c || !perm || !c->have_tree) return ph_set_error(PH_ERR_STATE, "no tree");
    PH_CUDA_CHECK(cudaMemcpy(perm, c->b.perm, sizeof(int) * c->n, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int photons_get_positions(photons_ctx *c, double *pos)
{
    if (!c || !pos || !c->have_tree) return ph_set_error(PH_ERR_STATE, "no tree");
    std::vector<double> x(c->n), y(c->n), z(c->n);
    PH_CUDA_CHECK(cudaMemcpy(x.data(), c->b.x, sizeof(double) * c->n, cudaMemcpyDeviceToHost));
    PH_CUDA_CHECK(cudaMemcpy(y.data(), c->b.y, sizeof(double) * c->n, cudaMemcpyDeviceToHost));
    PH_CUDA_CHECK(cudaMemcpy(z.data(), c->b.z, sizeof(double) * c->n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < c->n; i++) { pos[3 * i] = x[i]; pos[3 * i + 1] = y[i]; pos[3 * i + 2] = z[i]; }
    return 0;
}

// host copy of the unified tree
int ph_download_tree(photons_ctx *c, HostTree &h, bool with_expansions)
{
    int nu = c->info.nleaf + c->info.nnode;
    h.nleaf = c->info.nleaf;
    h.nnode = c->info.nnode;
    h.ipart.resize(nu); h.npart.resize(nu); h.son0.resize(nu); h.son1.resize(nu); h.parent.resize(nu);
    h.cx.resize(nu); h.cy.resize(nu); h.cz.resize(nu); h.wx.resize(nu); h.wy.resize(nu); h.wz.resize(nu);
    h.split.resize(nu);
#define DL(dst, src, T) PH_CUDA_CHECK(cudaMemcpy(dst.data(), src, sizeof(T) * nu, cudaMemcpyDeviceToHost))
    DL(h.ipart, c->t.ipart, int); DL(h.npart, c->t.npart, int); DL(h.son0, c->t.son0, int);
    DL(h.son1, c->t.son1, int); DL(h.parent, c->t.parent, int);
    DL(h.cx, c->t.cx, double); DL(h.cy, c->t.cy, double); DL(h.cz, c->t.cz, double);
    DL(h.wx, c->t.wx, double); DL(h.wy, c->t.wy, double); DL(h.wz, c->t.wz, double);
    DL(h.split, c->t.split, double);
#undef DL
    if (with_expansions) {
        h.M.assign((size_t)nu * PH_NMULTI, 0.0);
        h.L.assign((size_t)nu * PH_NMULTI, 0.0);
        if (c->have_multipoles) {
            PH_CUDA_CHECK(cudaMemcpy(h.M.data(), c->M, sizeof(double) * PH_NMULTI * nu, cudaMemcpyDeviceToHost));
            PH_CUDA_CHECK(cudaMemcpy(h.L.data(), c->L, sizeof(double) * PH_NMULTI * nu, cudaMemcpyDeviceToHost));
        }
    }
    return 0;
}

// unified id -> the reference's index space
static inline int ref_id(const photons_ctx *c, int u)
{
    return u < c->info.nleaf ? c->n + u : c->n + c->info.nleaf_cap + (u - c->info.nleaf);
}

extern "C" int photons_copy_leaves(photons_ctx *c, int *ip_np, double *geom, double *M, double *L)
{
    if (!c || !c->have_tree) return ph_set_error(PH_ERR_STATE, "no tree");
    HostTree h;
    PH_TRY(ph_download_tree(c, h, true));
    for (int u = 0; u < h.nleaf; u++) {
        if (ip_np) { ip_np[2 * u] = h.ipart[u]; ip_np[2 * u + 1] = h.npart[u]; }
        if (geom) {
            double *g = geom + 6 * u;
            g[0] = h.cx[u]; g[1] = h.cy[u]; g[2] = h.cz[u]; g[3] = h.wx[u]; g[4] = h.wy[u]; g[5] = h.wz[u];
        }
        for (int m = 0; m < PH_NMULTI; m++) {
            if (M) M[PH_NMULTI * u + m] = h.M[(size_t)u * PH_NMULTI + m];
            if (L) L[PH_NMULTI * u + m] = h.L[(size_t)u * PH_NMULTI + m];
        }
    }
    return 0;
}

extern "C" int photons_copy_nodes(photons_ctx *c, int *info, double *geom, double *M, double *L)
{
    if (!c || !c->have_tree) return ph_set_error(PH_ERR_STATE, "no tree");
    HostTree h;
    PH_TRY(ph_download_tree(c, h, true));
    for (int k = 0; k < h.nnode; k++) {
        int u = h.nleaf + k;
        if (info) {
            info[3 * k] = h.npart[u];
            info[3 * k + 1] = ref_id(c, h.son0[u]);
            info[3 * k + 2] = ref_id(c, h.son1[u]);
        }
        if (geom) {
            double *g = geom + 7 * k;
            g[0] = h.split[u];
            g[1] = h.cx[u]; g[2] = h.cy[u]; g[3] = h.cz[u]; g[4] = h.wx[u]; g[5] = h.wy[u]; g[6] = h.wz[u];
        }
        for (int m = 0; m < PH_NMULTI; m++) {
            if (M) M[PH_NMULTI * k + m] = h.M[(size_t)u * PH_NMULTI + m];
            if (L) L[PH_NMULTI * k + m] = h.L[(size_t)u * PH_NMULTI + m];
        }
    }
    return 0;
}

// lists in the reference's index space, grouped by target
static int collect_lists(photons_ctx *c, int kind, std::vector<int> *t, std::vector<int> *s, std::vector<int> *im,
                         long long *count)
{
    if (!c || !c->have_lists) return ph_set_error(PH_ERR_STATE, "no lists");
    int nu = c->info.nleaf + c->info.nnode;
    bool p2p = (kind == 0 || kind == 2);
    bool want_image = (kind >= 2);
    std::vector<long long> off(nu);
    std::vector<int> cnt(nu);
    PH_CUDA_CHECK(cudaMemcpy(off.data(), p2p ? c->w.p2p_off : c->w.m2l_off, sizeof(long long) * nu,
                             cudaMemcpyDeviceToHost));
    PH_CUDA_CHECK(cudaMemcpy(cnt.data(), p2p ? c->w.p2p_cnt : c->w.m2l_cnt, sizeof(int) * nu, cudaMemcpyDeviceToHost));
    long long total = (long long)c->ws.c[p2p ? ph::WC_P2P_FILL : ph::WC_M2L_FILL];
    std::vector<uint32_t> pool((size_t)total);
    if (total)
        PH_CUDA_CHECK(cudaMemcpy(pool.data(), p2p ? c->w.p2p_pool : c->w.m2l_pool, sizeof(uint32_t) * total,
                                 cudaMemcpyDeviceToHost));
    long long k = 0;
    int ntargets = p2p ? c->info.nleaf : nu;
    for (int u = 0; u < ntargets; u++) {
        for (int j = 0; j < cnt[u]; j++) {
            uint32_t e = pool[off[u] + j];
            int img = PH_ENTRY_IMG(e);
            if ((img != 0) != want_image) continue;
            if (t) { t->push_back(ref_id(c, u)); s->push_back(ref_id(c, PH_ENTRY_ID(e))); im->push_back(img); }
            k++;
        }
    }
    *count = k;
    return 0;
}

extern "C" long long photons_list_size(photons_ctx *c, int kind)
{
    long long n = -1;
    if (collect_lists(c, kind, nullptr, nullptr, nullptr, &n)) return -1;
    return n;
}

extern "C" int photons_list_copy(photons_ctx *c, int kind, int *target, int *source, int *image)
{
    std::vector<int> t, s, im;
    long long n = 0;
    PH_TRY(collect_lists(c, kind, &t, &s, &im, &n));
    if (n && (!target || !source || !image)) return ph_set_error(PH_ERR_ARG, "null list arrays");
    if (n) {
        memcpy(target, t.data(), sizeof(int) * n);
        memcpy(source, s.data(), sizeof(int) * n);
        memcpy(image, im.data(), sizeof(int) * n);
    }
    return 0;
}

extern "C" int photons_op_batch(int op, int n, const double *d, const double *in, double *inout, double rs)
{
    photons_gpu_clear_error();
    if (n < 0 || op < 0 || op > 2 || (n > 0 && (!d || !in || !inout))) return ph_set_error(PH_ERR_ARG, "bad op batch");
    if (n == 0) return 0;
    double *dd = nullptr, *di = nullptr, *dio = nullptr;
    int rc = 0;
    if ((rc = dalloc(dd, (size_t)3 * n)) || (rc = dalloc(di, (size_t)PH_NMULTI * n)) ||
        (rc = dalloc(dio, (size_t)PH_NMULTI * n))) {
        dfree(dd); dfree(di); dfree(dio);
        return rc;
    }
    cudaError_t e = cudaMemcpy(dd, d, sizeof(double) * 3 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(di, in, sizeof(double) * PH_NMULTI * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dio, inout, sizeof(double) * PH_NMULTI * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = ph_set_cuda_error(e, "cudaMemcpy", __FILE__, __LINE__);
    if (!rc) rc = ph::launch_op_batch(op, n, dd, di, dio, rs, 0);
    if (!rc) {
        e = cudaMemcpy(inout, dio, sizeof(double) * PH_NMULTI * n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = ph_set_cuda_error(e, "cudaMemcpy", __FILE__, __LINE__);
    }
    dfree(dd); dfree(di); dfree(dio);
    return rc;
}
