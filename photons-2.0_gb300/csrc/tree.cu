// kd-tree build on the device.
//
// Restates src/fmm.c:30-264 (bksort_inplace, build_kdtree, center_kdtree,
// build_localtree) in two parts.
//
// Wide nodes (more than CHUNK particles) are split level-synchronously:
// every wide node of one depth in the same set of launches (the per-node
// bookkeeping of the first, small levels in single blocks).  Per level:
//   1. each node's particle range is cut into chunks of CHUNK particles;
//   2. chunk sums of the split coordinate (axis = depth mod 3) and a
//      fixed-order reduction give the node's mean;
//   3. the reference's two-ended swap partition (src/fmm.c:58-72) is
//      reproduced exactly: with S particles not above the mean, the k-th
//      particle above the mean counted from the left among positions < S
//      trades places with the k-th particle not above the mean counted from
//      the right among positions >= S.  Ranks come from chunk counts, so the
//      swaps are independent and run in parallel;
//   4. children with <= MAXLEAF particles become leaves, the others nodes
//      of the next level; child boxes come from the split plane.
// A node of at most CHUNK particles is not split by the levels: it roots a
// subtree that one block builds whole in shared memory (k_subtree_build),
// every node of it split by one warp with the arithmetic the levels would
// give a node of one chunk, so the tree is the one a build that splits
// every depth level by level makes.
// Special cases follow the reference: a pair splits at its midpoint and is
// ordered (src/fmm.c:38-47); if no particle lies above the mean the last
// one goes to the upper child.
// Afterwards leaves are renumbered in the reference's depth-first order and
// nodes in preorder (src/fmm.c:101-118), and geometry is written in the
// unified index space.
//
// The mean is a deterministic parallel sum, not the reference's sequential
// one, so a mean can differ from the reference's in the last bits; that
// changes the partition only for a particle within those bits of the mean.
#include <cstdio>
#include <vector>

#include "fmm_context.cuh"

#define CHUNK 1024
#define TB 256

// subtree blocks: one warp per node of the subtree level being split
#define SUB_TB 256
#define SUB_NW (SUB_TB / 32)
#define SUB_FAIL (1 << 20)  // failure mark in a subtree's node counters (above any node count)

// levels of at most this many nodes run their bookkeeping in one block
#define SMALL_LEVEL 32

// depth lists: unified ids per block (one warp) of the counting sort
#define DEPTH_R 4096

// temp-node modes: 0-2 the kinds of a split node (two-ended swap, nothing
// above the mean, a pair), then the two states of a node not yet split
#define MODE_DEFERRED 3  // at most CHUNK particles: split by k_subtree_build
#define MODE_PENDING 4   // wide: split by the levels

namespace ph {
namespace {

__host__ __device__ __forceinline__ const double *axis_ptr(const double *x, const double *y, const double *z, int D)
{
    return D == 0 ? x : (D == 1 ? y : z);
}

// An integer key that orders doubles as the FP64 comparison does (both
// zeros equal), so that !(x > mean) is key(x) <= key(mean) on the integer
// pipe; GB300's FP64 pipe runs at 1/64 of the FP32 rate.  Exact for every
// non-NaN x.
__device__ __forceinline__ long long order_key(double x)
{
    const long long b = __double_as_longlong(x);
    if ((b & 0x7FFFFFFFFFFFFFFFLL) == 0) return 0;
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}

// one root per box: its particle range and the box [0, L]^3 as
// src/fmm.c:194-197 derives the root from the domain box (centre 0.5*(L+0),
// width L-0, src/toptree.c:150-159)
__global__ void k_init_roots(BuildBufs b)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < b.nbox; t += gridDim.x * blockDim.x) {
        const BoxParams &B = b.boxes[t];
        b.tn_start[t] = B.first;
        b.tn_len[t] = B.count;
        b.tn_depth[t] = 0;
        b.tn_parent[t] = -1;
        b.tn_boxid[t] = t;
        b.tn_mode[t] = B.count <= CHUNK ? MODE_DEFERRED : MODE_PENDING;
        for (int d = 0; d < 3; d++) {
            // a rank's domain: its top-tree node's centre and width
            // (src/toptree.c:150-159) give the bounds of src/fmm.c:189-197
            const double lo = B.domain ? B.dom_lo[d] : 0.0, hi = B.domain ? B.dom_hi[d] : B.boxsize;
            const double c = 0.5 * (hi + lo), w = hi - lo;
            b.tn_box[d * b.cap_nodes + t] = c - 0.5 * w;
            b.tn_box[(3 + d) * b.cap_nodes + t] = c + 0.5 * w;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int i = 0; i < BC_NCOUNTERS; i++) b.cnt[i] = 0;
        b.cnt[BC_LEVEL_COUNT] = b.nbox;
        b.leaf_begin[0] = 0;
        b.leaf_count[0] = 0;
    }
}

__global__ void k_init_particles(const double *__restrict__ pos, int n, BuildBufs b)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        b.x[i] = pos[3 * i];
        b.y[i] = pos[3 * i + 1];
        b.z[i] = pos[3 * i + 2];
        b.perm[i] = i;
    }
}

// chunks per node; a deferred node has none and makes no children here
__device__ __forceinline__ void level_nch_node(BuildBufs &b, int lb, int i)
{
    const int t = lb + i;
    if (b.tn_mode[t] == MODE_DEFERRED) {
        b.tn_nch[i] = 0;
        b.tn_nodeflag[i] = 0;
        b.tn_leafflag[i] = 0;
    } else {
        b.tn_nch[i] = (b.tn_len[t] + CHUNK - 1) / CHUNK;
    }
}

__global__ void k_level_nch(BuildBufs b)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) level_nch_node(b, lb, i);
}

// chunk -> level-local node index, written once per level (a warp per node)
__device__ __forceinline__ void chunk_map_node(BuildBufs &b, int i, int lane)
{
    const int c0 = b.tn_chunk_base[i], nc = b.tn_nch[i];
    for (int k = lane; k < nc; k += 32) b.ch_node[c0 + k] = i;
}

__global__ void k_chunk_map(BuildBufs b)
{
    const int C = b.cnt[BC_LEVEL_COUNT];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < C; i += nw) chunk_map_node(b, i, lane);
}

// Chunk sums: lane l adds positions l, l+32, l+64, ... of the chunk in that
// order, then the warp butterfly.  Loads are issued eight at a time ahead
// of the adds, which keep their order.
__global__ void k_chunk_sum(BuildBufs b, int D)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN];
    const double *coord = axis_ptr(b.x, b.y, b.z, D);
    int W = b.cnt[BC_W];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int w = gw; w < W; w += nw) {
        int i = b.ch_node[w];
        int t = lb + i;
        int start = b.tn_start[t], len = b.tn_len[t];
        int s0 = (w - b.tn_chunk_base[i]) * CHUNK;
        int s1 = min(len, s0 + CHUNK);
        const double *cp = coord + start;
        double s = 0.0;
        int k = s0 + lane;
        for (; k + 224 < s1; k += 256) {
            double v[8];
#pragma unroll
            for (int q = 0; q < 8; q++) v[q] = cp[k + 32 * q];
#pragma unroll
            for (int q = 0; q < 8; q++) s += v[q];
        }
        for (; k < s1; k += 32) s += cp[k];
        s = warp_sum_d(s);
        if (lane == 0) b.ch_partial[w] = s;
    }
}

// Node means, a warp each: lane-strided sums of the chunk sums, then the
// warp reduction (fixed order)
__global__ void k_node_mean(BuildBufs b, int D)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < C; i += nw) {
        const int nc = b.tn_nch[i];
        if (nc == 0) continue;
        const int t = lb + i;
        const int c0 = b.tn_chunk_base[i];
        double s = 0.0;
        for (int k = lane; k < nc; k += 32) s += b.ch_partial[c0 + k];
        s = warp_sum_d(s);
        if (lane == 0) b.tn_split[t] = s / (double)b.tn_len[t];
    }
}

__global__ void k_chunk_count(BuildBufs b, int D)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN];
    const double *coord = axis_ptr(b.x, b.y, b.z, D);
    int W = b.cnt[BC_W];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int w = gw; w < W; w += nw) {
        int i = b.ch_node[w];
        int t = lb + i;
        int start = b.tn_start[t], len = b.tn_len[t];
        const long long km = order_key(b.tn_split[t]);
        int s0 = (w - b.tn_chunk_base[i]) * CHUNK;
        int s1 = min(len, s0 + CHUNK);
        const double *cp = coord + start;
        int c = 0;
        int k = s0 + lane;
        for (; k + 224 < s1; k += 256) {
            double v[8];
#pragma unroll
            for (int q = 0; q < 8; q++) v[q] = cp[k + 32 * q];
#pragma unroll
            for (int q = 0; q < 8; q++) c += order_key(v[q]) <= km;
        }
        for (; k < s1; k += 32) c += order_key(cp[k]) <= km;
        c = __reduce_add_sync(0xffffffffu, c);
        if (lane == 0) b.ch_cnt[w] = c;
    }
}

// the split kind and lower-child size of a node of len particles, S of them
// not above the mean
__device__ __forceinline__ void split_sizes(int len, int S, int &mode, int &left)
{
    if (len == 2) { mode = 2; left = 1; }
    else if (S == len) { mode = 1; left = len - 1; }
    else { mode = 0; left = S; }
}

// per node: the child kinds and sizes from the count of particles not above
// the mean
__device__ __forceinline__ void node_split_finish(BuildBufs &b, int i, int t, int len, int S, int maxleaf)
{
    int mode, left;
    split_sizes(len, S, mode, left);
    b.tn_S[t] = S;
    b.tn_mode[t] = mode;
    int right = len - left;
    // child sizes are stashed in child codes until the children exist
    b.tn_child0[t] = left;
    b.tn_child1[t] = right;
    b.tn_nodeflag[i] = (left > maxleaf) + (right > maxleaf);
    b.tn_leafflag[i] = (left <= maxleaf) + (right <= maxleaf);
}

// per wide node of the level, a warp each: prefix of chunk counts,
// partition sizes, child kinds.  Each lane sums a contiguous block of chunk
// counts (the prefix is exact integer arithmetic, so the blocking does not
// change it).
__device__ __forceinline__ void node_split_node(BuildBufs &b, int lb, int i, int lane, int maxleaf)
{
    const int nc = b.tn_nch[i];
    if (nc == 0) return;
    const int t = lb + i, c0 = b.tn_chunk_base[i];
    const int per = (nc + 31) / 32;
    const int kb = min(nc, lane * per), ke = min(nc, kb + per);
    int own = 0;
#pragma unroll 8
    for (int k = kb; k < ke; k++) own += b.ch_cnt[c0 + k];
    const int incl = warp_incl_scan(own);
    int run = incl - own;
    for (int k = kb; k < ke; k++) {
        b.ch_small_base[c0 + k] = run;
        run += b.ch_cnt[c0 + k];
    }
    const int S = shfl(incl, 31);
    if (lane == 0) node_split_finish(b, i, t, b.tn_len[t], S, maxleaf);
}

__global__ void k_node_split(BuildBufs b, int maxleaf)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < C; i += nw) node_split_node(b, lb, i, lane, maxleaf);
}

__device__ __forceinline__ void make_children_node(BuildBufs &b, int lb, int C, int leaves_before, int i, int maxleaf,
                                                   int D)
{
    {
        int t = lb + i;
        if (b.tn_mode[t] == MODE_DEFERRED) return;
        int start = b.tn_start[t];
        int depth = b.tn_depth[t];
        int sizes[2] = {b.tn_child0[t], b.tn_child1[t]};
        double split = b.tn_split[t];
        double lo[3], hi[3];
        for (int d = 0; d < 3; d++) {
            lo[d] = b.tn_box[d * b.cap_nodes + t];
            hi[d] = b.tn_box[(3 + d) * b.cap_nodes + t];
        }
        int nid = lb + C + b.tn_nodebase[i];
        int lid = leaves_before + b.tn_leafbase[i];
        int code[2];
        int ip = start;
        int wide = 0;
        for (int c = 0; c < 2; c++) {
            double clo[3] = {lo[0], lo[1], lo[2]}, chi[3] = {hi[0], hi[1], hi[2]};
            if (c == 0) chi[D] = split;
            else clo[D] = split;
            if (sizes[c] <= maxleaf) {
                if (lid >= b.rule_cap) {
                    atomicOr(&b.cnt[BC_FLAGS], PH_FLAG_LEAF_CAPACITY);
                    code[c] = ~0;
                } else {
                    b.tl_start[lid] = ip;
                    b.tl_len[lid] = sizes[c];
                    b.tl_depth[lid] = depth + 1;
                    b.tl_parent[lid] = t;
                    b.tl_boxid[lid] = b.tn_boxid[t];
                    for (int d = 0; d < 3; d++) {
                        b.tl_box[d * b.cap_leaves + lid] = clo[d];
                        b.tl_box[(3 + d) * b.cap_leaves + lid] = chi[d];
                    }
                    code[c] = ~lid;
                }
                lid++;
            } else {
                if (nid >= b.rule_cap) {
                    atomicOr(&b.cnt[BC_FLAGS], PH_FLAG_NODE_CAPACITY);
                    code[c] = 0;
                } else {
                    b.tn_start[nid] = ip;
                    b.tn_len[nid] = sizes[c];
                    b.tn_depth[nid] = depth + 1;
                    b.tn_parent[nid] = t;
                    b.tn_boxid[nid] = b.tn_boxid[t];
                    b.tn_mode[nid] = sizes[c] <= CHUNK ? MODE_DEFERRED : MODE_PENDING;
                    wide += sizes[c] > CHUNK;
                    for (int d = 0; d < 3; d++) {
                        b.tn_box[d * b.cap_nodes + nid] = clo[d];
                        b.tn_box[(3 + d) * b.cap_nodes + nid] = chi[d];
                    }
                    code[c] = nid;
                }
                nid++;
            }
            ip += sizes[c];
        }
        b.tn_child0[t] = code[0];
        b.tn_child1[t] = code[1];
        if (wide) atomicAdd(&b.cnt[BC_NEXT_WIDE], wide);
    }
}

__global__ void k_make_children(BuildBufs b, int maxleaf, int D)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    const int leaves_before = b.cnt[BC_LEAVES];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x)
        make_children_node(b, lb, C, leaves_before, i, maxleaf, D);
}

// Close level d: record its node range and the leaves it created, advance.
// When the last launched level (d = top - 1) made deferred nodes only,
// they are recorded as level top for k_subtree_build.  After a capacity
// overflow no further level is built.
__device__ void level_finish(BuildBufs &b, int d, int top)
{
    {
        const int C = b.cnt[BC_LEVEL_COUNT], lb = b.cnt[BC_LEVEL_BEGIN];
        if (C == 0) return;
        if (b.cnt[BC_FLAGS] & (PH_FLAG_LEAF_CAPACITY | PH_FLAG_NODE_CAPACITY)) {
            b.cnt[BC_LEVEL_COUNT] = 0;
            return;
        }
        b.lvl_begin[d] = lb;
        b.lvl_count[d] = C;
        b.leaf_begin[d + 1] = b.cnt[BC_LEAVES];
        b.leaf_count[d + 1] = b.cnt[BC_NEW_LEAVES];
        b.cnt[BC_LEAVES] += b.cnt[BC_NEW_LEAVES];
        b.cnt[BC_LEVEL_BEGIN] = lb + C;
        const int next = b.cnt[BC_NEXT_NODES];
        b.cnt[BC_LEVEL_COUNT] = next;
        b.cnt[BC_NLEVELS] = d + 1;
        if (d == top - 1 && next > 0 && b.cnt[BC_NEXT_WIDE] == 0) {
            b.lvl_begin[d + 1] = lb + C;
            b.lvl_count[d + 1] = next;
            b.cnt[BC_LEVEL_BEGIN] = lb + C + next;
            b.cnt[BC_LEVEL_COUNT] = 0;
            b.cnt[BC_NLEVELS] = d + 2;
        }
        b.cnt[BC_NEXT_WIDE] = 0;
    }
}

__global__ void k_level_finish(BuildBufs b, int d, int top)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) level_finish(b, d, top);
}

// ---------------- one block for the bookkeeping of a small level ----------------
// A level of at most SMALL_LEVEL nodes (the first levels) runs its per-node
// bookkeeping in single-block kernels: the same per-node work as the
// kernels above, the scans in one block.  k_level_plan closes the level
// before (when that was small too), then counts chunks, numbers them and
// maps them to nodes; k_level_close splits the nodes, numbers the children
// and makes them.  Integer work throughout, so the tree is unchanged.
#define SMALL_TB 1024

// exclusive scan of in[0, n) into out by the whole block; returns the total
__device__ int block_scan_excl(const int *in, int *out, int n, int *s_warp)
{
    const int lane = warp_lane(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int carry = 0;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < n ? in[i] : 0;
        const int incl = warp_incl_scan(v);
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int w = lane < nwarps ? s_warp[lane] : 0;
            const int wi = warp_incl_scan(w);
            s_warp[lane] = wi - w;
            if (lane == 31) s_warp[32] = wi;
        }
        __syncthreads();
        if (i < n) out[i] = carry + s_warp[warp] + incl - v;
        carry += s_warp[32];
        __syncthreads();
    }
    return carry;
}

__global__ void __launch_bounds__(SMALL_TB) k_level_plan(BuildBufs b, int finish_prev, int top)
{
    __shared__ int s_warp[33];
    if (finish_prev >= 0 && threadIdx.x == 0) level_finish(b, finish_prev, top);
    __syncthreads();
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    for (int i = threadIdx.x; i < C; i += blockDim.x) level_nch_node(b, lb, i);
    __syncthreads();
    const int W = block_scan_excl(b.tn_nch, b.tn_chunk_base, C, s_warp);
    if (threadIdx.x == 0) b.cnt[BC_W] = W;
    const int lane = warp_lane();
    for (int i = threadIdx.x >> 5; i < C; i += blockDim.x >> 5) chunk_map_node(b, i, lane);
}

__global__ void __launch_bounds__(SMALL_TB) k_level_close(BuildBufs b, int maxleaf, int D)
{
    __shared__ int s_warp[33];
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    const int lane = warp_lane();
    for (int i = threadIdx.x >> 5; i < C; i += blockDim.x >> 5) node_split_node(b, lb, i, lane, maxleaf);
    __syncthreads();
    const int next = block_scan_excl(b.tn_nodeflag, b.tn_nodebase, C, s_warp);
    const int fresh = block_scan_excl(b.tn_leafflag, b.tn_leafbase, C, s_warp);
    if (threadIdx.x == 0) {
        b.cnt[BC_NEXT_NODES] = next;
        b.cnt[BC_NEW_LEAVES] = fresh;
    }
    const int leaves_before = b.cnt[BC_LEAVES];
    for (int i = threadIdx.x; i < C; i += blockDim.x) make_children_node(b, lb, C, leaves_before, i, maxleaf, D);
}

// After k_subtree_build: totals, and PH_FLAG_TOP if wide nodes remain
// unsplit after the last launched level.  A failed build (capacity, depth
// or levels) reports an empty tree, so every later stage of the pass has
// no work and reads nothing stale.
__global__ void k_tree_totals(BuildBufs b)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (b.cnt[BC_LEVEL_COUNT] > 0) b.cnt[BC_FLAGS] |= PH_FLAG_TOP;
        b.cnt[BC_NODES] = b.cnt[BC_LEVEL_BEGIN] + b.cnt[BC_SUB_NODES];
        b.cnt[BC_LEAVES] += b.cnt[BC_SUB_LEAVES];
        if (b.cnt[BC_FLAGS] & (PH_FLAG_LEAF_CAPACITY | PH_FLAG_NODE_CAPACITY | PH_FLAG_DEPTH | PH_FLAG_TOP)) {
            b.cnt[BC_NODES] = 0;
            b.cnt[BC_LEAVES] = 0;
            b.cnt[BC_NLEVELS] = 0;
            b.cnt[BC_SUB_NODES] = 0;
            b.cnt[BC_SUB_LEAVES] = 0;
        }
    }
}

// Ranks for the swap partition.  A particle not above the mean that sits in
// the right region (p >= S) publishes its position under slot S-1-r (r =
// its rank among such particles, counted from the left); a particle above
// the mean in the left region (p < S) publishes its position under slot
// p-r (its rank among particles above the mean).  Slot k pairs the k-th
// from the left with the k-th from the right, which is the order
// src/fmm.c:60-72 swaps them in.  ch_swap records each chunk's slots
// (the left-region particles above the mean), so k_swap reads one record
// per chunk.
__global__ void k_rank(BuildBufs b, int D)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN];
    const double *coord = axis_ptr(b.x, b.y, b.z, D);
    int W = b.cnt[BC_W];
    int lane = warp_lane();
    unsigned lt = (1u << lane) - 1u;
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int w = gw; w < W; w += nw) {
        int i = b.ch_node[w];
        int t = lb + i;
        if (b.tn_mode[t] != 0) {
            if (lane == 0) b.ch_swap[w] = make_int4(0, 0, 0, 0);
            continue;
        }
        int start = b.tn_start[t], len = b.tn_len[t];
        const long long km = order_key(b.tn_split[t]);
        int S = b.tn_S[t];
        int s0 = (w - b.tn_chunk_base[i]) * CHUNK;
        int s1 = min(len, s0 + CHUNK);
        const double *cp = coord + start;
        int *bigpos = b.bigpos + start, *smallpos = b.smallpos + start;
        const int small_before = b.ch_small_base[w];
        int run = small_before;
        int nbig = 0;
        for (int k0 = s0; k0 < s1; k0 += 128) {
            double v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int p = k0 + 32 * q + lane;
                v[q] = p < s1 ? cp[p] : 0.0;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int p = k0 + 32 * q + lane;
                const bool in = p < s1;
                const bool small = in && order_key(v[q]) <= km;
                const unsigned m = __ballot_sync(0xffffffffu, small);
                const int r = run + __popc(m & lt);
                if (in) {
                    if (p < S) { if (!small) bigpos[p - r] = p; }
                    else if (small) smallpos[S - 1 - r] = p;
                }
                nbig += __popc(__ballot_sync(0xffffffffu, in && p < S && !small));
                run += __popc(m);
            }
        }
        // the chunk's swaps for k_swap: its node's first particle, its first
        // slot and its number of slots (none once s0 >= S)
        if (lane == 0) b.ch_swap[w] = make_int4(start, s0 - small_before, s0 < S ? nbig : 0, 0);
    }
}

// The swaps of a chunk's slots: its left-region particles above the mean
// hold slots [s0 - (particles not above the mean before s0), + their
// number), as k_rank recorded in ch_swap; each slot's two particles trade
// places.  Pairs are disjoint; a lane loads four slots' particles before it
// stores any.
__global__ void k_swap(BuildBufs b, int D)
{
    int W = b.cnt[BC_W];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int w = gw; w < W; w += nw) {
        const int4 c = b.ch_swap[w];
        const int start = c.x, kb = c.y, nb = c.z;
        if (nb == 0) continue;
        const int *bigpos = b.bigpos + start + kb, *smallpos = b.smallpos + start + kb;
        for (int k0 = 0; k0 < nb; k0 += 128) {
            int pi[4], pj[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int k = k0 + 32 * q + lane;
                pi[q] = k < nb ? start + bigpos[k] : -1;
                pj[q] = k < nb ? start + smallpos[k] : -1;
            }
            double xi[4], yi[4], zi[4], xj[4], yj[4], zj[4];
            int qi[4], qj[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (pi[q] >= 0) {
                    xi[q] = b.x[pi[q]]; yi[q] = b.y[pi[q]]; zi[q] = b.z[pi[q]]; qi[q] = b.perm[pi[q]];
                    xj[q] = b.x[pj[q]]; yj[q] = b.y[pj[q]]; zj[q] = b.z[pj[q]]; qj[q] = b.perm[pj[q]];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (pi[q] >= 0) {
                    b.x[pi[q]] = xj[q]; b.y[pi[q]] = yj[q]; b.z[pi[q]] = zj[q]; b.perm[pi[q]] = qj[q];
                    b.x[pj[q]] = xi[q]; b.y[pj[q]] = yi[q]; b.z[pj[q]] = zi[q]; b.perm[pj[q]] = qi[q];
                }
            }
        }
    }
}

// ---------------- subtrees of at most CHUNK particles ----------------
// Shared memory of one subtree block, 53.3 KB: four blocks per SM.
struct SubTree {
    // the subtree's particles; once written back, the region holds the
    // original permutation (bytes 0-4095) and the numbering arrays
    double x[CHUNK], y[CHUNK], z[CHUNK];
    unsigned short loc[CHUNK];                      // subtree-local index of the particle at each position
    unsigned short bigpos[CHUNK], smallpos[CHUNK];  // a node's slots, over its own local range
    // nodes by level in creation order (node 0 the subtree root): local
    // range, child codes (>= 0 node, < 0 ~leaf), split
    unsigned short n_start[CHUNK], n_len[CHUNK];
    short n_c0[CHUNK], n_c1[CHUNK];
    double n_split[CHUNK];
    unsigned short l_start[CHUNK], l_len[CHUNK];
    unsigned short lev[CHUNK + 2];  // first node of each level of the subtree
    // nodes made by a level are numbered after the level's end through
    // counter (L + 1) mod 3, which also records a failure (see
    // k_subtree_build)
    int nalloc[3];
    int nleaves, fail, nbase, lbase;
};

__device__ __forceinline__ void sub_swap(SubTree &s, int i, int j)
{
    double t;
    t = s.x[i]; s.x[i] = s.x[j]; s.x[j] = t;
    t = s.y[i]; s.y[i] = s.y[j]; s.y[j] = t;
    t = s.z[i]; s.z[i] = s.z[j]; s.z[j] = t;
    const unsigned short q = s.loc[i]; s.loc[i] = s.loc[j]; s.loc[j] = q;
}

// One warp splits node i of the subtree (at depth `depth`, level L of the
// subtree whose nodes end at lend): the mean, count, ranks and swaps a node
// of one chunk gets, with the same lane order and reductions (the sum is
// lane 0's butterfly result added to 0.0, as the one-term reduction of
// k_node_mean does), then its two children.
__device__ void sub_split_node(SubTree &s, int i, int depth, int L, int lend, int axis0, int maxleaf, int levels)
{
    const int lane = warp_lane();
    const unsigned lt = (1u << lane) - 1u;
    const int ns = s.n_start[i], len = s.n_len[i];
    const int D = (axis0 + depth) % 3;
    const double *cd = axis_ptr(s.x, s.y, s.z, D) + ns;
    double mean;
    if (len == 2) {
        mean = 0.5 * (cd[0] + cd[1]);
    } else {
        double sum = 0.0;
        for (int k = lane; k < len; k += 32) sum += cd[k];
        sum = __shfl_sync(0xffffffffu, warp_sum_d(sum), 0);
        double m = 0.0;
        m += sum;
        mean = m / (double)len;
    }
    const long long km = order_key(mean);
    int c = 0;
    for (int k = lane; k < len; k += 32) c += order_key(cd[k]) <= km;
    const int S = __reduce_add_sync(0xffffffffu, c);
    int mode, left;
    split_sizes(len, S, mode, left);
    if (len == 2) {
        if (lane == 0 && cd[0] > cd[1]) sub_swap(s, ns, ns + 1);
    } else if (mode == 0) {
        unsigned short *bigpos = s.bigpos + ns, *smallpos = s.smallpos + ns;
        int run = 0, nbig = 0;
        for (int k0 = 0; k0 < len; k0 += 32) {
            const int p = k0 + lane;
            const bool in = p < len;
            const bool small = in && order_key(cd[p]) <= km;
            const unsigned m = __ballot_sync(0xffffffffu, small);
            const int r = run + __popc(m & lt);
            if (in) {
                if (p < S) { if (!small) bigpos[p - r] = (unsigned short)p; }
                else if (small) smallpos[S - 1 - r] = (unsigned short)p;
            }
            nbig += __popc(__ballot_sync(0xffffffffu, in && p < S && !small));
            run += __popc(m);
        }
        __syncwarp();
        for (int k = lane; k < nbig; k += 32) sub_swap(s, ns + bigpos[k], ns + smallpos[k]);
    }
    __syncwarp();
    if (lane == 0) {
        s.n_split[i] = mean;
        const int sizes[2] = {left, len - left};
        int off = ns;
        for (int ch = 0; ch < 2; ch++) {
            int code;
            if (sizes[ch] <= maxleaf) {
                const int j = atomicAdd(&s.nleaves, 1);
                s.l_start[j] = (unsigned short)off;
                s.l_len[j] = (unsigned short)sizes[ch];
                code = ~j;
            } else {
                // a node below the launched depths fails the subtree
                const int j = lend + (atomicAdd(&s.nalloc[(L + 1) % 3], depth + 1 >= levels ? SUB_FAIL + 1 : 1) &
                                      (SUB_FAIL - 1));
                s.n_start[j] = (unsigned short)off;
                s.n_len[j] = (unsigned short)sizes[ch];
                code = j;
            }
            if (ch == 0) s.n_c0[i] = (short)code;
            else s.n_c1[i] = (short)code;
            off += sizes[ch];
        }
    }
}

// One block per deferred node: load its particles into shared memory, split
// its subtree level by level (a warp per node), write the particles back,
// number the subtree's nodes in preorder and its leaves depth-first, then
// write them into the temp arrays after the level-built ones, with boxes
// from the split planes.  A subtree node's own preorder number goes to
// tn_pre and its root to tn_subroot (leaves: tl_final, tl_subroot);
// k_subtree_number adds the root's numbers once the levels are numbered.
// Every barrier is reached by all threads of the block: loop bounds and
// failure flags are read after a barrier and not written again before the
// next one.  Level L numbers its new nodes through counter (L + 1) mod 3
// (a failure adds SUB_FAIL to it), which thread 0 cleared during level
// L - 1; counter (L + 2) mod 3, last read after level L - 2, is cleared
// during level L.  So one barrier per level.
__global__ void __launch_bounds__(SUB_TB) k_subtree_build(BuildBufs b, int axis0, int maxleaf, int levels)
{
    extern __shared__ __align__(16) unsigned char sub_smem[];
    SubTree &s = *reinterpret_cast<SubTree *>(sub_smem);
    if (b.cnt[BC_LEVEL_COUNT] > 0 || (b.cnt[BC_FLAGS] & (PH_FLAG_LEAF_CAPACITY | PH_FLAG_NODE_CAPACITY))) return;
    const int T0 = b.cnt[BC_LEVEL_BEGIN], L0 = b.cnt[BC_LEAVES];
    const int tid = threadIdx.x, warp = tid >> 5;
    int *operm = reinterpret_cast<int *>(s.x);
    unsigned short *sn = reinterpret_cast<unsigned short *>(s.x) + 2 * CHUNK;
    unsigned short *sl = sn + CHUNK, *pre = sl + CHUNK, *lb = pre + CHUNK, *lfin = lb + CHUNK;
    unsigned short *npar = lfin + CHUNK, *lpar = npar + CHUNK;
    for (int t = blockIdx.x; t < T0; t += gridDim.x) {
        if (b.tn_mode[t] != MODE_DEFERRED) continue;
        const int start = b.tn_start[t], len = b.tn_len[t], rd = b.tn_depth[t];
        for (int k = tid; k < len; k += SUB_TB) {
            s.x[k] = b.x[start + k];
            s.y[k] = b.y[start + k];
            s.z[k] = b.z[start + k];
            s.loc[k] = (unsigned short)k;
        }
        if (tid == 0) {
            s.nalloc[1] = 0;
            s.nleaves = 0;
            s.n_start[0] = 0;
            s.n_len[0] = (unsigned short)len;
            s.lev[0] = 0;
            s.fail = 0;
        }
        __syncthreads();
        int failed = rd >= levels;
        int nlev = 0, lbeg = 0, lend = 1;
        while (lbeg < lend && !failed) {
            if (tid == 0) s.nalloc[(nlev + 2) % 3] = 0;
            for (int i = lbeg + warp; i < lend; i += SUB_NW)
                sub_split_node(s, i, rd + nlev, nlev, lend, axis0, maxleaf, levels);
            __syncthreads();
            const int got = s.nalloc[(nlev + 1) % 3];
            lbeg = lend;
            lend += got & (SUB_FAIL - 1);
            failed = got >= SUB_FAIL;
            nlev++;
            if (tid == 0) s.lev[nlev] = (unsigned short)lbeg;
        }
        __syncthreads();  // lev[] complete
        if (failed) {
            if (tid == 0) atomicOr(&b.cnt[BC_FLAGS], PH_FLAG_DEPTH);
            continue;  // the next subtree's first writes follow a barrier all threads passed
        }
        for (int k = tid; k < len; k += SUB_TB) {
            b.x[start + k] = s.x[k];
            b.y[start + k] = s.y[k];
            b.z[start + k] = s.z[k];
        }
        __syncthreads();  // x, y, z read: their region now takes the original permutation
        for (int k = tid; k < len; k += SUB_TB) operm[k] = b.perm[start + k];
        __syncthreads();
        for (int k = tid; k < len; k += SUB_TB) b.perm[start + k] = operm[s.loc[k]];
        // parents from the child codes; subtree sizes bottom-up
        for (int i = tid; i < lend; i += SUB_TB) {
            const int c0 = s.n_c0[i], c1 = s.n_c1[i];
            if (c0 >= 0) npar[c0] = (unsigned short)i; else lpar[~c0] = (unsigned short)i;
            if (c1 >= 0) npar[c1] = (unsigned short)i; else lpar[~c1] = (unsigned short)i;
        }
        for (int L = nlev - 1; L >= 0; L--) {
            __syncthreads();
            for (int i = s.lev[L] + tid; i < s.lev[L + 1]; i += SUB_TB) {
                const int c0 = s.n_c0[i], c1 = s.n_c1[i];
                sn[i] = (unsigned short)(1 + (c0 >= 0 ? sn[c0] : 0) + (c1 >= 0 ? sn[c1] : 0));
                sl[i] = (unsigned short)((c0 >= 0 ? sl[c0] : 1) + (c1 >= 0 ? sl[c1] : 1));
            }
        }
        __syncthreads();
        if (tid == 0) {
            const int ntot = sn[0], ltot = sl[0];
            const int nb = atomicAdd(&b.cnt[BC_SUB_NODES], ntot - 1);
            const int lbg = atomicAdd(&b.cnt[BC_SUB_LEAVES], ltot);
            s.nbase = T0 + nb;
            s.lbase = L0 + lbg;
            if (T0 + nb + ntot - 1 > b.rule_cap) {
                atomicOr(&b.cnt[BC_FLAGS], PH_FLAG_NODE_CAPACITY);
                s.fail = 1;
            }
            if (L0 + lbg + ltot > b.rule_cap) {
                atomicOr(&b.cnt[BC_FLAGS], PH_FLAG_LEAF_CAPACITY);
                s.fail = 1;
            }
            b.tn_sub_nodes[t] = ntot;
            b.tn_sub_leaves[t] = ltot;
            pre[0] = 0;
            lb[0] = 0;
        }
        __syncthreads();
        failed = s.fail;
        __syncthreads();
        if (failed) continue;
        for (int L = 0; L < nlev; L++) {
            for (int i = s.lev[L] + tid; i < s.lev[L + 1]; i += SUB_TB) {
                const int c0 = s.n_c0[i], c1 = s.n_c1[i];
                const int P = pre[i], B = lb[i];
                const int off_n = c0 >= 0 ? sn[c0] : 0, off_l = c0 >= 0 ? sl[c0] : 1;
                if (c0 >= 0) { pre[c0] = (unsigned short)(P + 1); lb[c0] = (unsigned short)B; }
                else lfin[~c0] = (unsigned short)B;
                if (c1 >= 0) { pre[c1] = (unsigned short)(P + 1 + off_n); lb[c1] = (unsigned short)(B + off_l); }
                else lfin[~c1] = (unsigned short)(B + off_l);
            }
            __syncthreads();
        }
        const int nbase = s.nbase, lbase = s.lbase, boxid = b.tn_boxid[t];
        // nodes level by level: a node's box is its parent's, written a level earlier, cut at the parent's split
        for (int L = 0; L < nlev; L++) {
            for (int i = s.lev[L] + tid; i < s.lev[L + 1]; i += SUB_TB) {
                const int ti = i == 0 ? t : nbase + pre[i] - 1;
                const int c0 = s.n_c0[i], c1 = s.n_c1[i];
                b.tn_child0[ti] = c0 >= 0 ? nbase + pre[c0] - 1 : ~(lbase + lfin[~c0]);
                b.tn_child1[ti] = c1 >= 0 ? nbase + pre[c1] - 1 : ~(lbase + lfin[~c1]);
                b.tn_split[ti] = s.n_split[i];
                if (i == 0) continue;
                const int par = npar[i];
                const int tp = par == 0 ? t : nbase + pre[par] - 1;
                b.tn_start[ti] = start + s.n_start[i];
                b.tn_len[ti] = s.n_len[i];
                b.tn_depth[ti] = rd + L;
                b.tn_parent[ti] = tp;
                b.tn_boxid[ti] = boxid;
                b.tn_pre[ti] = pre[i];
                b.tn_subroot[ti] = t;
                const int Dp = (axis0 + rd + L - 1) % 3;
                const bool upper = s.n_c0[par] != i;
                for (int d = 0; d < 3; d++) {
                    double lo = b.tn_box[d * b.cap_nodes + tp], hi = b.tn_box[(3 + d) * b.cap_nodes + tp];
                    if (d == Dp) {
                        if (upper) lo = s.n_split[par];
                        else hi = s.n_split[par];
                    }
                    b.tn_box[d * b.cap_nodes + ti] = lo;
                    b.tn_box[(3 + d) * b.cap_nodes + ti] = hi;
                }
            }
            __syncthreads();
        }
        for (int j = tid; j < s.nleaves; j += SUB_TB) {
            const int tl = lbase + lfin[j];
            const int par = lpar[j];
            const int tp = par == 0 ? t : nbase + pre[par] - 1;
            const int pd = b.tn_depth[tp];
            b.tl_start[tl] = start + s.l_start[j];
            b.tl_len[tl] = s.l_len[j];
            b.tl_depth[tl] = pd + 1;
            b.tl_parent[tl] = tp;
            b.tl_boxid[tl] = boxid;
            b.tl_final[tl] = lfin[j];
            b.tl_subroot[tl] = t;
            const int Dp = (axis0 + pd) % 3;
            const bool upper = s.n_c0[par] != ~j;
            for (int d = 0; d < 3; d++) {
                double lo = b.tn_box[d * b.cap_nodes + tp], hi = b.tn_box[(3 + d) * b.cap_nodes + tp];
                if (d == Dp) {
                    if (upper) lo = s.n_split[par];
                    else hi = s.n_split[par];
                }
                b.tl_box[d * b.cap_leaves + tl] = lo;
                b.tl_box[(3 + d) * b.cap_leaves + tl] = hi;
            }
        }
        __syncthreads();
    }
}

// ---------------- renumbering ----------------
// Level nodes bottom-up; a deferred node's counts come from k_subtree_build.
__global__ void k_subtree_counts(BuildBufs b, int d)
{
    if (d >= b.cnt[BC_NLEVELS]) return;
    const int lb = b.lvl_begin[d], C = b.lvl_count[d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        int t = lb + i;
        if (b.tn_mode[t] == MODE_DEFERRED) continue;
        int sn = 1, sl = 0;
        int c[2] = {b.tn_child0[t], b.tn_child1[t]};
        for (int k = 0; k < 2; k++) {
            if (PH_IS_LEAF_CODE(c[k])) sl += 1;
            else { sn += b.tn_sub_nodes[c[k]]; sl += b.tn_sub_leaves[c[k]]; }
        }
        b.tn_sub_nodes[t] = sn;
        b.tn_sub_leaves[t] = sl;
    }
}

// the boxes' trees follow one another in box order: root r starts after the
// nodes and leaves of roots 0..r-1
__global__ void k_root_bases(BuildBufs b)
{
    if (blockIdx.x == 0 && threadIdx.x == 0 && b.cnt[BC_NLEVELS] > 0) {
        int nodes = 0, leaves = 0;
        for (int r = 0; r < b.nbox; r++) {
            b.tn_pre[r] = nodes;
            b.tn_lbase[r] = leaves;
            nodes += b.tn_sub_nodes[r];
            leaves += b.tn_sub_leaves[r];
        }
    }
}

// preorder node numbers and depth-first leaf numbers, src/fmm.c:101-118;
// a deferred node's subtree is numbered by k_subtree_number
__global__ void k_number(BuildBufs b, int d)
{
    if (d >= b.cnt[BC_NLEVELS]) return;
    const int lb = b.lvl_begin[d], C = b.lvl_count[d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        int t = lb + i;
        if (b.tn_mode[t] == MODE_DEFERRED) continue;
        int pre = b.tn_pre[t], lbase = b.tn_lbase[t];
        int c0 = b.tn_child0[t], c1 = b.tn_child1[t];
        int off_nodes, off_leaves;
        if (PH_IS_LEAF_CODE(c0)) { b.tl_final[~c0] = lbase; off_nodes = 0; off_leaves = 1; }
        else { b.tn_pre[c0] = pre + 1; b.tn_lbase[c0] = lbase; off_nodes = b.tn_sub_nodes[c0]; off_leaves = b.tn_sub_leaves[c0]; }
        if (PH_IS_LEAF_CODE(c1)) b.tl_final[~c1] = lbase + off_leaves;
        else { b.tn_pre[c1] = pre + 1 + off_nodes; b.tn_lbase[c1] = lbase + off_leaves; }
    }
}

// subtree nodes and leaves: the subtree root's numbers plus their own
__global__ void k_subtree_number(BuildBufs b)
{
    const int nodes = b.cnt[BC_NODES], leaves = b.cnt[BC_LEAVES];
    const int t0 = nodes - b.cnt[BC_SUB_NODES], l0 = leaves - b.cnt[BC_SUB_LEAVES];
    for (int t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < nodes; t += gridDim.x * blockDim.x)
        b.tn_pre[t] += b.tn_pre[b.tn_subroot[t]];
    for (int l = l0 + blockIdx.x * blockDim.x + threadIdx.x; l < leaves; l += gridDim.x * blockDim.x)
        b.tl_final[l] += b.tn_lbase[b.tl_subroot[l]];
}

__device__ __forceinline__ void write_geom(TreeBufs &T, int u, const double *box, int cap, int idx)
{
    double lo0 = box[0 * cap + idx], lo1 = box[1 * cap + idx], lo2 = box[2 * cap + idx];
    double hi0 = box[3 * cap + idx], hi1 = box[4 * cap + idx], hi2 = box[5 * cap + idx];
    // width = right - left, centre = 0.5*(right + left), src/fmm.c:126-131
    double w0 = hi0 - lo0, w1 = hi1 - lo1, w2 = hi2 - lo2;
    T.wx[u] = w0; T.wy[u] = w1; T.wz[u] = w2;
    T.cx[u] = 0.5 * (hi0 + lo0); T.cy[u] = 0.5 * (hi1 + lo1); T.cz[u] = 0.5 * (hi2 + lo2);
    T.wsum[u] = w0 + w1 + w2;
}

__global__ void k_scatter_nodes(BuildBufs b, TreeBufs T)
{
    const int nnodes = b.cnt[BC_NODES], nleaves = b.cnt[BC_LEAVES];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nnodes; t += gridDim.x * blockDim.x) {
        int u = nleaves + b.tn_pre[t];
        T.ipart[u] = b.tn_start[t];
        T.npart[u] = b.tn_len[t];
        T.depth[u] = b.tn_depth[t];
        int par = b.tn_parent[t];
        T.parent[u] = par < 0 ? -1 : nleaves + b.tn_pre[par];
        int c0 = b.tn_child0[t], c1 = b.tn_child1[t];
        T.son0[u] = PH_IS_LEAF_CODE(c0) ? b.tl_final[~c0] : nleaves + b.tn_pre[c0];
        T.son1[u] = PH_IS_LEAF_CODE(c1) ? b.tl_final[~c1] : nleaves + b.tn_pre[c1];
        T.split[u] = b.tn_split[t];
        T.boxid[u] = b.tn_boxid[t];
        if (t < b.nbox) b.boxes[t].root = u;
        write_geom(T, u, b.tn_box, b.cap_nodes, t);
    }
}

__global__ void k_scatter_leaves(BuildBufs b, TreeBufs T)
{
    const int nleaves = b.cnt[BC_LEAVES];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nleaves; l += gridDim.x * blockDim.x) {
        int u = b.tl_final[l];
        T.ipart[u] = b.tl_start[l];
        T.npart[u] = b.tl_len[l];
        T.depth[u] = b.tl_depth[l];
        T.parent[u] = nleaves + b.tn_pre[b.tl_parent[l]];
        T.son0[u] = -1;
        T.son1[u] = -1;
        T.split[u] = 0.0;
        T.boxid[u] = b.tl_boxid[l];
        write_geom(T, u, b.tl_box, b.cap_leaves, l);
    }
}

// ---------------- depth lists ----------------
// A stable counting sort of the unified ids by depth: depth d's list holds
// its leaves (depth-first order) then its nodes (preorder).  Block k counts
// the depths of ids [k R, (k+1) R) into cells (depth, block), stored depth
// by depth; an exclusive scan of the cells gives each block its first slot
// per depth.
__global__ void __launch_bounds__(32) k_depth_count(BuildBufs b, TreeBufs T, int ndepth)
{
    __shared__ int h[PH_MAX_DEPTH_CAP + 2];
    const int nu = b.cnt[BC_NODES] + b.cnt[BC_LEAVES], nblk = gridDim.x, k = blockIdx.x, lane = threadIdx.x;
    for (int d = lane; d < ndepth; d += 32) h[d] = 0;
    __syncwarp();
    const int u0 = k * DEPTH_R, u1 = min(nu, u0 + DEPTH_R);
    for (int u = u0 + lane; u < u1; u += 32) {
        const int d = T.depth[u];
        if (d >= 0 && d < ndepth) atomicAdd(&h[d], 1);
    }
    __syncwarp();
    for (int d = lane; d < ndepth; d += 32) T.depth_blk[d * nblk + k] = h[d];
    if (k == 0 && lane == 0) b.cnt[BC_DEPTH_CELLS] = ndepth * nblk;
}

__global__ void __launch_bounds__(32) k_depth_place(BuildBufs b, TreeBufs T, int ndepth)
{
    __shared__ int cur[PH_MAX_DEPTH_CAP + 2];
    const int nu = b.cnt[BC_NODES] + b.cnt[BC_LEAVES], nblk = gridDim.x, k = blockIdx.x, lane = threadIdx.x;
    const unsigned lt = (1u << lane) - 1u;
    const int *first = T.depth_blk + (size_t)ndepth * nblk;  // the scanned cells
    for (int d = lane; d < ndepth; d += 32) cur[d] = first[d * nblk + k];
    if (k == 0) {
        // per-depth offsets and counts, and the deepest depth holding an id
        int deepest = 0;
        for (int d = lane; d < ndepth; d += 32) {
            const int o = first[d * nblk], e = d + 1 < ndepth ? first[(d + 1) * nblk] : nu;
            T.depth_off[d] = o;
            T.depth_cnt[d] = e - o;
            if (e > o) deepest = d;
        }
        deepest = __reduce_max_sync(0xffffffffu, deepest);
        if (lane == 0) {
            T.depth_off[ndepth] = nu;
            b.cnt[BC_DEPTH] = deepest;
        }
    }
    __syncwarp();
    const int u0 = k * DEPTH_R, u1 = min(nu, u0 + DEPTH_R);
    for (int base = u0; base < u1; base += 32) {
        const int u = base + lane;
        int d = u < u1 ? T.depth[u] : -1;
        if (d >= ndepth) d = -1;
        const unsigned same = __match_any_sync(0xffffffffu, d);
        if (d >= 0) T.depth_list[cur[d] + __popc(same & lt)] = u;
        __syncwarp();
        if (d >= 0 && (same & lt) == 0) cur[d] += __popc(same);
        __syncwarp();
    }
}

}  // namespace

int launch_init_particles(BuildBufs &b, const double *pos, int n, cudaStream_t st)
{
    ph::note_launch(), k_init_particles<<<device_sm_count() * 8, TB, 0, st>>>(pos, n, b);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int depth_sort_blocks(int cap_u) { return (cap_u + DEPTH_R - 1) / DEPTH_R; }

// Enqueue the whole build, no host sync: at most `top` levels of wide
// nodes, then the subtrees, with nodes at depths < `levels`.  Levels past
// the last wide node exit at once.  Wide nodes left after `top` levels
// raise PH_FLAG_TOP in b.cnt[BC_FLAGS] and a node at depth `levels` raises
// PH_FLAG_DEPTH (the caller grows the count and builds again); capacity
// overflows raise their flags there too.  Depth lists cover depths
// 0..levels.
int build_tree(BuildBufs &b, TreeBufs &T, const PassParams &p, int levels, int top, cudaStream_t st)
{
    const int maxb = device_sm_count() * 8;
    if (levels < 1 || levels + 1 > T.max_depth_cap || T.max_depth_cap > PH_MAX_DEPTH_CAP)
        return ph_set_error(7, "tree deeper than %d levels", T.max_depth_cap - 1);
    if (top < 1 || top > levels) top = levels;
    const int ndepth = levels + 1;  // leaves can sit one level below the deepest nodes
    const int nblk = T.depth_nblk;
    if (nblk < 1 || nblk != depth_sort_blocks(T.cap_u)) return ph_set_error(7, "depth-sort buffers not allocated");
    // the subtree blocks' shared memory is above the 48 KB default: allowed
    // once per device
    static bool sub_attr[64] = {};
    int dev = 0;
    PH_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !sub_attr[dev]) {
        PH_CUDA_CHECK(cudaFuncSetAttribute(k_subtree_build, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)sizeof(SubTree)));
        if (dev >= 0 && dev < 64) sub_attr[dev] = true;
    }
    PH_CUDA_CHECK(cudaMemsetAsync(b.lvl_count, 0, sizeof(int) * (top + 2), st));
    PH_CUDA_CHECK(cudaMemsetAsync(b.leaf_count, 0, sizeof(int) * (top + 2), st));
    ph::note_launch(), k_init_roots<<<(b.nbox + TB - 1) / TB, TB, 0, st>>>(b);
    // a level has at most nbox 2^d nodes: the first levels are small enough for
    // single-block bookkeeping (7 launches a level instead of 19)
    bool pending = false;  // a small level whose k_level_finish is still to come
    // nodes of one level: the roots, or the children of the level above's
    // wide nodes (more than CHUNK particles each, so at most N / CHUNK)
    const long long lvl_bound = 2LL * (b.cap_n / CHUNK) + 2LL * b.nbox + 2;
    const int lvl_max = lvl_bound < b.cap_nodes ? (int)lvl_bound : b.cap_nodes;
    for (int d = 0; d < top; d++) {
        const int D = (p.axis0 + d) % 3;  // from direct_local_start; the axis cycles (src/fmm.c:99)
        const bool small = d < 24 && ((long long)b.nbox << d) <= SMALL_LEVEL;
        if (small) {
            ph::note_launch(), k_level_plan<<<1, SMALL_TB, 0, st>>>(b, pending ? d - 1 : -1, top);
        } else {
            if (pending) ph::note_launch(), k_level_finish<<<1, 1, 0, st>>>(b, d - 1, top);
            ph::note_launch(), k_level_nch<<<maxb, TB, 0, st>>>(b);
            scan_exclusive_i32_bounded(b.tn_nch, b.tn_chunk_base, b.cnt + BC_LEVEL_COUNT, b.cap_nodes, lvl_max,
                                       b.cnt + BC_W, b.scan_scratch, b.scan_scratch_elems, st);
            ph::note_launch(), k_chunk_map<<<maxb, TB, 0, st>>>(b);
        }
        ph::note_launch(), k_chunk_sum<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_node_mean<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_chunk_count<<<maxb, TB, 0, st>>>(b, D);
        if (small) {
            ph::note_launch(), k_level_close<<<1, SMALL_TB, 0, st>>>(b, p.maxleaf, D);
        } else {
            ph::note_launch(), k_node_split<<<maxb, TB, 0, st>>>(b, p.maxleaf);
            scan_exclusive_i32_bounded(b.tn_nodeflag, b.tn_nodebase, b.cnt + BC_LEVEL_COUNT, b.cap_nodes, lvl_max,
                                       b.cnt + BC_NEXT_NODES, b.scan_scratch, b.scan_scratch_elems, st);
            scan_exclusive_i32_bounded(b.tn_leafflag, b.tn_leafbase, b.cnt + BC_LEVEL_COUNT, b.cap_nodes, lvl_max,
                                       b.cnt + BC_NEW_LEAVES, b.scan_scratch, b.scan_scratch_elems, st);
            ph::note_launch(), k_make_children<<<maxb, TB, 0, st>>>(b, p.maxleaf, D);
        }
        ph::note_launch(), k_rank<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_swap<<<maxb, TB, 0, st>>>(b, D);
        if (small) {
            pending = true;
        } else {
            ph::note_launch(), k_level_finish<<<1, 1, 0, st>>>(b, d, top);
            pending = false;
        }
    }
    if (pending) ph::note_launch(), k_level_finish<<<1, 1, 0, st>>>(b, top - 1, top);
    ph::note_launch(), k_subtree_build<<<device_sm_count() * 4, SUB_TB, sizeof(SubTree), st>>>(b, p.axis0, p.maxleaf,
                                                                                                levels);
    ph::note_launch(), k_tree_totals<<<1, 1, 0, st>>>(b);
    // subtree sizes bottom-up, numbers top-down, over the recorded levels (top + 1 at most)
    for (int d = top; d >= 0; d--) ph::note_launch(), k_subtree_counts<<<maxb, TB, 0, st>>>(b, d);
    ph::note_launch(), k_root_bases<<<1, 1, 0, st>>>(b);
    for (int d = 0; d <= top; d++) ph::note_launch(), k_number<<<maxb, TB, 0, st>>>(b, d);
    ph::note_launch(), k_subtree_number<<<maxb, TB, 0, st>>>(b);
    ph::note_launch(), k_scatter_nodes<<<maxb, TB, 0, st>>>(b, T);
    ph::note_launch(), k_scatter_leaves<<<maxb, TB, 0, st>>>(b, T);
    ph::note_launch(), k_depth_count<<<nblk, 32, 0, st>>>(b, T, ndepth);
    scan_exclusive_i32(T.depth_blk, T.depth_blk + (size_t)ndepth * nblk, b.cnt + BC_DEPTH_CELLS, ndepth * nblk,
                       b.cnt + BC_DEPTH_TOTAL, b.scan_scratch, b.scan_scratch_elems, st);
    ph::note_launch(), k_depth_place<<<nblk, 32, 0, st>>>(b, T, ndepth);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// host view of the finished build (after the stream has been synchronised)
int read_tree_info(const BuildBufs &b, const TreeBufs &T, int levels, TreeInfo &info)
{
    int h[BC_NCOUNTERS];
    PH_CUDA_CHECK(cudaMemcpy(h, b.cnt, sizeof(h), cudaMemcpyDeviceToHost));
    info.nleaf = h[BC_LEAVES];
    info.nnode = h[BC_NODES];
    info.depth = h[BC_DEPTH];
    info.levels = h[BC_NLEVELS];
    info.flags = h[BC_FLAGS];
    info.depth_off.resize(levels + 2);
    PH_CUDA_CHECK(cudaMemcpy(info.depth_off.data(), T.depth_off, sizeof(int) * (levels + 2), cudaMemcpyDeviceToHost));
    return 0;
}

}  // namespace ph
