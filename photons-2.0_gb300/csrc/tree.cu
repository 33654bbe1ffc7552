// kd-tree build on the device.
//
// Restates src/fmm.c:30-264 (bksort_inplace, build_kdtree, center_kdtree,
// build_localtree) as a level-synchronous build: every node of one depth
// is split in the same set of launches.  Per level:
//   1. each node's particle range is cut into chunks of CHUNK particles
//      (a node of at most one chunk is split by one warp in k_narrow_split,
//      which does steps 2-3 for it in one kernel);
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

namespace ph {
namespace {

__device__ __forceinline__ const double *axis_ptr(const double *x, const double *y, const double *z, int D)
{
    return D == 0 ? x : (D == 1 ? y : z);
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


__global__ void k_level_nch(BuildBufs b)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        const int len = b.tn_len[lb + i];
        b.tn_nch[i] = len <= CHUNK ? 0 : (len + CHUNK - 1) / CHUNK;  // one chunk or less: k_narrow_split
    }
}

// chunk -> level-local node index, written once per level
__global__ void k_chunk_map(BuildBufs b)
{
    const int C = b.cnt[BC_LEVEL_COUNT];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < C; i += nw) {
        int c0 = b.tn_chunk_base[i], nc = b.tn_nch[i];
        for (int k = lane; k < nc; k += 32) b.ch_node[c0 + k] = i;
    }
}

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
        double s = 0.0;
        for (int k = s0 + lane; k < s1; k += 32) s += coord[start + k];
        s = warp_sum_d(s);
        if (lane == 0) b.ch_partial[w] = s;
    }
}

// Node means of the nodes of more than one chunk, a warp each:
// lane-strided sums of the chunk sums, then the warp reduction (fixed order)
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
        double mean = b.tn_split[t];
        int s0 = (w - b.tn_chunk_base[i]) * CHUNK;
        int s1 = min(len, s0 + CHUNK);
        int c = 0;
        for (int k = s0 + lane; k < s1; k += 32) c += !(coord[start + k] > mean);
        c = __reduce_add_sync(0xffffffffu, c);
        if (lane == 0) b.ch_cnt[w] = c;
    }
}

// per node: the child kinds and sizes from the count of particles not above
// the mean
__device__ __forceinline__ void node_split_finish(BuildBufs &b, int i, int t, int len, int S, int maxleaf)
{
    int mode, left;
    if (len == 2) { mode = 2; left = 1; }
    else if (S == len) { mode = 1; left = len - 1; }
    else { mode = 0; left = S; }
    b.tn_S[t] = S;
    b.tn_mode[t] = mode;
    int right = len - left;
    // child sizes are stashed in child codes until the children exist
    b.tn_child0[t] = left;
    b.tn_child1[t] = right;
    b.tn_nodeflag[i] = (left > maxleaf) + (right > maxleaf);
    b.tn_leafflag[i] = (left <= maxleaf) + (right <= maxleaf);
}

// per node of more than one chunk, a warp each: prefix of chunk counts,
// partition sizes, child kinds.  Each lane sums a contiguous block of chunk
// counts (the prefix is exact integer arithmetic, so the blocking does not
// change it).
__global__ void k_node_split(BuildBufs b, int maxleaf)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < C; i += nw) {
        const int nc = b.tn_nch[i];
        if (nc == 0) continue;
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
}

__global__ void k_make_children(BuildBufs b, int maxleaf, int D)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    int leaves_before = b.cnt[BC_LEAVES];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        int t = lb + i;
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
    }
}

// close level d: record its node range and the leaves it created, advance.
// After a capacity overflow no further level is built.
__global__ void k_level_finish(BuildBufs b, int d)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
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
        b.cnt[BC_LEVEL_COUNT] = b.cnt[BC_NEXT_NODES];
        b.cnt[BC_NLEVELS] = d + 1;
    }
}

// After the last launched level: totals, and PH_FLAG_DEPTH if nodes remain
// unsplit.  A failed build (capacity or depth) reports an empty tree, so
// every later stage of the pass has no work and reads nothing stale.
__global__ void k_tree_totals(BuildBufs b)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        b.cnt[BC_NODES] = b.cnt[BC_LEVEL_BEGIN];
        if (b.cnt[BC_LEVEL_COUNT] > 0) b.cnt[BC_FLAGS] |= PH_FLAG_DEPTH;
        if (b.cnt[BC_FLAGS] & (PH_FLAG_LEAF_CAPACITY | PH_FLAG_NODE_CAPACITY | PH_FLAG_DEPTH)) {
            b.cnt[BC_NODES] = 0;
            b.cnt[BC_LEAVES] = 0;
            b.cnt[BC_NLEVELS] = 0;
        }
    }
}

// Ranks for the swap partition.  A particle not above the mean that sits in
// the right region (p >= S) publishes its position under slot S-1-r (r =
// its rank among such particles, counted from the left); a particle above
// the mean in the left region (p < S) records slot p-r (its rank among
// particles above the mean).  Slot k pairs the k-th from the left with the
// k-th from the right, which is the order src/fmm.c:60-72 swaps them in.
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
        if (b.tn_mode[t] != 0) continue;
        int start = b.tn_start[t], len = b.tn_len[t];
        double mean = b.tn_split[t];
        int S = b.tn_S[t];
        int s0 = (w - b.tn_chunk_base[i]) * CHUNK;
        int s1 = min(len, s0 + CHUNK);
        int run = b.ch_small_base[w];
        for (int k0 = s0; k0 < s1; k0 += 32) {
            int p = k0 + lane;
            bool in = p < s1;
            bool small = in && !(coord[start + p] > mean);
            unsigned m = __ballot_sync(0xffffffffu, small);
            int r = run + __popc(m & lt);
            if (in) {
                if (p < S) b.bigslot[start + p] = small ? -1 : (p - r);
                else if (small) b.smallpos[start + (S - 1 - r)] = p;
            }
            run += __popc(m);
        }
    }
}

__device__ __forceinline__ void swap_particles(BuildBufs &b, int i, int j)
{
    double t;
    t = b.x[i]; b.x[i] = b.x[j]; b.x[j] = t;
    t = b.y[i]; b.y[i] = b.y[j]; b.y[j] = t;
    t = b.z[i]; b.z[i] = b.z[j]; b.z[j] = t;
    int q = b.perm[i]; b.perm[i] = b.perm[j]; b.perm[j] = q;
}

// Nodes of at most one chunk, a warp each, in one kernel while the node's
// data is in cache: the sum, mean, count, child kinds, ranks and swaps that
// k_chunk_sum, k_node_mean, k_chunk_count, k_node_split, k_rank and k_swap
// give a node of one chunk, with the same lane order and reductions (the
// chunk sum is lane 0's butterfly result; the mean adds it to 0.0 first, as
// the one-term reduction of k_node_mean does).
__global__ void k_narrow_split(BuildBufs b, int D, int maxleaf)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN], C = b.cnt[BC_LEVEL_COUNT];
    const double *coord = axis_ptr(b.x, b.y, b.z, D);
    const int lane = warp_lane();
    const unsigned lt = (1u << lane) - 1u;
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < C; i += nw) {
        if (b.tn_nch[i] != 0) continue;
        const int t = lb + i;
        const int start = b.tn_start[t], len = b.tn_len[t];
        const double *cd = coord + start;
        double mean;
        if (len == 2) {
            mean = 0.5 * (cd[0] + cd[1]);
        } else {
            double s = 0.0;
            for (int k = lane; k < len; k += 32) s += cd[k];
            s = __shfl_sync(0xffffffffu, warp_sum_d(s), 0);
            double m = 0.0;
            m += s;
            mean = m / (double)len;
        }
        int c = 0;
        for (int k = lane; k < len; k += 32) c += !(cd[k] > mean);
        const int S = __reduce_add_sync(0xffffffffu, c);
        if (lane == 0) {
            b.tn_split[t] = mean;
            node_split_finish(b, i, t, len, S, maxleaf);
        }
        if (len == 2) {
            if (lane == 0 && cd[0] > cd[1]) swap_particles(b, start, start + 1);
            continue;
        }
        if (S == len) continue;  // nothing above the mean: the last particle goes up, no swaps
        int run = 0;
        for (int k0 = 0; k0 < len; k0 += 32) {
            const int p = k0 + lane;
            const bool in = p < len;
            const bool small = in && !(cd[p] > mean);
            const unsigned m = __ballot_sync(0xffffffffu, small);
            const int r = run + __popc(m & lt);
            if (in) {
                if (p < S) b.bigslot[start + p] = small ? -1 : (p - r);
                else if (small) b.smallpos[start + (S - 1 - r)] = p;
            }
            run += __popc(m);
        }
        __syncwarp();
        for (int p = lane; p < S; p += 32) {
            const int k = b.bigslot[start + p];
            if (k >= 0) swap_particles(b, start + p, start + b.smallpos[start + k]);
        }
        __syncwarp();
    }
}

// Each pair is exchanged by the thread of its left-region member only, so
// the exchanges are disjoint.
__global__ void k_swap(BuildBufs b, int D)
{
    const int lb = b.cnt[BC_LEVEL_BEGIN];
    const double *coord = axis_ptr(b.x, b.y, b.z, D);
    int W = b.cnt[BC_W];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int w = gw; w < W; w += nw) {
        int i = b.ch_node[w];
        int t = lb + i;
        int mode = b.tn_mode[t];
        int start = b.tn_start[t], len = b.tn_len[t];
        if (mode == 2) {
            if (lane == 0 && coord[start] > coord[start + 1]) swap_particles(b, start, start + 1);
            continue;
        }
        if (mode != 0) continue;
        int S = b.tn_S[t];
        int s0 = (w - b.tn_chunk_base[i]) * CHUNK;
        int s1 = min(min(len, s0 + CHUNK), S);
        for (int p = s0 + lane; p < s1; p += 32) {
            int k = b.bigslot[start + p];
            if (k >= 0) swap_particles(b, start + p, start + b.smallpos[start + k]);
        }
    }
}

// ---------------- renumbering ----------------
__global__ void k_subtree_counts(BuildBufs b, int d)
{
    if (d >= b.cnt[BC_NLEVELS]) return;
    const int lb = b.lvl_begin[d], C = b.lvl_count[d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        int t = lb + i;
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

// preorder node numbers and depth-first leaf numbers, src/fmm.c:101-118
__global__ void k_number(BuildBufs b, int d)
{
    if (d >= b.cnt[BC_NLEVELS]) return;
    const int lb = b.lvl_begin[d], C = b.lvl_count[d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
        int t = lb + i;
        int pre = b.tn_pre[t], lbase = b.tn_lbase[t];
        int c0 = b.tn_child0[t], c1 = b.tn_child1[t];
        int off_nodes, off_leaves;
        if (PH_IS_LEAF_CODE(c0)) { b.tl_final[~c0] = lbase; off_nodes = 0; off_leaves = 1; }
        else { b.tn_pre[c0] = pre + 1; b.tn_lbase[c0] = lbase; off_nodes = b.tn_sub_nodes[c0]; off_leaves = b.tn_sub_leaves[c0]; }
        if (PH_IS_LEAF_CODE(c1)) b.tl_final[~c1] = lbase + off_leaves;
        else { b.tn_pre[c1] = pre + 1 + off_nodes; b.tn_lbase[c1] = lbase + off_leaves; }
    }
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

// depth lists: depth d holds the level-d nodes (temp order) then the leaves
// created by level d-1 (temp order); offsets by a one-thread prefix
__global__ void k_depth_offsets(BuildBufs b, TreeBufs T, int ndepth)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int off = 0;
        const int nlev = b.cnt[BC_NLEVELS];
        int deepest = 0;
        for (int d = 0; d < ndepth; d++) {
            T.depth_off[d] = off;
            const int nc = d < nlev ? b.lvl_count[d] : 0;
            const int lc = d <= nlev ? b.leaf_count[d] : 0;
            T.depth_cnt[d] = nc + lc;
            if (nc + lc) deepest = d;
            off += nc + lc;
        }
        T.depth_off[ndepth] = off;
        b.cnt[BC_DEPTH] = deepest;
    }
}

__global__ void k_depth_lists(BuildBufs b, TreeBufs T)
{
    const int d = blockIdx.y;
    const int nlev = b.cnt[BC_NLEVELS], nleaves = b.cnt[BC_LEAVES];
    const int node_c = d < nlev ? b.lvl_count[d] : 0;
    const int node_b = d < nlev ? b.lvl_begin[d] : 0;
    const int leaf_c = d <= nlev ? b.leaf_count[d] : 0, leaf_b = d <= nlev ? b.leaf_begin[d] : 0;
    const int off = T.depth_off[d];
    const int tot = node_c + leaf_c;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += gridDim.x * blockDim.x) {
        const int u = (i < node_c) ? nleaves + b.tn_pre[node_b + i] : b.tl_final[leaf_b + (i - node_c)];
        T.depth_list[off + i] = u;
    }
}

}  // namespace

int launch_init_particles(BuildBufs &b, const double *pos, int n, cudaStream_t st)
{
    ph::note_launch(), k_init_particles<<<device_sm_count() * 8, TB, 0, st>>>(pos, n, b);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// Enqueue the whole build for at most `levels` node levels; no host sync.
// Levels past the real depth exit at once.  If nodes remain after the last
// level, PH_FLAG_DEPTH is raised in b.cnt[BC_FLAGS] (the caller grows
// `levels` and builds again); capacity overflows raise their flags there too.
// Depth lists cover depths 0..levels.
int build_tree(BuildBufs &b, TreeBufs &T, const PassParams &p, int levels, cudaStream_t st)
{
    const int maxb = device_sm_count() * 8;
    if (levels < 1 || levels + 1 > T.max_depth_cap)
        return ph_set_error(7, "tree deeper than %d levels", T.max_depth_cap - 1);
    PH_CUDA_CHECK(cudaMemsetAsync(b.lvl_count, 0, sizeof(int) * (levels + 1), st));
    PH_CUDA_CHECK(cudaMemsetAsync(b.leaf_count, 0, sizeof(int) * (levels + 2), st));
    ph::note_launch(), k_init_roots<<<(b.nbox + TB - 1) / TB, TB, 0, st>>>(b);
    for (int d = 0; d < levels; d++) {
        const int D = (p.axis0 + d) % 3;  // from direct_local_start; the axis cycles (src/fmm.c:99)
        ph::note_launch(), k_level_nch<<<maxb, TB, 0, st>>>(b);
        ph::note_launch(), k_narrow_split<<<maxb, TB, 0, st>>>(b, D, p.maxleaf);
        scan_exclusive_i32(b.tn_nch, b.tn_chunk_base, b.cnt + BC_LEVEL_COUNT, b.cap_nodes, b.cnt + BC_W,
                           b.scan_scratch, b.scan_scratch_elems, st);
        ph::note_launch(), k_chunk_map<<<maxb, TB, 0, st>>>(b);
        ph::note_launch(), k_chunk_sum<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_node_mean<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_chunk_count<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_node_split<<<maxb, TB, 0, st>>>(b, p.maxleaf);
        scan_exclusive_i32(b.tn_nodeflag, b.tn_nodebase, b.cnt + BC_LEVEL_COUNT, b.cap_nodes, b.cnt + BC_NEXT_NODES,
                           b.scan_scratch, b.scan_scratch_elems, st);
        scan_exclusive_i32(b.tn_leafflag, b.tn_leafbase, b.cnt + BC_LEVEL_COUNT, b.cap_nodes, b.cnt + BC_NEW_LEAVES,
                           b.scan_scratch, b.scan_scratch_elems, st);
        ph::note_launch(), k_make_children<<<maxb, TB, 0, st>>>(b, p.maxleaf, D);
        ph::note_launch(), k_rank<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_swap<<<maxb, TB, 0, st>>>(b, D);
        ph::note_launch(), k_level_finish<<<1, 1, 0, st>>>(b, d);
    }
    ph::note_launch(), k_tree_totals<<<1, 1, 0, st>>>(b);
    // subtree sizes bottom-up, numbers top-down
    for (int d = levels - 1; d >= 0; d--) ph::note_launch(), k_subtree_counts<<<maxb, TB, 0, st>>>(b, d);
    ph::note_launch(), k_root_bases<<<1, 1, 0, st>>>(b);
    for (int d = 0; d < levels; d++) ph::note_launch(), k_number<<<maxb, TB, 0, st>>>(b, d);
    ph::note_launch(), k_scatter_nodes<<<maxb, TB, 0, st>>>(b, T);
    ph::note_launch(), k_scatter_leaves<<<maxb, TB, 0, st>>>(b, T);
    const int ndepth = levels + 1;  // leaves can sit one level below the deepest nodes
    ph::note_launch(), k_depth_offsets<<<1, 1, 0, st>>>(b, T, ndepth);
    ph::note_launch(), k_depth_lists<<<dim3(64, ndepth), TB, 0, st>>>(b, T);
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
