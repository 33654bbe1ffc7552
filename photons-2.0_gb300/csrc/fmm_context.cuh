// Device buffers of one force-pass context and the host-side entry points
// of each stage.
#pragma once

#include <vector>

#include "fmm_internal.cuh"

namespace ph {

// Tree build scratch and results.  "temp" nodes/leaves are numbered in the
// order the level-synchronous build creates them; the final (reference)
// numbering is assigned afterwards.
struct BuildBufs {
    // particles, tree order after the build
    double *x = nullptr, *y = nullptr, *z = nullptr;
    int *perm = nullptr;
    int *smallpos = nullptr;   // slot -> position of a right-region particle not above the mean
    int *bigpos = nullptr;     // slot -> position of a left-region particle above the mean
    // temp nodes
    int *tn_start = nullptr, *tn_len = nullptr, *tn_depth = nullptr, *tn_parent = nullptr;
    int *tn_child0 = nullptr, *tn_child1 = nullptr, *tn_mode = nullptr, *tn_S = nullptr;
    double *tn_box = nullptr;  // [6][cap_nodes]
    double *tn_split = nullptr;
    int *tn_nch = nullptr, *tn_chunk_base = nullptr;
    int *tn_nodeflag = nullptr, *tn_leafflag = nullptr, *tn_nodebase = nullptr, *tn_leafbase = nullptr;
    int *tn_sub_nodes = nullptr, *tn_sub_leaves = nullptr, *tn_pre = nullptr, *tn_lbase = nullptr;
    int *tn_subroot = nullptr;  // nodes of a shared-memory subtree: the subtree's root
    // temp leaves
    int *tl_start = nullptr, *tl_len = nullptr, *tl_depth = nullptr, *tl_parent = nullptr, *tl_final = nullptr;
    int *tl_subroot = nullptr;
    double *tl_box = nullptr;  // [6][cap_leaves]
    // chunks
    double *ch_partial = nullptr;
    int *ch_cnt = nullptr, *ch_small_base = nullptr, *ch_node = nullptr;
    int4 *ch_swap = nullptr;  // per chunk: node start, first slot, slots to swap
    // small device counters
    int *cnt = nullptr;  // see BuildCounter
    int *lvl_begin = nullptr, *lvl_count = nullptr;    // per node level: first temp node, count
    int *leaf_begin = nullptr, *leaf_count = nullptr;  // per depth: temp leaves created by the level above
    int *scan_scratch = nullptr;
    size_t scan_scratch_elems = 0;
    int cap_nodes = 0, cap_leaves = 0, cap_chunks = 0, cap_n = 0;
    int rule_cap = 0;  // this pass's 2N/MAXLEAF capacity (src/fmm.c:203-209), <= cap_nodes
    int *level_begin_h = nullptr;  // host copy, per level
    // boxes: temp node / leaf -> box, and the per-box table
    int *tn_boxid = nullptr, *tl_boxid = nullptr;
    BoxParams *boxes = nullptr;
    int nbox = 1;
};

enum BuildCounter {
    BC_LEVEL_COUNT = 0,   // nodes in the current level
    BC_W = 1,             // chunks in the current level
    BC_NEXT_NODES = 2,    // node children created by the current level
    BC_NEW_LEAVES = 3,    // leaf children created by the current level
    BC_LEAVES = 4,        // temp leaves so far
    BC_FLAGS = 5,
    BC_LEVEL_BEGIN = 6,   // first temp node of the current level
    BC_NODES = 7,         // temp nodes in total (after the build)
    BC_NLEVELS = 8,       // node levels built
    BC_DEPTH = 9,         // deepest depth holding a node or leaf
    BC_SUB_NODES = 10,    // nodes below the roots of shared-memory subtrees
    BC_SUB_LEAVES = 11,   // leaves of shared-memory subtrees
    BC_NEXT_WIDE = 12,    // wide nodes created by the current level
    BC_DEPTH_CELLS = 13,  // cells of the depth-list counting sort
    BC_DEPTH_TOTAL = 14,
    BC_NCOUNTERS = 16
};

// deepest tree the depth lists hold (depths 0..PH_MAX_DEPTH_CAP-1)
#define PH_MAX_DEPTH_CAP 2048

// Final tree in unified index space (leaves then nodes).
struct TreeBufs {
    int cap_u = 0;
    int *ipart = nullptr, *npart = nullptr, *depth = nullptr, *parent = nullptr;
    int *son0 = nullptr, *son1 = nullptr;  // unified ids (nodes only)
    double *cx = nullptr, *cy = nullptr, *cz = nullptr;
    double *wx = nullptr, *wy = nullptr, *wz = nullptr;
    double *wsum = nullptr, *split = nullptr;
    float4 *chi = nullptr, *clo = nullptr, *w32 = nullptr;  // FP32 copies (centre hi/lo, widths + sum)
    int *boxid = nullptr;                                    // box of each unified id
    int2 *son2 = nullptr;                                    // (son0, son1)
    // per-depth lists of unified ids
    int *depth_off = nullptr;   // [max_depth+2]
    int *depth_list = nullptr;  // [cap_u]
    int *depth_cnt = nullptr;   // [max_depth+1]
    int max_depth_cap = 0;
    int *depth_blk = nullptr;   // counting-sort cells and their scan, 2 x max_depth_cap x depth_nblk
    int depth_nblk = 0;
};

struct TreeInfo {
    int nleaf = 0, nnode = 0, depth = 0;  // depth = deepest level index
    int levels = 0, flags = 0;
    int nleaf_cap = 0, nnode_cap = 0;      // the reference's 2N/MAXLEAF capacity
    std::vector<int> depth_off;            // host copy of TreeBufs::depth_off
};

enum WalkCounter {
    WC_PD_FILL0 = 0, WC_PD_FILL1, WC_P2P_FILL, WC_M2L_FILL,
    WC_P2P_LOCAL, WC_P2P_IMAGE, WC_M2L_LOCAL, WC_M2L_IMAGE,
    WC_PAIRS_LOCAL, WC_PAIRS_IMAGE, WC_FLAGS, WC_MAX_STACK, WC_MAX_STAGE, WC_PD_MAX,
    WC_WORK0, WC_WORK1,  // next target of the depth being walked (depth parity)
    WC_N
};

// Interaction lists.  P2P lists are per target leaf, M2L lists per target
// (leaf or node), push-down lists per node (consumed by its children at the
// next depth; two pools alternate by depth parity).
struct WalkBufs {
    uint32_t *pd_pool[2] = {nullptr, nullptr};
    long long pd_cap = 0;
    long long *pd_off = nullptr;
    int *pd_cnt = nullptr;
    uint32_t *p2p_pool = nullptr;
    long long p2p_cap = 0;
    long long *p2p_off = nullptr;
    int *p2p_cnt = nullptr;
    uint32_t *m2l_pool = nullptr;
    long long m2l_cap = 0;
    long long *m2l_off = nullptr;
    int *m2l_cnt = nullptr;
    uint32_t *scratch = nullptr;  // per resident warp: stack, then three staging areas
    int nwarps = 0, stack_cap = 0, stage_cap = 0;
    unsigned long long *ctr = nullptr;  // WalkCounter
};

struct WalkStats {
    unsigned long long c[WC_N];
};

// Everything below only enqueues work on st; tree sizes are read on the
// device from tree_cnt (the build counters, BuildBufs::cnt).
int launch_geom32(const TreeBufs &t, const int *tree_cnt, cudaStream_t st);
// Trees received from other ranks, appended to the unified arrays from
// unified id `base` on: the walk adds (root[k], PH_IMG_IMPORT) to the local
// root's list.  A received node is a leaf iff it holds <= MAXLEAF
// particles; a node sent without children (son0 < 0) was pruned by its
// sender.  Only for a pass over one box.
struct WalkImports {
    const int *root = nullptr;  // device: first unified id of each received tree
    int nroot = 0;
    int base = 0x7fffffff;      // unified id of the first received node
};

// image_mask: bit 0 the local tree, bit k the k-th periodic image;
// ndepth = depths to launch (at least the tree's deepest + 1)
int walk_lists(WalkBufs &w, const TreeBufs &t, const int *tree_cnt, const BoxParams *boxes, int ndepth,
               const PassParams &p, unsigned image_mask, cudaStream_t st, const WalkImports &imp = WalkImports());

// top: launched levels of wide nodes (<= levels); levels: depth bound
int build_tree(BuildBufs &b, TreeBufs &t, const PassParams &p, int levels, int top, cudaStream_t st);
int depth_sort_blocks(int cap_u);
int read_tree_info(const BuildBufs &b, const TreeBufs &t, int levels, TreeInfo &info);

}  // namespace ph
