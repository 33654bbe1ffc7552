// Dual-tree walk: interaction lists for the local tree and the 26 periodic
// images in one traversal.
//
// Restates the pair rules of src/fmm.c:406-538 (walk_task_p2p),
// src/fmm.c:569-712 (walk_task_m2l), src/remotes.c:213-372
// (walk_task_p2p_ext) and src/remotes.c:405-552 (walk_task_m2l_ext).  The
// P2P and M2L walks of the reference make the same decisions and differ
// only in what they record, so one traversal records both.  The image
// walks start from (root, shifted root) and use the sender-side pruning of
// src/remotes.c:60-169; the pruned copy is not materialised, a node's
// pruning for an image is evaluated where the walk needs it.
//
// Organisation: the walk is processed target-first.  Every pair (a, b)
// the reference visits is rewritten by one rule that either records it,
// drops it, opens the source b (pairs (a, b0), (a, b1): same target), or
// opens the target a (pairs (a0, b), (a1, b)).  Pairs that open the target
// go to a's push-down list, which both children inherit; the self pair
// (a, a) of a node pushes down (a0, a) and (a1, a) in the form of its two
// children.  So the whole walk is: for each depth, for each target at that
// depth, expand the inherited list with a warp-wide stack until only
// records and push-downs remain.  The multiset of recorded pairs is the
// reference's; only their order differs.
//
// Acceptance is evaluated in FP64 with explicit round-to-nearest operations
// (no contraction) so that every decision equals the reference's.
#include <cstdio>
#include <cstring>

#include "fmm_context.cuh"

#define WALK_TB 256

namespace ph {
namespace {

struct Geo {
    const double *cx, *cy, *cz, *wx, *wy, *wz, *wsum;
    const int *son0, *son1, *npart, *parent;
    const int2 *son;                // (son0, son1) of nodes, for one load
    const float4 *chi, *clo, *w32;  // FP32 copies: centre hi/lo, (width xyz, width sum)
};

// MAC of src/fmm.c:266-326 (LONGSHORT): 1 accept, 0 open, -1 drop
__device__ __forceinline__ int acceptance_fp64(double wi0, double wi1, double wi2, double wj0, double wj1, double wj2,
                                               double d0, double d1, double d2, double theta2, double c2)
{
    double w0 = __dmul_rn(__dadd_rn(wi0, wj0), 0.5);
    double w1 = __dmul_rn(__dadd_rn(wi1, wj1), 0.5);
    double w2 = __dmul_rn(__dadd_rn(wi2, wj2), 0.5);
    double dd2 = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
    double m0 = __dsub_rn(fabs(d0), w0), m1 = __dsub_rn(fabs(d1), w1), m2 = __dsub_rn(fabs(d2), w2);
    if (m0 <= 0.0) m0 = 0.0;
    if (m1 <= 0.0) m1 = 0.0;
    if (m2 <= 0.0) m2 = 0.0;
    if (__dadd_rn(__dadd_rn(m0, m1), m2) < 0.0001) return 0;
    double dm2 = __dadd_rn(__dadd_rn(__dmul_rn(m0, m0), __dmul_rn(m1, m1)), __dmul_rn(m2, m2));
    if (dm2 >= c2) return -1;
    if (dd2 > c2) return 0;
    double wmax = w0;
    if (w1 > wmax) wmax = w1;
    if (w2 > wmax) wmax = w2;
    wmax = __dmul_rn(wmax, 2.0);
    return (__dmul_rn(wmax, wmax) < __dmul_rn(theta2, dd2)) ? 1 : 0;
}

// (c_b + shift) - c_a along one axis from FP32 hi/lo centres: the box side
// is taken off whichever centre lies near the far face, where it is exact
__device__ __forceinline__ float centre_diff32(float hb, float lb, float ha, float la, int o, float Lhi, float Llo)
{
    if (o < 0) { hb -= Lhi; lb -= Llo; }
    else if (o > 0) { ha -= Lhi; la -= Llo; }
    return (hb - ha) + (lb - la);
}

// The MAC in FP32 with error margins.  Inputs: d = c_a - c_b' (relative
// error ~1e-7 from the hi/lo difference), FP32 widths.  Every comparison of
// the reference's sequence is decided only if the FP32 value clears its
// threshold by a margin several times the worst-case FP32 error; otherwise
// -2 is returned and the caller evaluates the exact FP64 MAC.
__device__ __forceinline__ int acceptance_fp32(float wi0, float wi1, float wi2, float wj0, float wj1, float wj2,
                                               float d0, float d1, float d2, float theta2, float c2)
{
    const float w0 = (wi0 + wj0) * 0.5f, w1 = (wi1 + wj1) * 0.5f, w2 = (wi2 + wj2) * 0.5f;
    const float a0 = fabsf(d0), a1 = fabsf(d1), a2 = fabsf(d2);
    const float u0 = a0 + w0, u1 = a1 + w1, u2 = a2 + w2;  // error scale of each gap
    float g0 = a0 - w0, g1 = a1 - w1, g2 = a2 - w2;
    g0 = g0 > 0.f ? g0 : 0.f;
    g1 = g1 > 0.f ? g1 : 0.f;
    g2 = g2 > 0.f ? g2 : 0.f;
    const float S = g0 + g1 + g2;
    const float eS = 2e-6f * (u0 + u1 + u2);
    if (S < 1e-4f - eS) return 0;        // touching
    if (S < 1e-4f + eS) {
        // Near the touching threshold (touching boxes: S = 0 up to FP32
        // error, which can exceed the window for large boxes) the answer is
        // 0 on either side of it: the gaps are too small for the cutoff drop
        // (dm2 <= S^2 < c2), and the opening-angle accept needs
        // 2 wmax < theta dd with dd <= sqrt(3) (wmax/2 + S), impossible for
        // theta <= 1 and S < 0.15 wmax/2 (wmax/2: the largest half-width sum)
        const float smax = 1e-4f + 2.f * eS, hw = fmaxf(w0, fmaxf(w1, w2));
        return (theta2 <= 1.f && smax < 0.1f * hw && smax * smax < c2) ? 0 : -2;
    }
    const float dm2 = g0 * g0 + g1 * g1 + g2 * g2;
    const float edm = 4e-6f * (g0 * u0 + g1 * u1 + g2 * u2) + 1e-6f * (dm2 + c2);
    if (dm2 >= c2 + edm) return -1;      // beyond the cutoff
    if (dm2 > c2 - edm) return -2;
    const float dd2 = d0 * d0 + d1 * d1 + d2 * d2;
    const float edd = 2e-6f * (dd2 + c2);
    if (dd2 > c2 + edd) return 0;
    if (dd2 >= c2 - edd) return -2;
    float wmax = fmaxf(w0, fmaxf(w1, w2)) * 2.f;
    const float lhs = wmax * wmax, rhs = theta2 * dd2;
    const float ew = 2e-6f * (lhs + rhs);
    if (lhs < rhs - ew) return 1;
    if (lhs > rhs + ew) return 0;
    return -2;
}

struct WalkArgs {
    Geo g;
    WalkBufs w;
    const int *depth_list;
    const int *depth_off;  // device [depth+2]: this depth's slice of depth_list
    const int *tree_cnt;   // device build counters: leaves at BC_LEAVES (the root is unified id nleaf)
    int depth;
    int nroot;               // entries of the root's list: (root, img) for the selected images
    int root_img[PH_NIMG];
    const int *boxid;        // box of each unified id
    const BoxParams *boxes;  // per box: side, rcut, root
    double theta2, theta;
    float theta2f;
    float prune_k2f;  // (0.95 theta)^2 in FP32: the image pruning rule's width test
    WalkImports imp;  // received trees (none outside a rank's domain pass)
    int maxleaf;
};

// a source is a leaf: a local leaf, or a received node of <= MAXLEAF particles
__device__ __forceinline__ bool source_is_leaf(const WalkArgs &A, int b, int nleaf)
{
    return b < nleaf || (b >= A.imp.base && A.g.npart[b] <= A.maxleaf);
}

// sender-side pruning of an image node, src/remotes.c:97-158
__device__ __forceinline__ bool image_pruned(const WalkArgs &A, int r, double rcut, int b, double s0, double s1,
                                             double s2)
{
    const Geo &g = A.g;
    double sx[3] = {s0, s1, s2};
    double rc[3] = {g.cx[r], g.cy[r], g.cz[r]}, rw[3] = {g.wx[r], g.wy[r], g.wz[r]};
    double bc[3] = {g.cx[b], g.cy[b], g.cz[b]}, bw[3] = {g.wx[b], g.wy[b], g.wz[b]};
    double dr = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double gap = __dsub_rn(__dsub_rn(rc[d], bc[d]), sx[d]);
        if (gap < 0.0) gap = -gap;
        gap = __dsub_rn(gap, __dmul_rn(__dadd_rn(rw[d], bw[d]), 0.5));
        if (gap > 0.0) dr = __dadd_rn(dr, __dmul_rn(gap, gap));
    }
    dr = __dsqrt_rn(dr);
    double wmax = bw[0];
    if (wmax < bw[1]) wmax = bw[1];
    if (wmax < bw[2]) wmax = bw[2];
    if (dr >= rcut) return true;
    return wmax < __dmul_rn(__dmul_rn(0.95, A.theta), dr);
}

// The pruning rule in FP32 with error margins, as acceptance_fp32 does the
// MAC: 1 pruned, 0 not, -2 too close to a threshold (the caller evaluates
// image_pruned).  d = (c_b + shift) - c_r from the hi/lo centres (relative
// error ~1e-7), FP32 widths of the receiving root r and of node b.
__device__ __forceinline__ int image_pruned_fp32(float d0, float d1, float d2, float4 rw, float4 bw, float rc2,
                                                 float k2)
{
    const float h0 = (rw.x + bw.x) * 0.5f, h1 = (rw.y + bw.y) * 0.5f, h2 = (rw.z + bw.z) * 0.5f;
    const float a0 = fabsf(d0), a1 = fabsf(d1), a2 = fabsf(d2);
    const float u0 = a0 + h0, u1 = a1 + h1, u2 = a2 + h2;  // error scale of each gap
    float g0 = a0 - h0, g1 = a1 - h1, g2 = a2 - h2;
    g0 = g0 > 0.f ? g0 : 0.f;
    g1 = g1 > 0.f ? g1 : 0.f;
    g2 = g2 > 0.f ? g2 : 0.f;
    const float dm2 = g0 * g0 + g1 * g1 + g2 * g2;
    const float edm = 4e-6f * (g0 * u0 + g1 * u1 + g2 * u2) + 1e-6f * (dm2 + rc2);
    if (dm2 >= rc2 + edm) return 1;  // dr >= rcut
    if (dm2 > rc2 - edm) return -2;
    // wmax < 0.95 theta dr, squared (k2 = (0.95 theta)^2)
    const float wmax = fmaxf(bw.x, fmaxf(bw.y, bw.z));
    const float lhs = wmax * wmax, rhs = k2 * dm2;
    const float ew = 2e-6f * (lhs + rhs) + k2 * edm;
    if (lhs < rhs - ew) return 1;
    if (lhs > rhs + ew) return 0;
    return -2;
}

enum { OUT_NONE = 0, OUT_P2P = 1, OUT_M2L = 2, OUT_PUSH = 3, OUT_OPEN = 4, OUT_SELF_PUSH = 5 };

// Per-warp stack and output staging: the first entries live in shared
// memory, the rest in the warp's global scratch (same index space).
#define WS_STACK 256
#define WS_P2P 640
#define WS_PD 448
#define WS_M2L 128
#define WS_TOTAL (WS_STACK + WS_P2P + WS_PD + WS_M2L)

__device__ __forceinline__ void put2(uint32_t *s, int scap, uint32_t *g, int pos, uint32_t v)
{
    if (pos < scap) s[pos] = v;
    else g[pos] = v;
}
__device__ __forceinline__ uint32_t get2(const uint32_t *s, int scap, const uint32_t *g, int pos)
{
    return pos < scap ? s[pos] : g[pos];
}

template <int MINB>
__global__ void __launch_bounds__(WALK_TB, MINB) k_walk_level(WalkArgs A)
{
    const Geo &g = A.g;
    WalkBufs &W = A.w;
    const int lane = warp_lane();
    const unsigned lt = (1u << lane) - 1u;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // this depth counts in the counters of its parity; the other parity's,
    // last used by the depth before, are reset for the next depth (which
    // starts after this kernel), its pool fill kept in WC_PD_MAX
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int o = (A.depth + 1) & 1;
        const unsigned long long f = W.ctr[WC_PD_FILL0 + o];
        if (f > W.ctr[WC_PD_MAX]) W.ctr[WC_PD_MAX] = f;
        W.ctr[WC_PD_FILL0 + o] = 0;
        W.ctr[WC_WORK0 + o] = 0;
    }
    if (gw >= W.nwarps) return;
    uint32_t *stack = W.scratch + (size_t)gw * (W.stack_cap + 3 * W.stage_cap);
    uint32_t *st_p2p = stack + W.stack_cap;
    uint32_t *st_m2l = st_p2p + W.stage_cap;
    uint32_t *st_pd = st_m2l + W.stage_cap;
    __shared__ uint32_t s_buf[WALK_TB / 32][WS_TOTAL];
    uint32_t *sh_stack = s_buf[threadIdx.x >> 5];
    uint32_t *sh_p2p = sh_stack + WS_STACK;
    uint32_t *sh_pd = sh_p2p + WS_P2P;
    uint32_t *sh_m2l = sh_pd + WS_PD;
    const int parity = A.depth & 1;
    const int nleaf = A.tree_cnt[BC_LEAVES];
    const int list_begin = A.depth_off[A.depth], list_end = A.depth_off[A.depth + 1];
    unsigned long long c_p2p_loc = 0, c_p2p_img = 0, c_m2l_loc = 0, c_m2l_img = 0, c_pl = 0, c_pi = 0;
    unsigned flags = 0;
    int max_stack = 0, max_stage = 0;

    // targets are handed out one at a time (their lists differ in length by
    // more than tenfold on clustered input); each is expanded by one warp
    for (;;) {
        unsigned long long tk = 0;
        if (lane == 0) tk = atomicAdd(&W.ctr[WC_WORK0 + parity], 1ULL);
        const long long ti = list_begin + (long long)__shfl_sync(0xffffffffu, tk, 0);
        if (ti >= list_end) break;
        const int a = A.depth_list[ti];
        const bool leaf_a = a < nleaf;
        // the target's box: its root (the receiving domain of the image
        // pruning), side and cutoff
        const BoxParams &B = A.boxes[A.boxid[a]];
        const int root = B.root;
        const double boxL = B.boxsize, rcut = B.rcut, c2 = B.rcut2;
        const float Lhi = B.Lhi, Llo = B.Llo, c2f = B.c2f;
        const double ca0 = g.cx[a], ca1 = g.cy[a], ca2 = g.cz[a];
        const double wa0 = g.wx[a], wa1 = g.wy[a], wa2 = g.wz[a], wsa = g.wsum[a];
        const float4 ah = g.chi[a], al = g.clo[a], aw = g.w32[a];
        const int na = g.npart[a];
        const int a0 = leaf_a ? -1 : g.son0[a], a1 = leaf_a ? -1 : g.son1[a];
        const int par = g.parent[a];
        const uint32_t *input = nullptr;
        int n_in;
        if (par < 0) {
            n_in = A.nroot + A.imp.nroot;
        } else {
            input = W.pd_pool[parity ^ 1] + W.pd_off[par];
            n_in = W.pd_cnt[par];
        }
        int top = 0, in_pos = 0;
        int n_p2p = 0, n_m2l = 0, n_pd = 0;
        for (;;) {
            // up to 64 entries per step, two per lane, stack first
            int k;
            uint32_t e[2] = {0u, 0u};
            if (top > 0) {
                k = min(64, top);
                top -= k;
                if (lane < k) e[0] = get2(sh_stack, WS_STACK, stack, top + lane);
                if (lane + 32 < k) e[1] = get2(sh_stack, WS_STACK, stack, top + lane + 32);
            } else if (in_pos < n_in) {
                k = min(64, n_in - in_pos);
                if (input) {
                    if (lane < k) e[0] = input[in_pos + lane];
                    if (lane + 32 < k) e[1] = input[in_pos + lane + 32];
                } else {
                    // the root's list: itself under each selected image, then the received trees
                    for (int s2 = 0; s2 < 2; s2++) {
                        const int i = in_pos + lane + 32 * s2;
                        if (lane + 32 * s2 < k)
                            e[s2] = i < A.nroot ? PH_ENTRY(a, A.root_img[i])
                                                : PH_ENTRY(A.imp.root[i - A.nroot], PH_IMG_IMPORT);
                    }
                }
                in_pos += k;
            } else {
                break;
            }
            __syncwarp();
            // load phase: everything both slots need, before any use
            int b[2], img[2], need[2], npb[2];
            float4 bh[2], bl[2], bw[2];
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const bool valid = lane + 32 * s < k;
                b[s] = PH_ENTRY_ID(e[s]);
                img[s] = PH_ENTRY_IMG(e[s]);
                const bool leaf_b = source_is_leaf(A, b[s], nleaf);
                const bool self = img[s] == 0 && b[s] == a;
                need[s] = valid && !self && !(leaf_a && leaf_b);
                npb[s] = (valid && !self && leaf_a && leaf_b) ? g.npart[b[s]] : 0;
                if (need[s]) {
                    bh[s] = g.chi[b[s]];
                    bl[s] = g.clo[b[s]];
                    bw[s] = g.w32[b[s]];
                }
            }
            int kind[2];
#pragma unroll
            for (int s = 0; s < 2; s++) {
                kind[s] = OUT_NONE;
                if (lane + 32 * s >= k) continue;
                const int bb = b[s], im = img[s];
                const bool leaf_b = source_is_leaf(A, bb, nleaf);
                if (im == 0 && bb == a) {
                    if (leaf_a) {
                        kind[s] = OUT_P2P;
                        c_p2p_loc++;
                        c_pl += (unsigned long long)na * (na - 1);
                    } else {
                        kind[s] = OUT_SELF_PUSH;
                    }
                } else if (leaf_a && leaf_b) {
                    kind[s] = OUT_P2P;
                    const unsigned long long pr = (unsigned long long)na * npb[s];
                    if (im == 0) { c_p2p_loc++; c_pl += pr; }
                    else { c_p2p_img++; c_pi += pr; }
                } else {
                    int mi, mj, mk;
                    image_offsets(im, mi, mj, mk);
                    const float e0 = centre_diff32(bh[s].x, bl[s].x, ah.x, al.x, mi, Lhi, Llo);
                    const float e1 = centre_diff32(bh[s].y, bl[s].y, ah.y, al.y, mj, Lhi, Llo);
                    const float e2 = centre_diff32(bh[s].z, bl[s].z, ah.z, al.z, mk, Lhi, Llo);
                    int flag = acceptance_fp32(aw.x, aw.y, aw.z, bw[s].x, bw[s].y, bw[s].z, e0, e1, e2, A.theta2f,
                                               c2f);
                    // the image shift in FP64 only where an exact decision needs it
                    // (GB300 runs FP64 at 1/64 of the FP32 rate)
                    if (flag == -2) {
                        // image node centre = local centre + shift (src/remotes.c:123-125)
                        double cb0 = g.cx[bb], cb1 = g.cy[bb], cb2 = g.cz[bb];
                        if (im) {
                            cb0 = __dadd_rn(cb0, mi * boxL);
                            cb1 = __dadd_rn(cb1, mj * boxL);
                            cb2 = __dadd_rn(cb2, mk * boxL);
                        }
                        flag = acceptance_fp64(wa0, wa1, wa2, g.wx[bb], g.wy[bb], g.wz[bb], __dsub_rn(ca0, cb0),
                                               __dsub_rn(ca1, cb1), __dsub_rn(ca2, cb2), A.theta2, c2);
                    }
                    // width-sum comparison of the open rule: FP32 decides unless the values tie
                    const bool bigger_a = (aw.w != bw[s].w) ? (aw.w > bw[s].w) : (wsa > g.wsum[bb]);
                    int kd;
                    if (flag == -1) {
                        kd = OUT_NONE;
                    } else if (im == 0) {
                        if (flag == 1) kd = OUT_M2L;
                        else if (leaf_a) kd = OUT_OPEN;
                        else if (leaf_b) kd = OUT_PUSH;
                        else kd = bigger_a ? OUT_PUSH : OUT_OPEN;
                    } else {
                        // an image node is pruned by the rule of src/remotes.c:97-158 evaluated
                        // here; a received node came without children when its sender pruned it
                        bool pruned = false;
                        if (!leaf_b) {
                            if (im == PH_IMG_IMPORT) {
                                pruned = g.son0[bb] < 0;
                            } else {
                                // the receiving root's centre against the node's, in FP32 first
                                const float4 rh = g.chi[root], rl = g.clo[root], rw = g.w32[root];
                                const float f0 = centre_diff32(bh[s].x, bl[s].x, rh.x, rl.x, mi, Lhi, Llo);
                                const float f1 = centre_diff32(bh[s].y, bl[s].y, rh.y, rl.y, mj, Lhi, Llo);
                                const float f2 = centre_diff32(bh[s].z, bl[s].z, rh.z, rl.z, mk, Lhi, Llo);
                                const int pr = image_pruned_fp32(f0, f1, f2, rw, bw[s], c2f, A.prune_k2f);
                                pruned = pr == -2 ? image_pruned(A, root, rcut, bb, mi * boxL, mj * boxL, mk * boxL)
                                                  : pr == 1;
                            }
                        }
                        if (leaf_a) kd = (flag == 1 || pruned) ? OUT_M2L : OUT_OPEN;
                        else if (flag == 1) kd = OUT_M2L;
                        else kd = (leaf_b || pruned || bigger_a) ? OUT_PUSH : OUT_OPEN;
                    }
                    if (kd == OUT_M2L) {
                        if (im == 0) c_m2l_loc++;
                        else c_m2l_img++;
                    }
                    kind[s] = kd;
                }
            }
            // children of opened sources, both slots
            int2 ch[2];
#pragma unroll
            for (int s = 0; s < 2; s++)
                if (kind[s] == OUT_OPEN) ch[s] = g.son[b[s]];
            // compaction, slot 0 then slot 1
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const int kd = kind[s];
                const unsigned mp = __ballot_sync(0xffffffffu, kd == OUT_P2P);
                const unsigned mm = __ballot_sync(0xffffffffu, kd == OUT_M2L);
                const int npush = (kd == OUT_PUSH) ? 1 : (kd == OUT_SELF_PUSH ? 2 : 0);
                const int nopen = (kd == OUT_OPEN) ? 2 : 0;
                const int push_incl = warp_incl_scan(npush);
                const int open_incl = warp_incl_scan(nopen);
                const int push_tot = shfl(push_incl, 31), open_tot = shfl(open_incl, 31);
                if (kd == OUT_P2P) {
                    const int pos = n_p2p + __popc(mp & lt);
                    if (pos < W.stage_cap) put2(sh_p2p, WS_P2P, st_p2p, pos, e[s]);
                } else if (kd == OUT_M2L) {
                    const int pos = n_m2l + __popc(mm & lt);
                    if (pos < W.stage_cap) put2(sh_m2l, WS_M2L, st_m2l, pos, e[s]);
                } else if (kd == OUT_PUSH) {
                    const int pos = n_pd + push_incl - 1;
                    if (pos < W.stage_cap) put2(sh_pd, WS_PD, st_pd, pos, e[s]);
                } else if (kd == OUT_SELF_PUSH) {
                    const int pos = n_pd + push_incl - 2;
                    if (pos + 1 < W.stage_cap) {
                        put2(sh_pd, WS_PD, st_pd, pos, PH_ENTRY(a0, 0));
                        put2(sh_pd, WS_PD, st_pd, pos + 1, PH_ENTRY(a1, 0));
                    }
                } else if (kd == OUT_OPEN) {
                    const int pos = top + open_incl - 2;
                    if (pos + 1 < W.stack_cap) {
                        put2(sh_stack, WS_STACK, stack, pos, PH_ENTRY(ch[s].x, img[s]));
                        put2(sh_stack, WS_STACK, stack, pos + 1, PH_ENTRY(ch[s].y, img[s]));
                    }
                }
                n_p2p += __popc(mp);
                n_m2l += __popc(mm);
                n_pd += push_tot;
                top += open_tot;
                if (top > W.stack_cap) {
                    flags |= PH_FLAG_STACK_OVERFLOW;
                    top = W.stack_cap;  // entries beyond were dropped; results are invalid
                }
            }
            max_stack = max(max_stack, top);
            __syncwarp();
        }
        int stage_hi = max(n_p2p, max(n_m2l, n_pd));
        max_stage = max(max_stage, stage_hi);
        if (stage_hi > W.stage_cap) flags |= PH_FLAG_STAGE_OVERFLOW;
        // commit staged lists
        long long off = 0;
        if (leaf_a) {
            if (lane == 0) off = (long long)atomicAdd((unsigned long long *)&W.ctr[WC_P2P_FILL], (unsigned long long)n_p2p);
            off = __shfl_sync(0xffffffffu, off, 0);
            bool ok = off + n_p2p <= W.p2p_cap && n_p2p <= W.stage_cap;
            if (!ok) flags |= PH_FLAG_POOL_OVERFLOW;
            else
#pragma unroll 4
                for (int i = lane; i < n_p2p; i += 32) W.p2p_pool[off + i] = get2(sh_p2p, WS_P2P, st_p2p, i);
            if (lane == 0) { W.p2p_off[a] = ok ? off : 0; W.p2p_cnt[a] = ok ? n_p2p : 0; }
        } else {
            if (lane == 0) off = (long long)atomicAdd((unsigned long long *)&W.ctr[WC_PD_FILL0 + parity], (unsigned long long)n_pd);
            off = __shfl_sync(0xffffffffu, off, 0);
            bool ok = off + n_pd <= W.pd_cap && n_pd <= W.stage_cap;
            if (!ok) flags |= PH_FLAG_POOL_OVERFLOW;
            else
#pragma unroll 4
                for (int i = lane; i < n_pd; i += 32) W.pd_pool[parity][off + i] = get2(sh_pd, WS_PD, st_pd, i);
            if (lane == 0) { W.pd_off[a] = ok ? off : 0; W.pd_cnt[a] = ok ? n_pd : 0; }
        }
        if (lane == 0) off = (long long)atomicAdd((unsigned long long *)&W.ctr[WC_M2L_FILL], (unsigned long long)n_m2l);
        off = __shfl_sync(0xffffffffu, off, 0);
        {
            bool ok = off + n_m2l <= W.m2l_cap && n_m2l <= W.stage_cap;
            if (!ok) flags |= PH_FLAG_POOL_OVERFLOW;
            else
#pragma unroll 4
                for (int i = lane; i < n_m2l; i += 32) W.m2l_pool[off + i] = get2(sh_m2l, WS_M2L, st_m2l, i);
            if (lane == 0) { W.m2l_off[a] = ok ? off : 0; W.m2l_cnt[a] = ok ? n_m2l : 0; }
        }
        __syncwarp();
    }
    // per-warp counters
    c_p2p_loc = warp_sum_ll(c_p2p_loc);
    c_p2p_img = warp_sum_ll(c_p2p_img);
    c_m2l_loc = warp_sum_ll(c_m2l_loc);
    c_m2l_img = warp_sum_ll(c_m2l_img);
    c_pl = warp_sum_ll(c_pl);
    c_pi = warp_sum_ll(c_pi);
    if (lane == 0) {
        if (c_p2p_loc) atomicAdd(&W.ctr[WC_P2P_LOCAL], c_p2p_loc);
        if (c_p2p_img) atomicAdd(&W.ctr[WC_P2P_IMAGE], c_p2p_img);
        if (c_m2l_loc) atomicAdd(&W.ctr[WC_M2L_LOCAL], c_m2l_loc);
        if (c_m2l_img) atomicAdd(&W.ctr[WC_M2L_IMAGE], c_m2l_img);
        if (c_pl) atomicAdd(&W.ctr[WC_PAIRS_LOCAL], c_pl);
        if (c_pi) atomicAdd(&W.ctr[WC_PAIRS_IMAGE], c_pi);
        if (flags) atomicOr(&W.ctr[WC_FLAGS], (unsigned long long)flags);
        atomicMax(&W.ctr[WC_MAX_STACK], (unsigned long long)max_stack);
        atomicMax(&W.ctr[WC_MAX_STAGE], (unsigned long long)max_stage);
    }
}

// FP32 copies of the geometry for every unified id: centre as hi + lo,
// widths and width sum rounded
__global__ void k_geom32(const double *cx, const double *cy, const double *cz, const double *wx, const double *wy,
                         const double *wz, const double *wsum, const int *son0, const int *son1, const int *tree_cnt, float4 *chi,
                         float4 *clo, float4 *w32, int2 *son2)
{
    const int nu = tree_cnt[BC_LEAVES] + tree_cnt[BC_NODES];
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += gridDim.x * blockDim.x) {
        son2[u] = make_int2(son0[u], son1[u]);
        double c0 = cx[u], c1 = cy[u], c2 = cz[u];
        float h0 = (float)c0, h1 = (float)c1, h2 = (float)c2;
        chi[u] = make_float4(h0, h1, h2, 0.f);
        clo[u] = make_float4((float)(c0 - h0), (float)(c1 - h1), (float)(c2 - h2), 0.f);
        w32[u] = make_float4((float)wx[u], (float)wy[u], (float)wz[u], (float)wsum[u]);
    }
}

}  // namespace

int launch_geom32(const TreeBufs &t, const int *tree_cnt, cudaStream_t st)
{
    const int blocks = device_sm_count() * 8;
    ph::note_launch(), k_geom32<<<blocks, 256, 0, st>>>(t.cx, t.cy, t.cz, t.wx, t.wy, t.wz, t.wsum, t.son0, t.son1, tree_cnt,
                                                    t.chi, t.clo, t.w32, t.son2);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// Enqueue the walk of depths 0..ndepth-1; depths past the tree's deepest
// exit at once.  Counters and flags stay on the device (w.ctr).
int walk_lists(WalkBufs &w, const TreeBufs &t, const int *tree_cnt, const BoxParams *boxes, int ndepth,
               const PassParams &p, unsigned image_mask, cudaStream_t st, const WalkImports &imp)
{
    PH_CUDA_CHECK(cudaMemsetAsync(w.ctr, 0, sizeof(unsigned long long) * WC_N, st));
    WalkArgs A{};
    A.g.cx = t.cx; A.g.cy = t.cy; A.g.cz = t.cz;
    A.g.wx = t.wx; A.g.wy = t.wy; A.g.wz = t.wz; A.g.wsum = t.wsum;
    A.g.son0 = t.son0; A.g.son1 = t.son1; A.g.npart = t.npart; A.g.parent = t.parent;
    A.g.chi = t.chi; A.g.clo = t.clo; A.g.w32 = t.w32; A.g.son = t.son2;
    A.theta2f = (float)(p.theta * p.theta);
    A.prune_k2f = (float)((0.95 * p.theta) * (0.95 * p.theta));
    A.boxid = t.boxid;
    A.boxes = boxes;
    A.w = w;
    A.depth_list = t.depth_list;
    A.depth_off = t.depth_off;
    A.tree_cnt = tree_cnt;
    A.nroot = 0;
    for (int img = 0; img < PH_NIMG; img++)
        if (image_mask & (1u << img)) A.root_img[A.nroot++] = img;
    A.theta = p.theta;
    A.theta2 = p.theta * p.theta;
    A.imp = imp;
    A.maxleaf = p.maxleaf;
    const int blocks = (w.nwarps * 32 + WALK_TB - 1) / WALK_TB;
    for (int d = 0; d < ndepth; d++) {
        A.depth = d;
        if (w.nwarps == device_sm_count() * 3 * 8)
            ph::note_launch(), k_walk_level<3><<<blocks, WALK_TB, 0, st>>>(A);
        else
            ph::note_launch(), k_walk_level<2><<<blocks, WALK_TB, 0, st>>>(A);
    }
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace ph
