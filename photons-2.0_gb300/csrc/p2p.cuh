// P2P launch interface.
#pragma once

#include "fmm_context.cuh"

namespace ph {

struct SplitConsts {
    // scalar kernel: unscaled offsets, mass folded into a[] and clin
    float eps2, kq, pia, clin;
    float a[8];
    // packed kernel: offsets scaled by sig (exp(-u^2) = 2^(-|dx'|^2)); the
    // per-target sums are multiplied by P2PArgs::acc_scale = m sig^2
    float sig, e2s, pias, cs;
    float as[8];
};

struct P2PArgs {
    // tree (leaf part of the unified arrays)
    const int *ipart, *npart;
    const double *cx, *cy, *cz;
    const int *tree_cnt;                     // device build counters (leaves at BC_LEAVES)
    const unsigned long long *walk_flags;    // device walk flags; nonzero: lists incomplete, no work
    // lists
    const uint32_t *p2p_pool;
    const long long *p2p_off;
    const int *p2p_cnt;
    // particles (tree order)
    const float4 *pos4;  // FP32 offsets from the leaf centre
    const float4 *chi, *clo;  // leaf centres as FP32 hi + lo pairs
    const double *px, *py, *pz;
    // output (tree order); written, not accumulated
    double *ax, *ay, *az;
    int *work_counter;
    double boxsize, eps, mass, rs;  // scalar FP32 kernel (one box)
    const int *boxid;               // box of each unified id
    const BoxParams *boxes;         // per-box constants (packed FP32 and FP64 kernels)
    int nbox;
    SplitConsts k;                  // scalar kernel: all fields; packed: the polynomial coefficients
    int variant;  // FP32: 0 packed (default), 1 scalar
    int shape;    // mutual kernel build (0: by MAXLEAF; see launch_p2p_mutual)
    int bulk;     // mutual kernel: stage source leaves with TMA bulk copies (else per-lane cp.async)
    int stage_extra;  // bytes each bulk copy's mbarrier expects beyond the copy (0; a test sets 16)
};

// buffers of the mutual kernels, FP32 and FP64 (see launch_p2p_mutual)
struct MutualBufs {
    uint32_t *pool;          // the P2P pool, each target's list sorted in place
    int *sorted, *nrecv;     // per leaf: list sorted; received (lower-id) entries
    long long *size, *rbase; // per leaf: reaction floats owed to it, and their offset
    long long *total;        // device: floats needed
    long long *scan_scratch;
    int *slot;               // per pool entry: owner rank, -2 received, -1 one way
    int *over;               // device: bit 0 the reaction buffer was too small (all one way);
                             // bit 1 a source-staging copy did not land in time (pass failed)
    float *buf;              // reactions (FP64 passes: doubles over the same bytes)
    long long buf_cap;       // reaction values that fit (floats, or doubles in an FP64 pass)
    int cap_leaves;
    int2 *ev;                // per pool offset: the entries a target evaluates, packed in list order
    int *nev;                // per leaf: their number
    int maxleaf;             // selects the kernel build
    int *pq;                 // per pool entry: received rank, or the owned pair's partner position
};

SplitConsts make_split_consts(const PassParams &p);
// FP32 P2P with mutual pairs (MAXLEAF <= 64; chosen for 48-64): sorts the
// lists, pairs the entries, evaluates, adds the received reactions
int launch_p2p_mutual(const P2PArgs &a, const MutualBufs &m, int fp64, cudaStream_t st);
// the FP64 kernels' split factor g(u) at n device points (exact: erfc and exp)
int launch_split_factor_fp64(const double *u, int n, int exact, double *g, cudaStream_t st);
double split_sig(const PassParams &p);
int launch_leaf_offsets(const BuildBufs &b, const TreeBufs &t, float4 *pos4, cudaStream_t st);
int launch_p2p(const P2PArgs &a, int fp64, cudaStream_t st);
// one leaf pair in FP64 (inc/kernels.h): out[3 nt] = forces on tpos[3 nt]
// (indices tfirst..) from spos[3 ns] (indices sfirst..), equal indices skipped
int launch_leaf_pair_fp64(const double *tpos, int nt, int tfirst, const double *spos, int ns, int sfirst, double eps,
                          double mass, double rs, int exact, double *out, cudaStream_t st);

}  // namespace ph
