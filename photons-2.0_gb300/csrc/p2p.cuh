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
};

SplitConsts make_split_consts(const PassParams &p);
double split_sig(const PassParams &p);
int launch_leaf_offsets(const BuildBufs &b, const TreeBufs &t, float4 *pos4, cudaStream_t st);
int launch_p2p(const P2PArgs &a, int fp64, cudaStream_t st);

}  // namespace ph
