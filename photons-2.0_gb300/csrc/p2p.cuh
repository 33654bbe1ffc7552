// P2P launch interface.
#pragma once

#include "fmm_context.cuh"

namespace ph {

struct SplitConsts {
    float eps2, kq, pia, clin;
    float a[8];
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
    double boxsize, eps, mass, rs;
    SplitConsts k;
    int variant;  // FP32: 0 packed (default), 1 scalar
};

SplitConsts make_split_consts(const PassParams &p);
int launch_leaf_offsets(const BuildBufs &b, const TreeBufs &t, float4 *pos4, cudaStream_t st);
int launch_p2p(const P2PArgs &a, int fp64, cudaStream_t st);

}  // namespace ph
