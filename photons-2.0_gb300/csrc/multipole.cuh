// Far-field launch interface.
#pragma once

#include "fmm_context.cuh"

namespace ph {

struct MultipoleArgs {
    const double *px, *py, *pz;
    const int *ipart, *npart, *son0, *son1, *parent;
    const double *cx, *cy, *cz;
    const int *tree_cnt;                   // device build counters (BC_LEAVES, BC_NODES)
    const unsigned long long *walk_flags;  // device walk flags; nonzero: lists incomplete, M2L does nothing
    int ndepth;                            // depths to launch (at least the tree's deepest + 1)
    const int *depth_list;
    const int *depth_off;  // device [ndepth+1]
    const uint32_t *m2l_pool;
    const long long *m2l_off;
    const int *m2l_cnt;
    double *M, *L;  // [nunified][20]
    const float4 *chi, *clo, *pos4;  // FP32 centres (hi + lo) and leaf offsets, for the split far field
    double *ax, *ay, *az;
    const int *boxid;         // box of each unified id
    const BoxParams *boxes;   // per box: mass (P2M), rs and side (M2L)
    // device switches (null: always run): gate_m for P2M/M2M, gate_l for
    // M2L/L2L/L2P; set by launch_far_gate from the walk's M2L count
    const int *gate_m, *gate_l;
    int *work;  // device counter of the split M2L's targets
};

// M2L of every list, accumulated into L
int run_m2l(const MultipoleArgs &a, cudaStream_t st);
// L2L top-down, then L2P accumulated into ax/ay/az
int run_downward(const MultipoleArgs &a, cudaStream_t st);
// split precision: FP32 M2L (M rounded into M32) and FP32 L2P after FP64 L2L
int run_m2l_f32(const MultipoleArgs &a, float *M32, cudaStream_t st);
int run_downward_f32(const MultipoleArgs &a, cudaStream_t st);
// P2M and M2M, and L zeroed for the M2L that follows
int run_p2m_m2m(const MultipoleArgs &a, cudaStream_t st);
// the far-field switches of a captured pass (gate[2], see MultipoleArgs)
int launch_far_gate(const unsigned long long *walk_ctr, int keep_multipoles, int *gate, cudaStream_t st);
// op: 0 m2l (in = M, inout = L, rs), 1 m2m (in = M, inout = M'), 2 l2l (in = L, inout = L')
int launch_op_batch(int op, int n, const double *d, const double *in, double *inout, double rs, cudaStream_t st);

}  // namespace ph
