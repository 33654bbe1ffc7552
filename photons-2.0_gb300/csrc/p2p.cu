// Near-field (P2P) kernels: the softened, erfc-truncated pair force of
// src/fmm.c:823-855 (local tasks) and src/remotes.c:26-56 (image tasks),
//     a_i += m * g(r / 2rs) * (x_j - x_i) / max(r, eps)^3,
//     g(u) = erfc(u) + (2/sqrt(pi)) u exp(-u^2),
// over each target leaf's list of source leaves.
//
// Work decomposition (both variants): one warp per target leaf, leaves
// taken from a global counter in index (= spatial) order.  The warp stages
// its sources in shared memory and lanes are (target particle, source
// stream) pairs: with m <= 32 targets in a round, 32/m streams each take
// every (32/m)-th staged source, so small leaves still fill the warp.
// Partial sums of the streams are combined at the end in a fixed order.
//
// Split-precision variant (FP32): particles are stored as FP32 offsets from
// their own leaf centre.  Per task the centre difference (c_s + shift) - c_t
// is formed in FP64 and rounded once; staged sources are then FP32
// positions relative to the target leaf's centre, so every pair costs FP32
// arithmetic only.  g is evaluated as exp(-u^2) (t P(t) + (2/sqrt(pi)) u)
// with t = 1/(1 + p u) (coefficients from fit_split_kernel.py).  Each
// lane's partial sum over one staged batch is added to its running sum with
// Kahan compensation.
//
// FP64 variant: the reference's pair force in FP64 on absolute positions,
// image positions formed as pos + shift like the exported bodies of
// src/remotes.c:83-89, self pair skipped by index.  1/r comes from rsqrt and
// g(u) = erfc(u) + (2/sqrt(pi)) u exp(-u^2) from piecewise polynomials
// (fit_split_fp64.py, within 5.3e-17 of g), which is fewer FP64 operations
// than the reference's sqrt, division, erfc and exp and agrees with them to
// a few ulp of the force.
#include <cmath>

#include "fmm_context.cuh"
#include "p2p.cuh"
#include "split_kernel_coeffs.h"
#include "split_fp64_table.h"

#define P2P_TB 256
#define P2P_WARPS (P2P_TB / 32)
#define STAGE32 256  // staged sources per warp, FP32 variant
#define STAGE64 128  // staged sources per warp, FP64 variant

#ifndef P2P_MINB
#define P2P_MINB 3  // resident blocks per SM the packed kernel is compiled for (80 registers)
#endif
#ifndef P2P_FP64_FAST
#define P2P_FP64_FAST 1  // 0: sqrt, division, erfc and exp as written in the reference
#endif
#ifndef P2P_DUAL_UNROLL
#define P2P_DUAL_UNROLL 2  // two source pairs per step of the dual sweep: four independent chains per lane
#endif
constexpr int kDualUnroll = P2P_DUAL_UNROLL;
#ifndef P2P_ROUND_UNROLL
#define P2P_ROUND_UNROLL 4  // source pairs per step of a single round (leaves of up to 32 in one-way passes)
#endif
constexpr int kRoundUnroll = P2P_ROUND_UNROLL;

namespace ph {
namespace {

__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float a)
{
    float y = a - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// kahan_add on both halves of a float2 with the paired FP32 instructions:
// per element the same operations and roundings
__device__ __forceinline__ void kahan_add2(float2 &s, float2 &c, float2 a)
{
    const float2 y = __fadd2_rn(a, make_float2(-c.x, -c.y));
    const float2 t = __fadd2_rn(s, y);
    c = __fadd2_rn(__fadd2_rn(t, make_float2(-s.x, -s.y)), make_float2(-y.x, -y.y));
    s = t;
}

__device__ __forceinline__ void leaf_shift(int img, double L, double &s0, double &s1, double &s2)
{
    int mi, mj, mk;
    image_offsets(img, mi, mj, mk);
    s0 = mi * L;
    s1 = mj * L;
    s2 = mk * L;
}

// ---------------------------------------------------------------------
// FP32 split-precision kernel
// ---------------------------------------------------------------------
// target leaves of this pass; none if the walk overflowed a list pool
// (its lists are then incomplete and the pass is repeated with larger pools)
__device__ __forceinline__ int p2p_targets(const P2PArgs &A)
{
    return *A.walk_flags ? 0 : A.tree_cnt[BC_LEAVES];
}

__global__ void __launch_bounds__(P2P_TB) k_p2p_split(P2PArgs A)
{
    __shared__ float4 s_src[P2P_WARPS][STAGE32];
    __shared__ double s_red[P2P_WARPS][32][3];
    const int lane = warp_lane();
    const int wib = threadIdx.x >> 5;
    float4 *src = s_src[wib];
    const SplitConsts K = A.k;

    const int nleaf = p2p_targets(A);
    for (;;) {
        int t;
        if (lane == 0) t = atomicAdd(A.work_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= nleaf) break;
        const int nt = A.npart[t], it = A.ipart[t];
        if (nt == 0) continue;
        const double ct0 = A.cx[t], ct1 = A.cy[t], ct2 = A.cz[t];
        const long long eoff = A.p2p_off[t];
        const int ecnt = A.p2p_cnt[t];

        for (int r0 = 0; r0 < nt; r0 += 32) {
            const int m = min(32, nt - r0);
            const int G = 32 / m;
            const int q = lane % m, kstream = lane / m;
            const bool active = kstream < G;
            float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
            if (active) oi = A.pos4[it + r0 + q];
            float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;

            int e = 0;
            while (e < ecnt) {
                // lane i owns entry e+i: its source leaf, size and centre offset
                const int ne = min(32, ecnt - e);
                int is = 0, ns = 0;
                float d0 = 0.f, d1 = 0.f, d2 = 0.f;
                if (lane < ne) {
                    uint32_t en = A.p2p_pool[eoff + e + lane];
                    int s = PH_ENTRY_ID(en), img = PH_ENTRY_IMG(en);
                    is = A.ipart[s];
                    ns = A.npart[s];
                    double cs0 = A.cx[s], cs1 = A.cy[s], cs2 = A.cz[s];
                    if (img) {
                        double h0, h1, h2;
                        leaf_shift(img, A.boxsize, h0, h1, h2);
                        cs0 += h0; cs1 += h1; cs2 += h2;
                    }
                    d0 = (float)(cs0 - ct0);
                    d1 = (float)(cs1 - ct1);
                    d2 = (float)(cs2 - ct2);
                }
                int incl = warp_incl_scan(ns);
                // take the longest prefix of entries that fits the stage
                unsigned fit = __ballot_sync(0xffffffffu, lane < ne && incl <= STAGE32);
                int nfit = __popc(fit);  // entries are <= MAXLEAF <= STAGE64 < STAGE32, so nfit >= 1
                if (nfit == 0) break;    // unreachable under the MAXLEAF bound; never spin
                int nstaged = __shfl_sync(0xffffffffu, incl, nfit - 1);
                int base = incl - ns;
                if (lane < nfit) {
                    for (int j = 0; j < ns; j++) {
                        float4 o = A.pos4[is + j];
                        src[base + j] = make_float4(o.x + d0, o.y + d1, o.z + d2, 0.f);
                    }
                }
                __syncwarp();
                if (active) {
                    float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll 4
                    for (int j = kstream; j < nstaged; j += G) {
                        float4 sj = src[j];
                        float dx = sj.x - oi.x, dy = sj.y - oi.y, dz = sj.z - oi.z;
                        float qq = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                        qq = fmaxf(qq, K.eps2);
                        float rinv = rsqrt_approx(qq);
                        float r = qq * rinv;
                        float tt = rcp_approx(fmaf(K.pia, r, 1.0f));
                        float P = K.a[5];
                        P = fmaf(P, tt, K.a[4]);
                        P = fmaf(P, tt, K.a[3]);
                        P = fmaf(P, tt, K.a[2]);
                        P = fmaf(P, tt, K.a[1]);
                        P = fmaf(P, tt, K.a[0]);
                        float h = fmaf(tt, P, K.clin * r);
                        float ex = ex2_approx(qq * K.kq);
                        float rinv2 = rinv * rinv;
                        float f = (ex * h) * (rinv2 * rinv);
                        ax = fmaf(dx, f, ax);
                        ay = fmaf(dy, f, ay);
                        az = fmaf(dz, f, az);
                    }
                    kahan_add(sx, cx, ax);
                    kahan_add(sy, cy, ay);
                    kahan_add(sz, cz, az);
                }
                __syncwarp();
                e += nfit;
            }
            // combine the streams of each target in a fixed order
            double* red = &s_red[wib][0][0];
            red[3 * lane + 0] = (double)sx - (double)cx;
            red[3 * lane + 1] = (double)sy - (double)cy;
            red[3 * lane + 2] = (double)sz - (double)cz;
            __syncwarp();
            if (lane < m) {
                double a0 = 0.0, a1 = 0.0, a2 = 0.0;
                for (int k = 0; k < G; k++) {
                    int l = k * m + lane;
                    a0 += red[3 * l]; a1 += red[3 * l + 1]; a2 += red[3 * l + 2];
                }
                int ip = it + r0 + lane;
                A.ax[ip] += a0;
                A.ay[ip] += a1;
                A.az[ip] += a2;
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------
// FP32 split-precision kernel, packed (the default).
//
// * Centre differences without FP64: every leaf centre is kept as an FP32
//   pair hi + lo.  For an image shift of +-L along an axis the L is taken off
//   whichever centre lies near the far face (target for +L, source for -L),
//   where the subtraction is exact; then (hi_s - hi_t) + (lo_s - lo_t) is
//   exact up to the final rounding.
// * Staging: one lane per staged source (coalesced loads, conflict-free
//   shared stores); the lane finds its list entry by a binary search over
//   the 32 entries' prefix counts held in the warp.
// * Lanes: a block of up to 64 targets is taken in at most two rounds of
//   m = 32, 16, ..., 1 targets with 32/m source streams each; both rounds
//   run over every staged batch, accumulating in registers.
// * Arithmetic: two sources per lane per step with the paired FP32
//   instructions of sm_100+; each stream's batch partial is added to its
//   running sum with Kahan compensation.
// ---------------------------------------------------------------------
#define STAGE2 384  // staged sources per warp; 3 x 8 warps x 386 floats + reduction fit 48 KB

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float4 scaled(float4 o, float k) { return make_float4(o.x * k, o.y * k, o.z * k, 0.f); }

// Pair factor in scaled coordinates x' = sig x, sig^2 = log2(e) / (4 rs^2),
// so that exp(-u^2) = 2^(-|dx'|^2).  With t = 1 / (1 + p u) and r rinv = 1,
//   m g(u) / r^3 dx = m sig^2 * ex rinv'^2 (t P(t) rinv' + c') dx',
// c' = (2/sqrt(pi)) ia / sig; the constant m sig^2 is applied per target.
// FP32-pipe work per pair: 3 dx + 3 |dx|^2 + 1 r + 1 den + 5 Horner + 2 for
// t P rinv' + c' + 3 products + 3 accumulations = 21, plus rsqrt, rcp, ex2.
__device__ __forceinline__ float2 pair_factor(float2 qq, const SplitConsts &K, float2 pia2, float2 one2, float2 c2,
                                              float2 a0, float2 a1, float2 a2, float2 a3, float2 a4, float2 a5)
{
    qq.x = fmaxf(qq.x, K.e2s);
    qq.y = fmaxf(qq.y, K.e2s);
    const float2 rinv = make_float2(rsqrt_approx(qq.x), rsqrt_approx(qq.y));
    const float2 r = __fmul2_rn(qq, rinv);
    const float2 den = __ffma2_rn(pia2, r, one2);
    const float2 tt = make_float2(rcp_approx(den.x), rcp_approx(den.y));
    float2 P = __ffma2_rn(a5, tt, a4);
    P = __ffma2_rn(P, tt, a3);
    P = __ffma2_rn(P, tt, a2);
    P = __ffma2_rn(P, tt, a1);
    P = __ffma2_rn(P, tt, a0);
    const float2 g1 = __ffma2_rn(__fmul2_rn(tt, rinv), P, c2);
    const float2 ex = make_float2(ex2_approx(-qq.x), ex2_approx(-qq.y));
    return __fmul2_rn(__fmul2_rn(ex, __fmul2_rn(rinv, rinv)), g1);
}

// IL target pairs of one source, evaluated stage by stage so that the IL
// dependency chains interleave; accumulates into the target sums and the
// source's reaction sums
template <int IL>
__device__ __forceinline__ void mu_pairs(float2 sx, float2 sy, float2 sz, const float2 *nx, const float2 *ny,
                                         const float2 *nz, float2 *ax, float2 *ay, float2 *az, float2 &rx,
                                         float2 &ry, float2 &rz, bool owned, const SplitConsts &K, float2 pia2,
                                         float2 one2, float2 c2, float2 a0, float2 a1, float2 a2, float2 a3,
                                         float2 a4, float2 a5)
{
    float2 dx[IL], dy[IL], dz[IL], qq[IL], rinv[IL], tt[IL], P[IL], ex[IL];
#pragma unroll
    for (int k = 0; k < IL; k++) {
        dx[k] = __fadd2_rn(sx, nx[k]);
        dy[k] = __fadd2_rn(sy, ny[k]);
        dz[k] = __fadd2_rn(sz, nz[k]);
    }
#pragma unroll
    for (int k = 0; k < IL; k++) {
        qq[k] = __fmul2_rn(dx[k], dx[k]);
        qq[k] = __ffma2_rn(dy[k], dy[k], qq[k]);
        qq[k] = __ffma2_rn(dz[k], dz[k], qq[k]);
        qq[k].x = fmaxf(qq[k].x, K.e2s);
        qq[k].y = fmaxf(qq[k].y, K.e2s);
    }
#pragma unroll
    for (int k = 0; k < IL; k++) rinv[k] = make_float2(rsqrt_approx(qq[k].x), rsqrt_approx(qq[k].y));
#pragma unroll
    for (int k = 0; k < IL; k++) {
        const float2 den = __ffma2_rn(pia2, __fmul2_rn(qq[k], rinv[k]), one2);
        tt[k] = make_float2(rcp_approx(den.x), rcp_approx(den.y));
    }
#pragma unroll
    for (int k = 0; k < IL; k++) ex[k] = make_float2(ex2_approx(-qq[k].x), ex2_approx(-qq[k].y));
#pragma unroll
    for (int k = 0; k < IL; k++) P[k] = __ffma2_rn(a5, tt[k], a4);
#pragma unroll
    for (int k = 0; k < IL; k++) P[k] = __ffma2_rn(P[k], tt[k], a3);
#pragma unroll
    for (int k = 0; k < IL; k++) P[k] = __ffma2_rn(P[k], tt[k], a2);
#pragma unroll
    for (int k = 0; k < IL; k++) P[k] = __ffma2_rn(P[k], tt[k], a1);
#pragma unroll
    for (int k = 0; k < IL; k++) P[k] = __ffma2_rn(P[k], tt[k], a0);
#pragma unroll
    for (int k = 0; k < IL; k++) {
        const float2 g1 = __ffma2_rn(__fmul2_rn(tt[k], rinv[k]), P[k], c2);
        const float2 f = __fmul2_rn(__fmul2_rn(ex[k], __fmul2_rn(rinv[k], rinv[k])), g1);
        ax[k] = __ffma2_rn(dx[k], f, ax[k]);
        ay[k] = __ffma2_rn(dy[k], f, ay[k]);
        az[k] = __ffma2_rn(dz[k], f, az[k]);
        if (owned) {
            rx = __ffma2_rn(dx[k], f, rx);
            ry = __ffma2_rn(dy[k], f, ry);
            rz = __ffma2_rn(dz[k], f, rz);
        }
    }
}

// one round's share of a staged batch: stream k takes source pairs k, k+G, ...
__device__ __forceinline__ void p2p_round(const float2 *__restrict__ X2, const float2 *__restrict__ Y2,
                                          const float2 *__restrict__ Z2, int npairs, int k, int G, float ox,
                                          float oy, float oz, const SplitConsts &K, float &rx, float &ry, float &rz)
{
    const float2 nox = f2(-ox), noy = f2(-oy), noz = f2(-oz);
    const float2 pia2 = f2(K.pias), c2 = f2(K.cs), one2 = f2(1.0f);
    const float2 a0 = f2(K.as[0]), a1 = f2(K.as[1]), a2 = f2(K.as[2]), a3 = f2(K.as[3]), a4 = f2(K.as[4]),
                 a5 = f2(K.as[5]);
    float2 ax = f2(0.f), ay = f2(0.f), az = f2(0.f);
#pragma unroll kRoundUnroll
    for (int pp = k; pp < npairs; pp += G) {
        const float2 dx = __fadd2_rn(X2[pp], nox);
        const float2 dy = __fadd2_rn(Y2[pp], noy);
        const float2 dz = __fadd2_rn(Z2[pp], noz);
        float2 qq = __fmul2_rn(dx, dx);
        qq = __ffma2_rn(dy, dy, qq);
        qq = __ffma2_rn(dz, dz, qq);
        const float2 f = pair_factor(qq, K, pia2, one2, c2, a0, a1, a2, a3, a4, a5);
        ax = __ffma2_rn(dx, f, ax);
        ay = __ffma2_rn(dy, f, ay);
        az = __ffma2_rn(dz, f, az);
    }
    rx = ax.x + ax.y;
    ry = ay.x + ay.y;
    rz = az.x + az.y;
}

// two targets of equal stream layout in one sweep over the stage: each
// source pair is loaded once and feeds two independent dependency chains
__device__ __forceinline__ void p2p_round_dual(const float2 *__restrict__ X2, const float2 *__restrict__ Y2,
                                               const float2 *__restrict__ Z2, int npairs, int k, int G, float4 oA,
                                               float4 oB, const SplitConsts &K, float &rAx, float &rAy, float &rAz,
                                               float &rBx, float &rBy, float &rBz)
{
    const float2 pia2 = f2(K.pias), c2 = f2(K.cs), one2 = f2(1.0f);
    const float2 a0 = f2(K.as[0]), a1 = f2(K.as[1]), a2 = f2(K.as[2]), a3 = f2(K.as[3]), a4 = f2(K.as[4]),
                 a5 = f2(K.as[5]);
    const float2 nAx = f2(-oA.x), nAy = f2(-oA.y), nAz = f2(-oA.z);
    const float2 nBx = f2(-oB.x), nBy = f2(-oB.y), nBz = f2(-oB.z);
    float2 ax = f2(0.f), ay = f2(0.f), az = f2(0.f), bx = f2(0.f), by = f2(0.f), bz = f2(0.f);
#pragma unroll kDualUnroll
    for (int pp = k; pp < npairs; pp += G) {
        const float2 X = X2[pp], Y = Y2[pp], Z = Z2[pp];
#pragma unroll
        for (int w = 0; w < 2; w++) {
            const float2 dx = __fadd2_rn(X, w ? nBx : nAx);
            const float2 dy = __fadd2_rn(Y, w ? nBy : nAy);
            const float2 dz = __fadd2_rn(Z, w ? nBz : nAz);
            float2 qq = __fmul2_rn(dx, dx);
            qq = __ffma2_rn(dy, dy, qq);
            qq = __ffma2_rn(dz, dz, qq);
            const float2 f = pair_factor(qq, K, pia2, one2, c2, a0, a1, a2, a3, a4, a5);
            if (w) {
                bx = __ffma2_rn(dx, f, bx);
                by = __ffma2_rn(dy, f, by);
                bz = __ffma2_rn(dz, f, bz);
            } else {
                ax = __ffma2_rn(dx, f, ax);
                ay = __ffma2_rn(dy, f, ay);
                az = __ffma2_rn(dz, f, az);
            }
        }
    }
    rAx = ax.x + ax.y; rAy = ay.x + ay.y; rAz = az.x + az.y;
    rBx = bx.x + bx.y; rBy = by.x + by.y; rBz = bz.x + bz.y;
}

// centre difference (c_s + shift) - c_t per axis from hi/lo parts
__device__ __forceinline__ float centre_diff(float hs, float ls, float ht, float lt, int o, float Lhi, float Llo)
{
    if (o < 0) { hs -= Lhi; ls -= Llo; }
    else if (o > 0) { ht -= Lhi; lt -= Llo; }
    return (hs - ht) + (ls - lt);
}

__global__ void __launch_bounds__(P2P_TB, P2P_MINB) k_p2p_split_packed(P2PArgs A)
{
    __shared__ __align__(16) float s_x[P2P_WARPS][STAGE2 + 2];
    __shared__ __align__(16) float s_y[P2P_WARPS][STAGE2 + 2];
    __shared__ __align__(16) float s_z[P2P_WARPS][STAGE2 + 2];
    __shared__ double s_red[P2P_WARPS][32][3];
    const int lane = warp_lane();
    const int wib = threadIdx.x >> 5;
    float *sx = s_x[wib], *sy = s_y[wib], *sz = s_z[wib];
    const float2 *X2 = reinterpret_cast<const float2 *>(sx);
    const float2 *Y2 = reinterpret_cast<const float2 *>(sy);
    const float2 *Z2 = reinterpret_cast<const float2 *>(sz);
    SplitConsts K = A.k;  // polynomial coefficients; the rest per target box below

    const int nleaf = p2p_targets(A);
    for (;;) {
        int t;
        if (lane == 0) t = atomicAdd(A.work_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= nleaf) break;
        const int nt = A.npart[t], it = A.ipart[t];
        if (nt == 0) continue;
        const BoxParams &B = A.boxes[A.boxid[t]];
        K.sig = B.sig;
        K.e2s = B.e2s;
        K.pias = B.pias;
        K.cs = B.cs;
        const float Lhi = B.Lhi, Llo = B.Llo;
        const double acc_scale = B.acc_scale;
        const float4 cth = A.chi[t], ctl = A.clo[t];
        const long long eoff = A.p2p_off[t];
        const int ecnt = A.p2p_cnt[t];

        for (int tb = 0; tb < nt; tb += 64) {
            // rounds: m1 = largest power of two <= min(nb, 32); m2 covers the rest
            const int nb = min(64, nt - tb);
            const int lg1 = nb >= 32 ? 5 : 31 - __clz(nb);
            const int m1 = 1 << lg1;
            const int rest = nb - m1;
            const int lg2 = rest <= 0 ? -1 : (rest >= 32 ? 5 : 32 - __clz(rest - 1));  // ceil(log2(rest))
            const int m2 = lg2 < 0 ? 0 : (1 << lg2);
            const int G1 = 32 >> lg1, q1 = lane & (m1 - 1), k1 = lane >> lg1;
            const int G2 = m2 ? 32 >> lg2 : 1, q2 = m2 ? (lane & (m2 - 1)) : 0, k2 = m2 ? (lane >> lg2) : 0;
            const float4 o1 = scaled(A.pos4[it + tb + q1], K.sig);
            // round-2 lanes beyond the block's last target reuse it; their sums are discarded
            const float4 o2 = m2 ? scaled(A.pos4[it + tb + m1 + min(q2, rest - 1)], K.sig)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
            float s1x = 0.f, s1y = 0.f, s1z = 0.f, c1x = 0.f, c1y = 0.f, c1z = 0.f;
            float s2x = 0.f, s2y = 0.f, s2z = 0.f, c2x = 0.f, c2y = 0.f, c2z = 0.f;

            int e = 0;
            while (e < ecnt) {
                // lane i owns entry e+i: source leaf, size, centre offset
                const int ne = min(32, ecnt - e);
                int is = 0, ns = 0;
                float d0 = 0.f, d1 = 0.f, d2 = 0.f;
                if (lane < ne) {
                    uint32_t en = A.p2p_pool[eoff + e + lane];
                    int s = PH_ENTRY_ID(en), img = PH_ENTRY_IMG(en);
                    is = A.ipart[s];
                    ns = A.npart[s];
                    const float4 csh = A.chi[s], csl = A.clo[s];
                    int mi, mj, mk;
                    image_offsets(img, mi, mj, mk);
                    d0 = centre_diff(csh.x, csl.x, cth.x, ctl.x, mi, Lhi, Llo) * K.sig;
                    d1 = centre_diff(csh.y, csl.y, cth.y, ctl.y, mj, Lhi, Llo) * K.sig;
                    d2 = centre_diff(csh.z, csl.z, cth.z, ctl.z, mk, Lhi, Llo) * K.sig;
                }
                const int incl = warp_incl_scan(ns);
                const unsigned fit = __ballot_sync(0xffffffffu, lane < ne && incl <= STAGE2);
                const int nfit = __popc(fit);
                if (nfit == 0) break;  // unreachable under the MAXLEAF bound; never spin
                const int nstaged = __shfl_sync(0xffffffffu, incl, nfit - 1);
                const int pre = incl - ns;
                // cooperative staging: staged source idx -> its entry by binary search
                for (int s0 = 0; s0 < nstaged; s0 += 32) {
                    const int idx = s0 + lane;
                    int lo = 0;
#pragma unroll
                    for (int step = 16; step >= 1; step >>= 1) {
                        const int cand = lo + step;
                        const int pc = __shfl_sync(0xffffffffu, pre, cand & 31);
                        if (cand < nfit && pc <= idx) lo = cand;
                    }
                    const int eis = __shfl_sync(0xffffffffu, is, lo);
                    const int epre = __shfl_sync(0xffffffffu, pre, lo);
                    const float e0 = __shfl_sync(0xffffffffu, d0, lo);
                    const float e1 = __shfl_sync(0xffffffffu, d1, lo);
                    const float e2 = __shfl_sync(0xffffffffu, d2, lo);
                    if (idx < nstaged) {
                        const float4 o = A.pos4[eis + idx - epre];
                        sx[idx] = fmaf(o.x, K.sig, e0);
                        sy[idx] = fmaf(o.y, K.sig, e1);
                        sz[idx] = fmaf(o.z, K.sig, e2);
                    }
                }
                // an odd count gets one far-away source whose force is exactly 0
                if (lane == 0 && (nstaged & 1)) {
                    sx[nstaged] = 1e18f;
                    sy[nstaged] = 1e18f;
                    sz[nstaged] = 1e18f;
                }
                __syncwarp();
                const int npairs = (nstaged + 1) >> 1;
                float px, py, pz;
                if (m2 == m1) {
                    // equal rounds (a block of 2m targets): one sweep for both
                    float qx, qy, qz;
                    p2p_round_dual(X2, Y2, Z2, npairs, k1, G1, o1, o2, K, px, py, pz, qx, qy, qz);
                    kahan_add(s1x, c1x, px);
                    kahan_add(s1y, c1y, py);
                    kahan_add(s1z, c1z, pz);
                    kahan_add(s2x, c2x, qx);
                    kahan_add(s2y, c2y, qy);
                    kahan_add(s2z, c2z, qz);
                    __syncwarp();
                    e += nfit;
                    continue;
                }
                p2p_round(X2, Y2, Z2, npairs, k1, G1, o1.x, o1.y, o1.z, K, px, py, pz);
                kahan_add(s1x, c1x, px);
                kahan_add(s1y, c1y, py);
                kahan_add(s1z, c1z, pz);
                if (m2) {
                    p2p_round(X2, Y2, Z2, npairs, k2, G2, o2.x, o2.y, o2.z, K, px, py, pz);
                    kahan_add(s2x, c2x, px);
                    kahan_add(s2y, c2y, py);
                    kahan_add(s2z, c2z, pz);
                }
                __syncwarp();
                e += nfit;
            }
            // combine the streams of each target in a fixed order
            double *red = &s_red[wib][0][0];
            red[3 * lane + 0] = (double)s1x - (double)c1x;
            red[3 * lane + 1] = (double)s1y - (double)c1y;
            red[3 * lane + 2] = (double)s1z - (double)c1z;
            __syncwarp();
            if (lane < m1) {
                double b0 = 0.0, b1 = 0.0, b2 = 0.0;
                for (int k = 0; k < G1; k++) {
                    const int l = k * m1 + lane;
                    b0 += red[3 * l]; b1 += red[3 * l + 1]; b2 += red[3 * l + 2];
                }
                const int ip = it + tb + lane;
                A.ax[ip] += b0 * acc_scale;
                A.ay[ip] += b1 * acc_scale;
                A.az[ip] += b2 * acc_scale;
            }
            __syncwarp();
            if (m2) {
                red[3 * lane + 0] = (double)s2x - (double)c2x;
                red[3 * lane + 1] = (double)s2y - (double)c2y;
                red[3 * lane + 2] = (double)s2z - (double)c2z;
                __syncwarp();
                if (lane < rest) {
                    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
                    for (int k = 0; k < G2; k++) {
                        const int l = k * m2 + lane;
                        b0 += red[3 * l]; b1 += red[3 * l + 1]; b2 += red[3 * l + 2];
                    }
                    const int ip = it + tb + m1 + lane;
                    A.ax[ip] += b0 * acc_scale;
                    A.ay[ip] += b1 * acc_scale;
                    A.az[ip] += b2 * acc_scale;
                }
                __syncwarp();
            }
        }
    }
}

// ---------------------------------------------------------------------
// FP64 kernel: the reference's arithmetic
// ---------------------------------------------------------------------
// g(u) = erfc(u) + (2/sqrt(pi)) u exp(-u^2) (src/fmm.c:846-848) in FP64:
// piecewise polynomials of degree 8 on intervals of 1/16 (coefficients by
// fit_split_fp64.py, within 5.3e-17 of g on [0, 8)), erfc and exp beyond.
// tab: the coefficients k-major, [k][interval], in shared or global memory.
__device__ const double g_split64[SPLIT64_DEG + 1][SPLIT64_NI] = SPLIT64_C_INIT;
#define SPLIT64_N ((SPLIT64_DEG + 1) * SPLIT64_NI)

__device__ __forceinline__ double split_g_fp64(double u, const double *tab, double coeff)
{
    if (u < SPLIT64_NI * SPLIT64_W) {
        const int i = (int)(u * SPLIT64_INVW);
        const double d = u - ((double)i + 0.5) * SPLIT64_W;
        double acc = tab[SPLIT64_DEG * SPLIT64_NI + i];
#pragma unroll
        for (int k = SPLIT64_DEG - 1; k >= 0; k--) acc = fma(acc, d, tab[k * SPLIT64_NI + i]);
        return acc;
    }
    return erfc(u) + coeff * u * exp(-u * u);
}

// a block's copy of the coefficients in shared memory
__device__ __forceinline__ void load_split64(double *s_tab)
{
    for (int i = threadIdx.x; i < SPLIT64_N; i += blockDim.x) s_tab[i] = (&g_split64[0][0])[i];
    __syncthreads();
}

// the same with row k scaled by W^k (exact: W is a power of two), for the
// variable d' = d / W = t - (i + 1/2), t = u / W: Horner over the scaled
// rows gives bit for bit the unscaled result
__device__ __forceinline__ void load_split64_scaled(double *s_tab)
{
    for (int i = threadIdx.x; i < SPLIT64_N; i += blockDim.x) {
        const int k = i / SPLIT64_NI;
        s_tab[i] = ldexp((&g_split64[0][0])[i], -4 * k);
    }
    static_assert(SPLIT64_INVW == 16, "scaled rows assume intervals of 1/16");
    __syncthreads();
}

// Per-leaf constants of the mass-free FP64 pair factor
struct Pair64 {
    long long eps_bits, tmax_bits;  // eps and SPLIT64_NI as ordered bit patterns
    double ieps3, hrs, hrs_n, coeff;
};

__device__ __forceinline__ Pair64 pair64_consts(double eps, double rs)
{
    Pair64 c;
    c.eps_bits = __double_as_longlong(eps);
    c.tmax_bits = __double_as_longlong((double)SPLIT64_NI);
    c.ieps3 = 1.0 / (eps * eps * eps);
    c.hrs = 0.5 / rs;
    c.hrs_n = c.hrs * SPLIT64_INVW;
    c.coeff = 2.0 / sqrt(M_PI);
    return c;
}

// g(u) / max(r, eps)^3 for a source dx away, u = r / 2rs; the caller
// applies the mass once per target and per reaction slot.  r, eps and t
// are non-negative, so their comparisons run on bit patterns (integer pipe);
// t = u / W scales exactly, and the scaled rows (load_split64_scaled) give
// the g of split_g_fp64.  Two coincident particles get the softened factor.
__device__ __forceinline__ double pair_f_fp64(double dx, double dy, double dz, const Pair64 &c, const double *tabn)
{
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double rinv = __double_as_longlong(r2) == 0 ? 0.0 : rsqrt(r2);
    const double dr = r2 * rinv;
    const double w = __double_as_longlong(dr) < c.eps_bits ? c.ieps3 : rinv * rinv * rinv;
    const double t = dr * c.hrs_n;
    double g;
    if (__double_as_longlong(t) < c.tmax_bits) {
        const int i = (int)t;
        const double d = t - ((double)i + 0.5);
        double acc = tabn[SPLIT64_DEG * SPLIT64_NI + i];
#pragma unroll
        for (int k = SPLIT64_DEG - 1; k >= 0; k--) acc = fma(acc, d, tabn[k * SPLIT64_NI + i]);
        g = acc;
    } else {
        const double u = dr * c.hrs;
        g = erfc(u) + c.coeff * u * exp(-u * u);
    }
    return w * g;
}

// m g(u) / max(r, eps)^3 for a source dx away.  Fast form (the default):
// the same quantities with fewer FP64 operations (GB300's FP64 rate is 1/64
// of FP32): 1/r from rsqrt and g from the piecewise polynomials; two
// coincident particles get the softened factor (r = 0 < eps) as in the
// reference.
__device__ __forceinline__ double pair_ir3_fp64(double dx, double dy, double dz, double eps, double soft3,
                                                double mass, double rs, double hrs, double coeff, const double *tab)
{
#if P2P_FP64_FAST
    (void)rs;
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double rinv = r2 > 0.0 ? rsqrt(r2) : 0.0;
    const double dr = r2 * rinv;
    double ir3 = (dr < eps) ? soft3 : mass * (rinv * rinv * rinv);
    ir3 *= split_g_fp64(dr * hrs, tab, coeff);
#else
    (void)hrs;
    (void)tab;
    double dr = sqrt(dx * dx + dy * dy + dz * dz);
    double ir3 = (dr < eps) ? soft3 : mass / (dr * dr * dr);
    double drs = 0.5 * dr / rs;
    ir3 *= (erfc(drs) + coeff * drs * exp(-drs * drs));
#endif
    return ir3;
}

struct Src64 {
    double x, y, z;
    int idx;
    int pad;
};

__global__ void __launch_bounds__(P2P_TB) k_p2p_fp64(P2PArgs A)
{
    __shared__ Src64 s_src[P2P_WARPS][STAGE64];
    __shared__ double s_red[P2P_WARPS][32][3];
    __shared__ double s_tab[SPLIT64_N];
    load_split64(s_tab);
    const int lane = warp_lane();
    const int wib = threadIdx.x >> 5;
    Src64 *src = s_src[wib];
    const double coeff = 2.0 / sqrt(M_PI);

    const int nleaf = p2p_targets(A);
    for (;;) {
        int t;
        if (lane == 0) t = atomicAdd(A.work_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= nleaf) break;
        const int nt = A.npart[t], it = A.ipart[t];
        if (nt == 0) continue;
        const BoxParams &B = A.boxes[A.boxid[t]];
        const double eps = B.eps, mass = B.mass, rs = B.rs, boxL = B.boxsize;
        const double soft3 = mass / (eps * eps * eps);
        const double hrs = 0.5 / rs;  // u = r / (2 rs)
        const long long eoff = A.p2p_off[t];
        const int ecnt = A.p2p_cnt[t];
        for (int r0 = 0; r0 < nt; r0 += 32) {
            const int m = min(32, nt - r0);
            const int G = 32 / m;
            const int q = lane % m, kstream = lane / m;
            const bool active = kstream < G;
            const int ip = it + r0 + q;
            double px = 0.0, py = 0.0, pz = 0.0;
            if (active) { px = A.px[ip]; py = A.py[ip]; pz = A.pz[ip]; }
            double ax = 0.0, ay = 0.0, az = 0.0;
            int e = 0;
            while (e < ecnt) {
                const int ne = min(32, ecnt - e);
                int is = 0, ns = 0, img = 0;
                if (lane < ne) {
                    uint32_t en = A.p2p_pool[eoff + e + lane];
                    int s = PH_ENTRY_ID(en);
                    img = PH_ENTRY_IMG(en);
                    is = A.ipart[s];
                    ns = A.npart[s];
                }
                int incl = warp_incl_scan(ns);
                unsigned fit = __ballot_sync(0xffffffffu, lane < ne && incl <= STAGE64);
                int nfit = __popc(fit);
                if (nfit == 0) break;  // unreachable under the MAXLEAF bound; never spin
                int nstaged = __shfl_sync(0xffffffffu, incl, nfit - 1);
                int base = incl - ns;
                if (lane < nfit) {
                    double h0 = 0.0, h1 = 0.0, h2 = 0.0;
                    if (img) leaf_shift(img, boxL, h0, h1, h2);
                    for (int j = 0; j < ns; j++) {
                        Src64 sj;
                        sj.x = A.px[is + j] + h0;
                        sj.y = A.py[is + j] + h1;
                        sj.z = A.pz[is + j] + h2;
                        sj.idx = img ? -1 : is + j;
                        sj.pad = 0;
                        src[base + j] = sj;
                    }
                }
                __syncwarp();
                if (active) {
                    for (int j = kstream; j < nstaged; j += G) {
                        Src64 sj = src[j];
                        if (sj.idx == ip) continue;
                        double dx = sj.x - px, dy = sj.y - py, dz = sj.z - pz;
                        const double ir3 = pair_ir3_fp64(dx, dy, dz, eps, soft3, mass, rs, hrs, coeff, s_tab);
                        ax += dx * ir3;
                        ay += dy * ir3;
                        az += dz * ir3;
                    }
                }
                __syncwarp();
                e += nfit;
            }
            double *red = &s_red[wib][0][0];
            red[3 * lane + 0] = ax;
            red[3 * lane + 1] = ay;
            red[3 * lane + 2] = az;
            __syncwarp();
            if (lane < m) {
                double a0 = 0.0, a1 = 0.0, a2 = 0.0;
                for (int k = 0; k < G; k++) {
                    int l = k * m + lane;
                    a0 += red[3 * l]; a1 += red[3 * l + 1]; a2 += red[3 * l + 2];
                }
                int o = it + r0 + lane;
                A.ax[o] += a0;
                A.ay[o] += a1;
                A.az[o] += a2;
            }
            __syncwarp();
        }
    }
}

// FP32 offsets of every particle from its own leaf centre
__global__ void k_leaf_offsets(const double *px, const double *py, const double *pz, const int *ipart,
                               const int *npart, const double *cx, const double *cy, const double *cz,
                               const int *tree_cnt, float4 *pos4)
{
    const int nleaf = tree_cnt[BC_LEAVES];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int l = gw; l < nleaf; l += nw) {
        int ip = ipart[l], np = npart[l];
        double c0 = cx[l], c1 = cy[l], c2 = cz[l];
        for (int j = lane; j < np; j += 32)
            pos4[ip + j] = make_float4((float)(px[ip + j] - c0), (float)(py[ip + j] - c1), (float)(pz[ip + j] - c2), 0.f);
    }
}


// ---------------------------------------------------------------------
// FP32 split-precision P2P with mutual pairs.
//
// The P2P lists are symmetric: leaf B, shifted by the image offset s, is in
// A's list exactly when A shifted by -s is in B's (s = 0 for local pairs;
// A = B for a leaf and its own periodic image).  So each such pair is
// evaluated once.  The owner is the entry with the smaller (leaf id, image)
// key.  It computes the forces on its own particles and the equal and
// opposite reactions on the other leaf's particles, and stores those in a
// slot of a reaction buffer.  A second kernel adds each leaf's received
// reactions in list order.  Self pairs and entries whose partner is missing
// (or whose list is too long to sort) are evaluated one way.  Results are
// deterministic.
//
// Pairing: every target's list is sorted by raw entry value.  Entry (B, s)
// of A is paired when both lists are sorted and B's list holds (A, -s),
// found by binary search.  The received entries of B are numbered in list
// order.  B's k-th received slot lives at rbase[B] + 3 k r floats: x, then
// y, then z of B's nB particles, each row r = nB rounded up to 32 floats.

// Lanes: 8 target groups x 4 source groups; a lane holds 8 targets (as four
// pairs of the paired FP32 instructions) and takes 8 sources of each batch
// of 32, so reactions are summed over 8 target groups through shared memory
// and target sums over 4 source groups at the end (fixed order).
// ---------------------------------------------------------------------
#define MU_TB 128
#define MU_WARPS (MU_TB / 32)
#ifndef MU_UNROLL
#define MU_UNROLL 1
#endif
constexpr int kMuUnroll = MU_UNROLL;
#ifndef MU_FLUSH
#define MU_FLUSH 4  // evaluated entries per compensated flush of the partial sums
#endif
// Longer lists stay unsorted and are evaluated one way.  (Sorting lists of
// up to 8192 entries with a block each, so that halo leaves pair too, made
// 128^3 NFW at leaf 48 slower: 46.6 against 39.4 ms.)
#define MU_SORT_MAX 1024
// Four builds of the kernel (launch_p2p_mutual): 3 or 4 resident blocks per
// SM, one or two target pairs evaluated stage by stage together; the
// default is 4 blocks, one pair at a time, with the 6-target path for
// leaves of 33-48 (256^3 leaf 64: P2P phase 60.3 against 61.6 ms for 3
// blocks and two pairs)
#ifndef MU_BATCH
#define MU_BATCH 32  // sources per reaction reduction (32 or 16)
#endif

// Bitonic sort of a list of at most 32 R entries in registers: entry
// i = 32 r + lane in v[r] (padding 0xffffffff sorts last).  Partners at
// distance j >= 32 are in the same lane, the others one shuffle away.
template <int R>
__device__ __forceinline__ void mu_sort_regs(uint32_t *lst, int L, int lane)
{
    uint32_t v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = 32 * r + lane < L ? lst[32 * r + lane] : 0xffffffffu;
#pragma unroll
    for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int jr = j >> 5;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    if (r & jr) continue;
                    const int r2 = r | jr;
                    const bool up = ((32 * r + lane) & k) == 0;
                    const uint32_t a = v[r], b = v[r2];
                    if ((a > b) == up) { v[r] = b; v[r2] = a; }
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const uint32_t o = __shfl_xor_sync(0xffffffffu, v[r], j);
                    const bool up = ((32 * r + lane) & k) == 0, low = (lane & j) == 0;
                    v[r] = (low == up) ? min(v[r], o) : max(v[r], o);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < R; r++)
        if (32 * r + lane < L) lst[32 * r + lane] = v[r];
}

__global__ void __launch_bounds__(256) k_mu_sort(const int *tree_cnt, const unsigned long long *walk_flags,
                                                  uint32_t *pool, const long long *off, const int *cnt, int *sorted)
{
    __shared__ uint32_t s_buf[8][MU_SORT_MAX];
    const int lane = warp_lane(), wib = threadIdx.x >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int nleaf = *walk_flags ? 0 : tree_cnt[BC_LEAVES];
    uint32_t *buf = s_buf[wib];
    for (int t = gw; t < nleaf; t += nw) {
        const int L = cnt[t];
        uint32_t *lst = pool + off[t];
        const int ok = L <= MU_SORT_MAX;
        // lists of up to 256 entries (most of them) are sorted in registers
        if (L > 1 && L <= 32) {
            mu_sort_regs<1>(lst, L, lane);
        } else if (L > 32 && L <= 64) {
            mu_sort_regs<2>(lst, L, lane);
        } else if (L > 64 && L <= 128) {
            mu_sort_regs<4>(lst, L, lane);
        } else if (L > 128 && L <= 256) {
            mu_sort_regs<8>(lst, L, lane);
        } else if (ok && L > 1) {
            int P = 2;
            while (P < L) P <<= 1;
            for (int i = lane; i < P; i += 32) buf[i] = i < L ? lst[i] : 0xffffffffu;
            for (int k = 2; k <= P; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    __syncwarp();
                    for (int i = lane; i < P; i += 32) {
                        const int ixj = i ^ j;
                        if (ixj > i) {
                            const uint32_t a = buf[i], b = buf[ixj];
                            if ((a > b) == ((i & k) == 0)) {
                                buf[i] = b;
                                buf[ixj] = a;
                            }
                        }
                    }
                }
            __syncwarp();
            for (int i = lane; i < L; i += 32) lst[i] = buf[i];
            __syncwarp();
        }
        if (lane == 0) sorted[t] = ok;
    }
}

// position of value v in the sorted list lst[0, L), or -1
__device__ __forceinline__ int mu_find(const uint32_t *lst, int L, uint32_t v)
{
    int lo = 0, hi = L;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (lst[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return (lo < L && lst[lo] == v) ? lo : -1;
}

// floats per component row of a reaction slot: n rounded up to 32, so that
// every row starts on a 128-byte line
__host__ __device__ __forceinline__ int mu_row(int n) { return (n + 31) & ~31; }
// the same at granularity g (a power of two): FP64 slots pad rows to 4
// doubles, so that leaves of a few particles do not take rows of 32
__host__ __device__ __forceinline__ int mu_row_g(int n, int g) { return (n + g - 1) & ~(g - 1); }
#define MU64_ROW 4

// the image with the opposite shift (the partner of an image entry)
__device__ __forceinline__ int img_neg(int img)
{
    if (img == 0) return 0;
    const int c = img <= 13 ? img - 1 : img;  // index among the 27 cells (13 = no shift)
    const int cn = 26 - c;
    return cn <= 12 ? cn + 1 : cn;
}

// Pairing, per target t and list entry (b, img), b's list searched for the
// partner entry (t, -img).  Found: the entry with the smaller (id, image)
// key owns the pair, the other receives it.  Received entries are numbered
// in list order (their slots in t's reaction area); owned entries record the
// partner's position.  slot[e]: -1 one way, -2 received, -3 owned; pq[e]:
// the received rank, or the partner's position in b's list.
__global__ void k_mu_pair(const int *tree_cnt, const unsigned long long *walk_flags, const uint32_t *pool,
                          const long long *off, const int *cnt, const int *npart, const int *sorted, int *slot,
                          int *pq, int *nrecv, long long *size, int rowg)
{
    const int lane = warp_lane();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int nleaf = *walk_flags ? 0 : tree_cnt[BC_LEAVES];
    const unsigned below = (1u << lane) - 1u;
    for (int t = gw; t < nleaf; t += nw) {
        const long long o = off[t];
        const int L = cnt[t];
        const bool st = sorted[t];
        int recv = 0;
        for (int e0 = 0; e0 < L; e0 += 32) {
            const int e = e0 + lane;
            int kind = -1, q = -1;
            if (e < L) {
                const uint32_t v = pool[o + e];
                const int b = PH_ENTRY_ID(v), img = PH_ENTRY_IMG(v), nimg = img_neg(img);
                // received leaves (b >= nleaf) have no lists: those entries run one way
                if (st && b < nleaf && sorted[b] && !(img == 0 && b == t)) {
                    q = mu_find(pool + off[b], cnt[b], PH_ENTRY(t, nimg));
                    if (q >= 0) {
                        const unsigned long long mine = ((unsigned long long)t << 5) | (unsigned)img;
                        const unsigned long long theirs = ((unsigned long long)b << 5) | (unsigned)nimg;
                        kind = mine < theirs ? -3 : -2;
                    }
                }
            }
            const unsigned got = __ballot_sync(0xffffffffu, kind == -2);
            if (e < L) {
                slot[o + e] = kind;
                pq[o + e] = kind == -2 ? recv + __popc(got & below) : (kind == -3 ? q : -1);
            }
            recv += __popc(got);
        }
        if (lane == 0) {
            nrecv[t] = recv;
            size[t] = (long long)recv * mu_row_g(npart[t], rowg) * 3;
        }
    }
}

// Final slots once the reaction offsets are known: owned entries take the
// partner's received rank; with the reaction buffer too small every entry
// is evaluated one way.  The entries a target evaluates (all but the
// received) are packed in list order into ev[off + k] = (entry, slot),
// nev[t] of them.
__global__ void k_mu_slots(const int *tree_cnt, const unsigned long long *walk_flags, const uint32_t *pool,
                           const long long *off, const int *cnt, const long long *total, long long cap,
                           const int *pq, int *slot, int2 *ev, int *nev, int *over)
{
    const int lane = warp_lane();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int nleaf = *walk_flags ? 0 : tree_cnt[BC_LEAVES];
    const bool fits = *total <= cap;
    if (gw == 0 && lane == 0) *over = fits ? 0 : 1;
    const unsigned below = (1u << lane) - 1u;
    for (int t = gw; t < nleaf; t += nw) {
        const long long o = off[t];
        const int L = cnt[t];
        int kept = 0;
        for (int e0 = 0; e0 < L; e0 += 32) {
            const int e = e0 + lane;
            uint32_t v = 0;
            int r = -2;
            if (e < L) {
                v = pool[o + e];
                r = slot[o + e];
                if (!fits) r = -1;
                else if (r == -3) r = pq[off[PH_ENTRY_ID(v)] + pq[o + e]];
                slot[o + e] = r;
            }
            const unsigned keep = __ballot_sync(0xffffffffu, e < L && r != -2);
            if (e < L && r != -2) ev[o + kept + __popc(keep & below)] = make_int2((int)v, r);
            kept += __popc(keep);
        }
        if (lane == 0) nev[t] = kept;
    }
}

// one evaluated entry as the warp sees it: centre difference (source -
// target, scaled), source range, and where its reactions go
struct MuEntry {
    float d0, d1, d2;
    int is, ns;
    long long out;  // float offset of the pair's slot in the reaction buffer; -1: evaluated one way
};

// an entry as a warp keeps it in shared memory (24 bytes): ns (at most 64)
// in the low byte of the slot offset
struct MuMeta {
    float d0, d1, d2;
    int is;
    long long on;
};

__device__ __forceinline__ MuMeta mu_pack(const MuEntry &E)
{
    return MuMeta{E.d0, E.d1, E.d2, E.is, (long long)((unsigned long long)E.out << 8) | E.ns};
}

__device__ __forceinline__ MuEntry mu_unpack(const MuMeta &M)
{
    return MuEntry{M.d0, M.d1, M.d2, M.is, (int)(M.on & 255), M.on >> 8};
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// copy an entry's raw source offsets (leaf-centre relative) into a stage
__device__ __forceinline__ void mu_issue(const float4 *__restrict__ pos4, const MuEntry &E, float4 *buf, int lane)
{
    if (lane < E.ns) cp_async16(buf + lane, pos4 + E.is + lane);
    if (lane + 32 < E.ns) cp_async16(buf + lane + 32, pos4 + E.is + lane + 32);
}

// The same copy as one TMA bulk copy (cp.async.bulk): lane 0 arms the
// stage's mbarrier with the byte count and issues the copy; the warp waits
// on the barrier's phase.  A source leaf is contiguous in tree order, 16
// bytes a particle, so the source address, the shared stage and the size
// (16 ns bytes, at most 1 KB) are all multiples of 16.
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

// orders this thread's generic accesses to shared memory before later
// bulk-copy writes to it
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// (extra: bytes the barrier expects beyond the copy, 0 but in the test of
// the wait's time limit)
__device__ __forceinline__ void mu_issue_bulk(const float4 *__restrict__ pos4, const MuEntry &E, float4 *buf,
                                              unsigned long long *bar, int lane, int extra)
{
    if (lane != 0 || E.ns <= 0) return;
    const unsigned bytes = 16u * (unsigned)E.ns, b = smem_addr(bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b), "r"(bytes + (unsigned)extra)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_addr(buf)),
                 "l"(pos4 + E.is), "r"(bytes), "r"(b)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// waits for the barrier's phase; gives up after two seconds of global time
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned i = 1;; i++) {
        if (mbar_try(bar, parity)) return true;
        if ((i & 63u) == 0 && global_ns() - t0 > 2000000000ull) return false;
    }
}

// once the copies have landed: scale and shift them (relative to the
// target centre) from raw into buf, which may be the same stage; padding is
// far away
__device__ __forceinline__ void mu_place(const MuEntry &E, const float4 *raw, float4 *buf, float sig, int lane)
{
    const float far = 1e18f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int j = lane + 32 * h;
        float4 v = make_float4(far, far, far, 0.f);
        if (j < E.ns) {
            const float4 o = raw[j];
            v = make_float4(fmaf(o.x, sig, E.d0), fmaf(o.y, sig, E.d1), fmaf(o.z, sig, E.d2), 0.f);
        }
        buf[j] = v;
    }
}

// one target leaf with T targets per lane (8: leaves of up to 64
// particles, 4: up to 32), eight target groups x four source groups.
// Entries come in batches of 32: each lane loads one entry's metadata into
// shared memory, then the warp walks the batch with the next entry's
// sources in flight (into the second stage) while it evaluates the current
// one.  BULK: one TMA bulk copy per entry into the stage, completing on
// that stage's mbarrier (bars[c], its phase parity in bit c of phase); else
// per-lane cp.async.  Returns false if a bulk copy did not land within the
// wait's time limit (bit 1 set in *fail).
template <int T, int ILR, bool BULK>
__device__ __forceinline__ bool mu_target(const P2PArgs &A, const int2 *ev, int ne, const long long *rbase,
                                          float *rbuf, int t, int nt, int it, const SplitConsts &K, float Lhi,
                                          float Llo, float4 *src, MuMeta *meta, float *red, float *accw,
                                          unsigned long long *bars, unsigned &phase, int *fail, int lane)
{
    constexpr int TP = T / 2;  // target pairs per lane
    const int tg = lane >> 2, sg = lane & 3;
    const float far = 1e18f;
    const float2 pia2 = f2(K.pias), c2 = f2(K.cs), one2 = f2(1.0f);
    const float2 a0 = f2(K.as[0]), a1 = f2(K.as[1]), a2 = f2(K.as[2]), a3 = f2(K.as[3]), a4 = f2(K.as[4]),
                 a5 = f2(K.as[5]);
    const float4 cth = A.chi[t], ctl = A.clo[t];
    // this lane's targets as pairs, negated for dx = s - x
    float2 nx[TP], ny[TP], nz[TP];
#pragma unroll
    for (int p = 0; p < TP; p++) {
        const int q0 = tg * T + 2 * p, q1 = q0 + 1;
        const float4 o0 = q0 < nt ? scaled(A.pos4[it + q0], K.sig) : make_float4(far, far, far, 0.f);
        const float4 o1 = q1 < nt ? scaled(A.pos4[it + q1], K.sig) : make_float4(far, far, far, 0.f);
        nx[p] = make_float2(-o0.x, -o1.x);
        ny[p] = make_float2(-o0.y, -o1.y);
        nz[p] = make_float2(-o0.z, -o1.z);
    }
    // running sums: float2 (targets 2p, 2p + 1) per component, [value][lane];
    // their compensations 3 TP values further
    float2 *acc2 = reinterpret_cast<float2 *>(accw);
#pragma unroll
    for (int k = 0; k < 3 * T; k++) acc2[k * 32 + lane] = f2(0.f);
    // partial sums run over up to MU_FLUSH evaluated entries (at most 64 terms
    // per lane) before they join the compensated running sums
    float2 ax[TP], ay[TP], az[TP];
#pragma unroll
    for (int p = 0; p < TP; p++) ax[p] = ay[p] = az[p] = f2(0.f);
    int pending = 0;
    for (int k0 = 0; k0 < ne; k0 += 32) {
        const int kmax = min(32, ne - k0);
        if (lane < kmax) {
            const int2 en = ev[k0 + lane];
            const int s = PH_ENTRY_ID((uint32_t)en.x), img = PH_ENTRY_IMG((uint32_t)en.x);
            const float4 csh = A.chi[s], csl = A.clo[s];
            int mi, mj, mk;
            image_offsets(img, mi, mj, mk);
            MuEntry m;
            m.d0 = centre_diff(csh.x, csl.x, cth.x, ctl.x, mi, Lhi, Llo) * K.sig;
            m.d1 = centre_diff(csh.y, csl.y, cth.y, ctl.y, mj, Lhi, Llo) * K.sig;
            m.d2 = centre_diff(csh.z, csl.z, cth.z, ctl.z, mk, Lhi, Llo) * K.sig;
            m.is = A.ipart[s];
            m.ns = A.npart[s];
            m.out = en.y >= 0 ? rbase[s] + (long long)en.y * mu_row(m.ns) * 3 : -1;
            meta[lane] = mu_pack(m);
        }
        __syncwarp();
        int cur = 0;
        if constexpr (BULK) {
            mu_issue_bulk(A.pos4, mu_unpack(meta[0]), src, bars, lane, A.stage_extra);
        } else {
            mu_issue(A.pos4, mu_unpack(meta[0]), src, lane);
            cp_async_commit();
        }
        for (int kk = 0; kk < kmax; kk++) {
            const MuEntry E = mu_unpack(meta[kk]);
            float4 *stage = src + 64 * cur;
            if constexpr (BULK) {
                // the next entry's copy goes to the other stage (mbarrier
                // bars[cur ^ 1]) before this one's is awaited
                if (kk + 1 < kmax) mu_issue_bulk(A.pos4, mu_unpack(meta[kk + 1]), src + 64 * (cur ^ 1),
                                                 bars + (cur ^ 1), lane, A.stage_extra);
                if (E.ns > 0) {
                    // one answer for the warp, so that it stops or goes on as a whole
                    if (!__all_sync(0xffffffffu, mbar_wait(bars + cur, (phase >> cur) & 1u))) {
                        // a copy that never landed: record it, give the other
                        // stage's copy its own time limit, and stop this warp
                        if (lane == 0) atomicOr(fail, 2);
                        if (kk + 1 < kmax && mu_unpack(meta[kk + 1]).ns > 0)
                            mbar_wait(bars + (cur ^ 1), (phase >> (cur ^ 1)) & 1u);
                        return false;
                    }
                    phase ^= 1u << cur;
                }
                mu_place(E, stage, stage, K.sig, lane);
            } else {
                if (kk + 1 < kmax) mu_issue(A.pos4, mu_unpack(meta[kk + 1]), src + 64 * (cur ^ 1), lane);
                cp_async_commit();
                cp_async_wait_prev();
                mu_place(E, stage, stage, K.sig, lane);
            }
            __syncwarp();
            const int ns = E.ns;
            const bool owned = E.out >= 0;
            for (int c0 = 0; c0 < ns; c0 += MU_BATCH) {
                // the batch's sources spread evenly over the four source groups
                const int nr = min(MU_BATCH / 4, (ns - c0 + 3) >> 2);
#pragma unroll kMuUnroll
                for (int r = 0; r < nr; r++) {
                    const float4 S = stage[c0 + 4 * r + sg];
                    const float2 sx = f2(S.x), sy = f2(S.y), sz = f2(S.z);
                    float2 rx = f2(0.f), ry = f2(0.f), rz = f2(0.f);
                    // never more chains than this lane's TP target pairs
                    constexpr int IL = (ILR < TP && TP % ILR == 0) ? ILR : (TP % ILR == 0 ? TP : 1);
                    static_assert(TP % IL == 0, "target pairs in whole interleave groups");
                    if constexpr (IL > 1) {
#pragma unroll
                        for (int p = 0; p < TP; p += IL)
                            mu_pairs<IL>(sx, sy, sz, nx + p, ny + p, nz + p, ax + p, ay + p, az + p, rx, ry, rz,
                                         owned, K, pia2, one2, c2, a0, a1, a2, a3, a4, a5);
                    } else {
#pragma unroll
                        for (int p = 0; p < TP; p++) {
                            const float2 dx = __fadd2_rn(sx, nx[p]);
                            const float2 dy = __fadd2_rn(sy, ny[p]);
                            const float2 dz = __fadd2_rn(sz, nz[p]);
                            float2 qq = __fmul2_rn(dx, dx);
                            qq = __ffma2_rn(dy, dy, qq);
                            qq = __ffma2_rn(dz, dz, qq);
                            const float2 f = pair_factor(qq, K, pia2, one2, c2, a0, a1, a2, a3, a4, a5);
                            ax[p] = __ffma2_rn(dx, f, ax[p]);
                            ay[p] = __ffma2_rn(dy, f, ay[p]);
                            az[p] = __ffma2_rn(dz, f, az[p]);
                            if (owned) {
                                rx = __ffma2_rn(dx, f, rx);
                                ry = __ffma2_rn(dy, f, ry);
                                rz = __ffma2_rn(dz, f, rz);
                            }
                        }
                    }
                    if (owned) {
                        float *rr = red + (4 * r + sg) * 24 + tg;
                        rr[0] = rx.x + rx.y;
                        rr[8] = ry.x + ry.y;
                        rr[16] = rz.x + rz.y;
                    }
                }
                if (owned) {
                    // reactions of the batch's sources: minus the sum over the 8 target groups
                    __syncwarp();
                    // slot layout [component][source particle]
                    if (lane < MU_BATCH && c0 + lane < ns) {
                        float *out = rbuf + E.out + c0 + lane;
#pragma unroll
                        for (int cmp = 0; cmp < 3; cmp++) {
                            const float4 *rr = reinterpret_cast<const float4 *>(red + lane * 24 + cmp * 8);
                            const float4 u = rr[0], w = rr[1];
                            out[cmp * mu_row(ns)] = -((((u.x + u.y) + (u.z + u.w)) + ((w.x + w.y) + (w.z + w.w))));
                        }
                    }
                    __syncwarp();
                }
            }
            // every MU_FLUSH entries the partial sums join the running sums with
            // Kahan compensation (FP32: GB300's FP64 rate is 1/64 of FP32)
            if (++pending == MU_FLUSH) {
                pending = 0;
#pragma unroll
                for (int p = 0; p < TP; p++) {
                    kahan_add2(acc2[(3 * p + 0) * 32 + lane], acc2[(3 * TP + 3 * p + 0) * 32 + lane], ax[p]);
                    kahan_add2(acc2[(3 * p + 1) * 32 + lane], acc2[(3 * TP + 3 * p + 1) * 32 + lane], ay[p]);
                    kahan_add2(acc2[(3 * p + 2) * 32 + lane], acc2[(3 * TP + 3 * p + 2) * 32 + lane], az[p]);
                    ax[p] = ay[p] = az[p] = f2(0.f);
                }
            }
            // the stage is rewritten by a bulk copy in the next entry
            if constexpr (BULK) fence_proxy_async();
            __syncwarp();
            cur ^= 1;
        }
    }
#pragma unroll
    for (int p = 0; p < TP; p++) {
        kahan_add2(acc2[(3 * p + 0) * 32 + lane], acc2[(3 * TP + 3 * p + 0) * 32 + lane], ax[p]);
        kahan_add2(acc2[(3 * p + 1) * 32 + lane], acc2[(3 * TP + 3 * p + 1) * 32 + lane], ay[p]);
        kahan_add2(acc2[(3 * p + 2) * 32 + lane], acc2[(3 * TP + 3 * p + 2) * 32 + lane], az[p]);
    }
    __syncwarp();
    // targets: each lane takes one or two, summing its 4 source groups in order
    const double scale = A.boxes[A.boxid[t]].acc_scale;
    for (int tq = lane; tq < nt; tq += 32) {
        const int tgq = tq / T, q = tq - tgq * T, qp = q >> 1, qh = q & 1;
        float v[3], cmp[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            v[d] = 0.f;
            cmp[d] = 0.f;
#pragma unroll
            for (int g = 0; g < 4; g++) {
                const int l = tgq * 4 + g;
                const float2 sv = acc2[(3 * qp + d) * 32 + l], cv = acc2[(3 * TP + 3 * qp + d) * 32 + l];
                kahan_add(v[d], cmp[d], qh ? sv.y : sv.x);
                kahan_add(v[d], cmp[d], -(qh ? cv.y : cv.x));
            }
        }
        A.ax[it + tq] += ((double)v[0] - (double)cmp[0]) * scale;
        A.ay[it + tq] += ((double)v[1] - (double)cmp[1]) * scale;
        A.az[it + tq] += ((double)v[2] - (double)cmp[2]) * scale;
    }
    __syncwarp();
    return true;
}

template <int MINB, int ILR, bool T6, bool BULK>
__global__ void __launch_bounds__(MU_TB, MINB) k_p2p_mutual(P2PArgs A, const int2 *ev, const int *nev,
                                                            const long long *rbase, float *rbuf, int *fail)
{
    // shared layouts avoid bank conflicts: a batch's source k (of 32) is
    // read by source group k % 4, so the four groups read adjacent float4s;
    // reactions [source][component][target group] with a 24-word source
    // stride; running sums [value][lane].  12 KB per warp.
    __shared__ __align__(16) float4 s_src[MU_WARPS][2 * 64];  // two stages
    __shared__ __align__(16) MuMeta s_meta[MU_WARPS][32];
    __shared__ __align__(16) float s_red[MU_WARPS][MU_BATCH * 24];
    __shared__ __align__(16) float s_acc[MU_WARPS][48 * 32];  // Kahan sums and compensations, up to 8 targets x 3, per lane (read as float2)
    __shared__ __align__(8) unsigned long long s_bar[MU_WARPS][2];  // the stages' mbarriers (BULK)
    const int lane = warp_lane(), wib = threadIdx.x >> 5;
    SplitConsts K = A.k;
    unsigned phase = 0;
    if constexpr (BULK) {
        if (lane == 0) {
            mbar_init(&s_bar[wib][0]);
            mbar_init(&s_bar[wib][1]);
            mbar_init_fence();
        }
        __syncwarp();
    }

    const int nleaf = p2p_targets(A);
    for (;;) {
        int t;
        if (lane == 0) t = atomicAdd(A.work_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= nleaf) break;
        const int nt = A.npart[t], it = A.ipart[t];
        if (nt == 0) continue;
        const BoxParams &B = A.boxes[A.boxid[t]];
        K.sig = B.sig;
        K.e2s = B.e2s;
        K.pias = B.pias;
        K.cs = B.cs;
        const int2 *evt = ev + A.p2p_off[t];
        const int ne = nev[t];
        // the narrow build gives leaves of 33-48 particles 6 targets per lane
        // (48 slots; 128^3 NFW at leaf 48: 39.4 against 47.4 ms with 64);
        // in the wide build the extra path cost 1.3 % at 256^3 leaf 64
        bool ok;
        if (nt > 48 || (nt > 32 && !T6))
            ok = mu_target<8, ILR, BULK>(A, evt, ne, rbase, rbuf, t, nt, it, K, B.Lhi, B.Llo, s_src[wib], s_meta[wib],
                                         s_red[wib], s_acc[wib], s_bar[wib], phase, fail, lane);
        else if (nt > 32)
            ok = mu_target<6, ILR, BULK>(A, evt, ne, rbase, rbuf, t, nt, it, K, B.Lhi, B.Llo, s_src[wib], s_meta[wib],
                                         s_red[wib], s_acc[wib], s_bar[wib], phase, fail, lane);
        else
            ok = mu_target<4, ILR, BULK>(A, evt, ne, rbase, rbuf, t, nt, it, K, B.Lhi, B.Llo, s_src[wib], s_meta[wib],
                                         s_red[wib], s_acc[wib], s_bar[wib], phase, fail, lane);
        if (!ok) return;
    }
}

// each leaf adds the reactions its owners left in its slots, in list order.
// The k-th received entry of leaf t (slot == -2, counted in list order)
// holds [3][r] floats at rbase[t] + 3 k r (r = nt rounded up to 32).  Which
// entries are received is read once per 32 as a warp mask, and eight
// slots' loads are in flight at a time.
// 3 resident blocks of 256 threads per SM (80 registers); launched as one wave
__global__ void __launch_bounds__(256, 3) k_mu_gather(P2PArgs A, const int *slot, const int *nrecv, const long long *rbase, const float *rbuf)
{
    const int lane = warp_lane();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int nleaf = p2p_targets(A);
    for (int t = gw; t < nleaf; t += nw) {
        const int nt = A.npart[t], it = A.ipart[t], nr = nrecv[t];
        if (nr == 0 || nt == 0) continue;
        const long long eoff = A.p2p_off[t];
        const int L = A.p2p_cnt[t];
        const double scale = A.boxes[A.boxid[t]].acc_scale;
        const int rl = mu_row(nt);
        const long long stride = 3LL * rl;
        if (rl == 64) {
            // 33-64 particles: lane takes particles 2 lane and 2 lane + 1, one
            // float2 per component row, so one sweep of the list serves the
            // whole leaf with twice the bytes in flight per load.  Rows are
            // padded to 64 floats (in bounds for every lane) and every
            // particle's sum runs over the same slots in the same order as
            // below.  rbase and the rows are multiples of 32 floats: float2
            // aligned.
            const float2 *base = reinterpret_cast<const float2 *>(rbuf + rbase[t]) + lane;
            const long long stride2 = stride / 2;
            float2 v0 = make_float2(0.f, 0.f), v1 = v0, v2 = v0, c0 = v0, c1 = v0, c2 = v0;
            int k = 0;
            for (int e0 = 0; e0 < L && k < nr; e0 += 32) {
                unsigned got = __ballot_sync(0xffffffffu, e0 + lane < L && slot[eoff + e0 + lane] == -2);
                while (got) {
                    float2 in[8][3];
                    int cntk = 0;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const bool use = got != 0;
                        if (use) got &= got - 1;
                        cntk += use;
                        const float2 *src = base + (long long)(k + q) * stride2;
                        const float2 z = make_float2(0.f, 0.f);
                        in[q][0] = use ? src[0] : z;
                        in[q][1] = use ? src[32] : z;
                        in[q][2] = use ? src[64] : z;
                    }
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        if (q < cntk) {
                            kahan_add(v0.x, c0.x, in[q][0].x);
                            kahan_add(v0.y, c0.y, in[q][0].y);
                            kahan_add(v1.x, c1.x, in[q][1].x);
                            kahan_add(v1.y, c1.y, in[q][1].y);
                            kahan_add(v2.x, c2.x, in[q][2].x);
                            kahan_add(v2.y, c2.y, in[q][2].y);
                        }
                    }
                    k += cntk;
                }
            }
            const int j = 2 * lane;
            if (j < nt) {
                A.ax[it + j] += ((double)v0.x - (double)c0.x) * scale;
                A.ay[it + j] += ((double)v1.x - (double)c1.x) * scale;
                A.az[it + j] += ((double)v2.x - (double)c2.x) * scale;
            }
            if (j + 1 < nt) {
                A.ax[it + j + 1] += ((double)v0.y - (double)c0.y) * scale;
                A.ay[it + j + 1] += ((double)v1.y - (double)c1.y) * scale;
                A.az[it + j + 1] += ((double)v2.y - (double)c2.y) * scale;
            }
            continue;
        }
        for (int j0 = 0; j0 < nt; j0 += 32) {
            const int j = j0 + lane;
            const float *base = rbuf + rbase[t] + j;
            float v0 = 0.f, v1 = 0.f, v2 = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
            int k = 0;  // received entries before this chunk
            for (int e0 = 0; e0 < L && k < nr; e0 += 32) {
                unsigned got = __ballot_sync(0xffffffffu, e0 + lane < L && slot[eoff + e0 + lane] == -2);
                while (got) {
                    // up to eight received slots: loads first, then the adds in order
                    float in[8][3];
                    int cntk = 0;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const bool use = got != 0;
                        if (use) got &= got - 1;
                        cntk += use;
                        const bool ld = use && j < nt;
                        const float *src = base + (long long)(k + q) * stride;
                        in[q][0] = ld ? src[0] : 0.f;
                        in[q][1] = ld ? src[rl] : 0.f;
                        in[q][2] = ld ? src[2 * rl] : 0.f;
                    }
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        if (q < cntk) {
                            kahan_add(v0, c0, in[q][0]);
                            kahan_add(v1, c1, in[q][1]);
                            kahan_add(v2, c2, in[q][2]);
                        }
                    }
                    k += cntk;
                }
            }
            if (j < nt) {
                A.ax[it + j] += ((double)v0 - (double)c0) * scale;
                A.ay[it + j] += ((double)v1 - (double)c1) * scale;
                A.az[it + j] += ((double)v2 - (double)c2) * scale;
            }
        }
    }
}

// ---------------------------------------------------------------------
// FP64 P2P with mutual pairs: the pairing of the FP32 kernel (each
// symmetric leaf pair, local or image, evaluated once by its owner) with
// the FP64 pass's pair force.  One warp per target leaf.  Lanes are 8
// target groups x 4 source groups (lane = 4 tg + sg): target q belongs to
// group q mod 8, a lane holds up to T = 8 of them (64 per chunk; larger
// leaves run in chunks of 64), and takes sources sg, sg + 4, ... of each
// entry, staged with the image shift in shared memory.  For an owned entry
// the reaction on a source is summed over the 8 target groups (butterfly,
// lane tg = 0's sum kept) and stored in the pair's slot (x, y, z rows of
// r = n rounded up to 4 doubles; a second chunk adds to it).  Target sums
// are combined over the 4 source groups at the end.  The pair factor is
// pair_f_fp64's, without the mass, which multiplies each target sum and
// each reaction slot once; sums accumulate by FMA.  k_mu_gather64 adds
// each leaf's received slots in list order.
// ---------------------------------------------------------------------
#define MU64_TB 256
#define MU64_WARPS (MU64_TB / 32)

template <int T>
__device__ __forceinline__ void mu64_chunk(const P2PArgs &A, const int2 *ev, int ne, const long long *rbase,
                                           double *rbuf, int t, int it, int q0, int nq, double *stage,
                                           const double *tab, int lane)
{
    const int tg = lane >> 2, sg = lane & 3;
    const BoxParams &B = A.boxes[A.boxid[t]];
    const double mass = B.mass, boxL = B.boxsize;
    const Pair64 pc = pair64_consts(B.eps, B.rs);
    double px[T], py[T], pz[T], ax[T], ay[T], az[T];
#pragma unroll
    for (int k = 0; k < T; k++) {
        const int q = 8 * k + tg;
        px[k] = py[k] = pz[k] = 0.0;
        if (q < nq) { px[k] = A.px[it + q0 + q]; py[k] = A.py[it + q0 + q]; pz[k] = A.pz[it + q0 + q]; }
        ax[k] = ay[k] = az[k] = 0.0;
    }
    for (int e = 0; e < ne; e++) {
        const int2 en = ev[e];
        const int s = PH_ENTRY_ID((uint32_t)en.x), img = PH_ENTRY_IMG((uint32_t)en.x);
        const int is = A.ipart[s], ns = A.npart[s];
        double h0 = 0.0, h1 = 0.0, h2 = 0.0;
        if (img) leaf_shift(img, boxL, h0, h1, h2);
        __syncwarp();
        for (int j = lane; j < ns; j += 32) {
            stage[3 * j] = A.px[is + j] + h0;
            stage[3 * j + 1] = A.py[is + j] + h1;
            stage[3 * j + 2] = A.pz[is + j] + h2;
        }
        __syncwarp();
        const bool self = img == 0 && s == t;
        const bool owned = en.y >= 0;
        const int row = mu_row_g(ns, MU64_ROW);
        double *out = owned ? rbuf + rbase[s] + (long long)en.y * 3 * row : nullptr;
        for (int j0 = 0; j0 < ns; j0 += 4) {
            const int j = j0 + sg;
            double rx = 0.0, ry = 0.0, rz = 0.0;
            if (j < ns) {
                const double sx = stage[3 * j], sy = stage[3 * j + 1], sz = stage[3 * j + 2];
#pragma unroll
                for (int k = 0; k < T; k++) {
                    const int q = 8 * k + tg;
                    if (q < nq && !(self && q0 + q == j)) {
                        const double dx = sx - px[k], dy = sy - py[k], dz = sz - pz[k];
                        const double f = pair_f_fp64(dx, dy, dz, pc, tab);
                        ax[k] = fma(dx, f, ax[k]); ay[k] = fma(dy, f, ay[k]); az[k] = fma(dz, f, az[k]);
                        rx = fma(-dx, f, rx); ry = fma(-dy, f, ry); rz = fma(-dz, f, rz);
                    }
                }
            }
            if (owned) {
#pragma unroll
                for (int o = 4; o < 32; o <<= 1) {
                    rx += __shfl_xor_sync(0xffffffffu, rx, o);
                    ry += __shfl_xor_sync(0xffffffffu, ry, o);
                    rz += __shfl_xor_sync(0xffffffffu, rz, o);
                }
                if (tg == 0 && j < ns) {
                    rx *= mass; ry *= mass; rz *= mass;
                    if (q0 == 0) { out[j] = rx; out[row + j] = ry; out[2 * row + j] = rz; }
                    else { out[j] += rx; out[row + j] += ry; out[2 * row + j] += rz; }
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < T; k++) {
#pragma unroll
        for (int o = 1; o < 4; o <<= 1) {
            ax[k] += __shfl_xor_sync(0xffffffffu, ax[k], o);
            ay[k] += __shfl_xor_sync(0xffffffffu, ay[k], o);
            az[k] += __shfl_xor_sync(0xffffffffu, az[k], o);
        }
        const int q = 8 * k + tg;
        if (sg == 0 && q < nq) {
            A.ax[it + q0 + q] += ax[k] * mass;
            A.ay[it + q0 + q] += ay[k] * mass;
            A.az[it + q0 + q] += az[k] * mass;
        }
    }
}

__global__ void __launch_bounds__(MU64_TB, 1) k_p2p_mutual64(P2PArgs A, const int2 *ev, const int *nev,
                                                            const long long *rbase, double *rbuf)
{
    __shared__ double s_stage[MU64_WARPS][3 * PH_MAX_LEAF];
    __shared__ double s_tab[SPLIT64_N];
    load_split64_scaled(s_tab);
    const int lane = warp_lane(), wib = threadIdx.x >> 5;
    const int nleaf = p2p_targets(A);
    for (;;) {
        int t;
        if (lane == 0) t = atomicAdd(A.work_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= nleaf) break;
        const int nt = A.npart[t], it = A.ipart[t];
        const int ne = nev[t];
        const int2 *evt = ev + A.p2p_off[t];
        for (int q0 = 0; q0 < nt; q0 += 64) {
            const int nq = min(64, nt - q0);
            if (nq > 32) mu64_chunk<8>(A, evt, ne, rbase, rbuf, t, it, q0, nq, s_stage[wib], s_tab, lane);
            else if (nq > 16) mu64_chunk<4>(A, evt, ne, rbase, rbuf, t, it, q0, nq, s_stage[wib], s_tab, lane);
            else mu64_chunk<2>(A, evt, ne, rbase, rbuf, t, it, q0, nq, s_stage[wib], s_tab, lane);
        }
    }
}

// each leaf adds the FP64 reactions its owners left in its slots, the
// received entries in list order (received entry k at rbase + 3 k r).
// With the reaction buffer too small (over) every entry ran one way and no
// slot holds anything.
__global__ void k_mu_gather64(P2PArgs A, const int *over, const int *nrecv, const long long *rbase,
                              const double *rbuf)
{
    const int lane = warp_lane();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int nleaf = *over ? 0 : p2p_targets(A);
    for (int t = gw; t < nleaf; t += nw) {
        const int nt = A.npart[t], it = A.ipart[t], nr = nrecv[t];
        if (nr == 0 || nt == 0) continue;
        const int rl = mu_row_g(nt, MU64_ROW);
        const double *base = rbuf + rbase[t];
        for (int j = lane; j < nt; j += 32) {
            double v0 = 0.0, v1 = 0.0, v2 = 0.0;
            for (int k = 0; k < nr; k++) {
                const double *src = base + (long long)k * 3 * rl + j;
                v0 += src[0];
                v1 += src[rl];
                v2 += src[2 * rl];
            }
            A.ax[it + j] += v0;
            A.ay[it + j] += v1;
            A.az[it + j] += v2;
        }
    }
}

// One leaf pair in FP64, the entry points of inc/kernels.h: forces on the
// nt targets at tpos (particle indices tfirst..) from the ns sources at spos
// (indices sfirst..), a source skipped where its index is the target's (a
// leaf with itself), summed per target in source order as
// src/fmm.c:823-855 sums a task.  exact: sqrt, division, erfc and exp as the
// reference writes them; otherwise 1/r from rsqrt and g from the piecewise
// polynomials (the FP64 pass's form).  out[3 q + d] = the target's sum.
__global__ void k_leaf_pair_fp64(const double *tpos, int nt, int tfirst, const double *spos, int ns, int sfirst,
                                 double eps, double mass, double rs, int exact, double *out)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nt) return;
    const double px = tpos[3 * q], py = tpos[3 * q + 1], pz = tpos[3 * q + 2];
    const double coeff = 2.0 / sqrt(M_PI), soft3 = mass / (eps * eps * eps), hrs = 0.5 / rs;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int j = 0; j < ns; j++) {
        if (sfirst + j == tfirst + q) continue;
        const double dx = spos[3 * j] - px, dy = spos[3 * j + 1] - py, dz = spos[3 * j + 2] - pz;
        double ir3;
        if (exact) {
            const double dr = sqrt(dx * dx + dy * dy + dz * dz);
            ir3 = (dr < eps) ? soft3 : mass / (dr * dr * dr);
            const double drs = 0.5 * dr / rs;
            ir3 *= (erfc(drs) + coeff * drs * exp(-drs * drs));
        } else {
            ir3 = pair_ir3_fp64(dx, dy, dz, eps, soft3, mass, rs, hrs, coeff, &g_split64[0][0]);
        }
        ax += dx * ir3;
        ay += dy * ir3;
        az += dz * ir3;
    }
    out[3 * q] = ax;
    out[3 * q + 1] = ay;
    out[3 * q + 2] = az;
}

// the FP64 split factor g(u) at n points: the piecewise polynomials of the
// FP64 kernels, or (exact) erfc and exp as src/fmm.c:846-848 writes them
__global__ void k_split_factor_fp64(const double *u, int n, int exact, double *g)
{
    const double coeff = 2.0 / sqrt(M_PI);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = u[i];
        g[i] = exact ? erfc(x) + coeff * x * exp(-x * x) : split_g_fp64(x, &g_split64[0][0], coeff);
    }
}

}  // namespace

// coordinate scale of the packed kernel, rounded to FP32 first so that the
// constants below match the scaling the kernel applies
double split_sig(const PassParams &p)
{
    return (double)(float)(0.5 / p.rs * sqrt(1.4426950408889634));
}

SplitConsts make_split_consts(const PassParams &p)
{
    SplitConsts k;
    double ia = 0.5 / p.rs;
    k.eps2 = (float)(p.eps * p.eps);
    k.kq = (float)(-ia * ia * 1.4426950408889634);  // exp(-u^2) = 2^(-u^2 log2 e)
    k.pia = (float)(SPLIT_P * ia);
    for (int i = 0; i < SPLIT_NA; i++) k.a[i] = (float)(SPLIT_A[i] * p.mass);
    for (int i = SPLIT_NA; i < 8; i++) k.a[i] = 0.f;
    k.clin = (float)(p.mass * 2.0 / sqrt(M_PI) * ia);
    // packed kernel: scaled coordinates, mass applied per target
    const double sig = split_sig(p);
    k.sig = (float)sig;
    k.e2s = (float)(p.eps * p.eps * sig * sig);
    k.pias = (float)(SPLIT_P * ia / sig);
    k.cs = (float)(2.0 / sqrt(M_PI) * ia / sig);
    for (int i = 0; i < SPLIT_NA; i++) k.as[i] = (float)SPLIT_A[i];
    for (int i = SPLIT_NA; i < 8; i++) k.as[i] = 0.f;
    return k;
}

int launch_leaf_offsets(const BuildBufs &b, const TreeBufs &t, float4 *pos4, cudaStream_t st)
{
    int blocks = device_sm_count() * 8;
    ph::note_launch(), k_leaf_offsets<<<blocks, 256, 0, st>>>(b.x, b.y, b.z, t.ipart, t.npart, t.cx, t.cy, t.cz, b.cnt,
                                                              pos4);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

template <int MINB, int ILR, bool T6, bool BULK>
static int launch_mutual_one(const P2PArgs &a, const MutualBufs &m, int sms, cudaStream_t st)
{
    ph::note_launch(), k_p2p_mutual<MINB, ILR, T6, BULK><<<sms * MINB, MU_TB, 0, st>>>(a, m.ev, m.nev, m.rbase, m.buf,
                                                                                      m.over);
    return 0;
}

template <bool BULK>
static int launch_mutual_build(const P2PArgs &a, const MutualBufs &m, int shape, int sms, cudaStream_t st)
{
    switch (shape) {
    case 1: return launch_mutual_one<3, 2, false, BULK>(a, m, sms, st);
    case 2: return launch_mutual_one<4, 1, true, BULK>(a, m, sms, st);
    case 3: return launch_mutual_one<3, 1, false, BULK>(a, m, sms, st);
    default: return launch_mutual_one<4, 2, true, BULK>(a, m, sms, st);
    }
}

int launch_p2p_mutual(const P2PArgs &a, const MutualBufs &m, int fp64, cudaStream_t st)
{
    PH_CUDA_CHECK(cudaMemsetAsync(a.work_counter, 0, sizeof(int), st));
    const int sms = device_sm_count();
    ph::note_launch(), k_mu_sort<<<sms * 4, 256, 0, st>>>(a.tree_cnt, a.walk_flags, m.pool, a.p2p_off, a.p2p_cnt,
                                                           m.sorted);
    ph::note_launch(), k_mu_pair<<<sms * 8, 256, 0, st>>>(a.tree_cnt, a.walk_flags, m.pool, a.p2p_off, a.p2p_cnt,
                                                           a.npart, m.sorted, m.slot, m.pq, m.nrecv, m.size,
                                                           fp64 ? MU64_ROW : 32);
    scan_exclusive_i64(m.size, m.rbase, a.tree_cnt + BC_LEAVES, m.cap_leaves, m.total, m.scan_scratch, st);
    ph::note_launch(), k_mu_slots<<<sms * 8, 256, 0, st>>>(a.tree_cnt, a.walk_flags, m.pool, a.p2p_off, a.p2p_cnt,
                                                            m.total, m.buf_cap, m.pq, m.slot, m.ev, m.nev, m.over);
    if (fp64) {
        double *rbuf = reinterpret_cast<double *>(m.buf);
        // one block of 8 warps per SM (194 registers): the FP64 pipe, at 1/64
        // of the FP32 rate, is saturated by far fewer warps than that
        ph::note_launch(), k_p2p_mutual64<<<sms, MU64_TB, 0, st>>>(a, m.ev, m.nev, m.rbase, rbuf);
        ph::note_launch(), k_mu_gather64<<<sms * 4, 256, 0, st>>>(a, m.over, m.nrecv, m.rbase, rbuf);
        PH_CUDA_CHECK(cudaGetLastError());
        return 0;
    }
    // the build: shape 0 is build 2 (four blocks per SM, one chain, the
    // 6-target path: 256^3 leaf 64 P2P phase 60.3 ms against 61.6 for build
    // 1); 1-4 name a build for the autotuner (PHOTONS_F_P2P_SHAPE)
    int shape = a.shape;
    if (shape == 0) shape = 2;
    const int rc = a.bulk ? launch_mutual_build<true>(a, m, shape, sms, st)
                          : launch_mutual_build<false>(a, m, shape, sms, st);
    if (rc) return rc;
    ph::note_launch(), k_mu_gather<<<sms * 3, 256, 0, st>>>(a, m.slot, m.nrecv, m.rbase, m.buf);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_leaf_pair_fp64(const double *tpos, int nt, int tfirst, const double *spos, int ns, int sfirst, double eps,
                          double mass, double rs, int exact, double *out, cudaStream_t st)
{
    if (nt <= 0) return 0;
    ph::note_launch(), k_leaf_pair_fp64<<<(nt + 63) / 64, 64, 0, st>>>(tpos, nt, tfirst, spos, ns, sfirst, eps, mass, rs,
                                                                      exact, out);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_p2p(const P2PArgs &a, int fp64, cudaStream_t st)
{
    if (!fp64 && a.variant == 1 && a.nbox != 1)
        return ph_set_error(8, "the scalar FP32 P2P kernel runs one box per pass");
    PH_CUDA_CHECK(cudaMemsetAsync(a.work_counter, 0, sizeof(int), st));
    int blocks = device_sm_count() * (fp64 ? 4 : 4);
    if (fp64) ph::note_launch(), k_p2p_fp64<<<blocks, P2P_TB, 0, st>>>(a);
    else if (a.variant == 1) ph::note_launch(), k_p2p_split<<<blocks, P2P_TB, 0, st>>>(a);
    else ph::note_launch(), k_p2p_split_packed<<<blocks, P2P_TB, 0, st>>>(a);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_split_factor_fp64(const double *u, int n, int exact, double *g, cudaStream_t st)
{
    if (n <= 0) return 0;
    ph::note_launch(), k_split_factor_fp64<<<(n + 255) / 256, 256, 0, st>>>(u, n, exact, g);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace ph
