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
// FP64 variant: the reference's arithmetic (sqrt, division, erfc, exp) on
// absolute FP64 positions, image positions formed as pos + shift like the
// exported bodies of src/remotes.c:83-89, self pair skipped by index.
#include <cmath>

#include "fmm_context.cuh"
#include "p2p.cuh"
#include "split_kernel_coeffs.h"

#define P2P_TB 256
#define P2P_WARPS (P2P_TB / 32)
#define STAGE32 256  // staged sources per warp, FP32 variant
#define STAGE64 128  // staged sources per warp, FP64 variant

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
__global__ void __launch_bounds__(P2P_TB) k_p2p_split(P2PArgs A)
{
    __shared__ float4 s_src[P2P_WARPS][STAGE32];
    __shared__ double s_red[P2P_WARPS][32][3];
    const int lane = warp_lane();
    const int wib = threadIdx.x >> 5;
    float4 *src = s_src[wib];
    const SplitConsts K = A.k;

    for (;;) {
        int t;
        if (lane == 0) t = atomicAdd(A.work_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= A.nleaf) break;
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
// FP64 kernel: the reference's arithmetic
// ---------------------------------------------------------------------
struct Src64 {
    double x, y, z;
    int idx;
    int pad;
};

__global__ void __launch_bounds__(P2P_TB) k_p2p_fp64(P2PArgs A)
{
    __shared__ Src64 s_src[P2P_WARPS][STAGE64];
    __shared__ double s_red[P2P_WARPS][32][3];
    const int lane = warp_lane();
    const int wib = threadIdx.x >> 5;
    Src64 *src = s_src[wib];
    const double eps = A.eps, mass = A.mass, rs = A.rs;
    const double coeff = 2.0 / sqrt(M_PI);
    const double soft3 = mass / (eps * eps * eps);

    for (;;) {
        int t;
        if (lane == 0) t = atomicAdd(A.work_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= A.nleaf) break;
        const int nt = A.npart[t], it = A.ipart[t];
        if (nt == 0) continue;
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
                    if (img) leaf_shift(img, A.boxsize, h0, h1, h2);
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
                        double dr = sqrt(dx * dx + dy * dy + dz * dz);
                        double ir3 = (dr < eps) ? soft3 : mass / (dr * dr * dr);
                        double drs = 0.5 * dr / rs;
                        ir3 *= (erfc(drs) + coeff * drs * exp(-drs * drs));
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
                               const int *npart, const double *cx, const double *cy, const double *cz, int nleaf,
                               float4 *pos4)
{
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int l = gw; l < nleaf; l += nw) {
        int ip = ipart[l], np = npart[l];
        double c0 = cx[l], c1 = cy[l], c2 = cz[l];
        for (int j = lane; j < np; j += 32)
            pos4[ip + j] = make_float4((float)(px[ip + j] - c0), (float)(py[ip + j] - c1), (float)(pz[ip + j] - c2), 0.f);
    }
}

}  // namespace

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
    return k;
}

int launch_leaf_offsets(const BuildBufs &b, const TreeBufs &t, int nleaf, float4 *pos4, cudaStream_t st)
{
    int blocks = device_sm_count() * 8;
    ph::note_launch(), k_leaf_offsets<<<blocks, 256, 0, st>>>(b.x, b.y, b.z, t.ipart, t.npart, t.cx, t.cy, t.cz, nleaf, pos4);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_p2p(const P2PArgs &a, int fp64, cudaStream_t st)
{
    PH_CUDA_CHECK(cudaMemsetAsync(a.work_counter, 0, sizeof(int), st));
    int blocks = device_sm_count() * (fp64 ? 4 : 4);
    if (fp64) ph::note_launch(), k_p2p_fp64<<<blocks, P2P_TB, 0, st>>>(a);
    else ph::note_launch(), k_p2p_split<<<blocks, P2P_TB, 0, st>>>(a);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace ph
