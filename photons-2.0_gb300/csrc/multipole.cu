// Cartesian multipole operators of order 3 (octupole, 20 components), the
// expansions of src/operator.c written in multi-index form:
//   P2M  M_a   = sum_p m (-(x_p - c))^a / a!                 (operator.c:13-93)
//   M2M  M'_a += sum_{b<=a} M_b d^(a-b)/(a-b)!, d = c' - c    (operator.c:96-194)
//   M2L  L_b  += sum_{|a|<=3-|b|} M_a D_(a+b)(d), d = c_t - c_s (operator.c:255-392)
//   L2L  L'_b += sum_g L_(b+g) d^g/g!, d = c' - c              (operator.c:395-528)
//   L2P  a_i  += sum_{|g|<=2} L_(e_i+g) d^g/g!                 (operator.c:197-251)
// D is the derivative tensor of the short-range Green's function
// erfc(r/2rs)/r (the LONGSHORT branch), built from its radial factors
// f_k = ((1/r) d/dr)^k phi:  D_g = f_|g| x^g + f_(|g|-1) sum_i C(g_i,2) x^(g-2e_i).
// Component order is the reference's (inc/operator.h:24-60).  All in FP64.
#include <cmath>

#include "fmm_context.cuh"
#include "multipole.cuh"
#include "split_kernel_coeffs.h"

#define MP_TB 128

namespace ph {
namespace {

struct MITab {
    int e[PH_NMULTI][3];
    int ord[PH_NMULTI];
    double invf[PH_NMULTI];
    int idx[4][4][4];
};

constexpr MITab make_mitab()
{
    MITab t{};
    int i = 0;
    for (int k = 0; k <= 3; k++)
        for (int a = k; a >= 0; a--)
            for (int b = k - a; b >= 0; b--) {
                int c = k - a - b;
                t.e[i][0] = a; t.e[i][1] = b; t.e[i][2] = c;
                t.ord[i] = k;
                double f = 1.0;
                for (int q = 2; q <= a; q++) f *= q;
                for (int q = 2; q <= b; q++) f *= q;
                for (int q = 2; q <= c; q++) f *= q;
                t.invf[i] = 1.0 / f;
                t.idx[a][b][c] = i;
                i++;
            }
    return t;
}

constexpr __device__ MITab h_mi = make_mitab();

__device__ __forceinline__ void scaled_monomials(double dx, double dy, double dz, double *out)
{
    double px[4] = {1.0, dx, dx * dx, dx * dx * dx};
    double py[4] = {1.0, dy, dy * dy, dy * dy * dy};
    double pz[4] = {1.0, dz, dz * dz, dz * dz * dz};
#pragma unroll
    for (int i = 0; i < PH_NMULTI; i++)
        out[i] = px[h_mi.e[i][0]] * py[h_mi.e[i][1]] * pz[h_mi.e[i][2]] * h_mi.invf[i];
}

// ---------------- P2M ----------------
__global__ void k_p2m(const double *px, const double *py, const double *pz, const int *ipart, const int *npart,
                      const double *cx, const double *cy, const double *cz, const int *tree_cnt, const int *boxid,
                      const BoxParams *boxes, double *M, const int *gate)
{
    if (gate && !*gate) return;
    const int nleaf = tree_cnt[BC_LEAVES];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nleaf; l += gridDim.x * blockDim.x) {
        double acc[PH_NMULTI];
#pragma unroll
        for (int i = 0; i < PH_NMULTI; i++) acc[i] = 0.0;
        double c0 = cx[l], c1 = cy[l], c2 = cz[l];
        int ip = ipart[l], np = npart[l];
        const double mass = boxes[boxid[l]].mass;
        for (int p = ip; p < ip + np; p++) {
            double mono[PH_NMULTI];
            scaled_monomials(-(px[p] - c0), -(py[p] - c1), -(pz[p] - c2), mono);
#pragma unroll
            for (int i = 0; i < PH_NMULTI; i++) acc[i] += mass * mono[i];
        }
#pragma unroll
        for (int i = 0; i < PH_NMULTI; i++) M[(size_t)l * PH_NMULTI + i] = acc[i];
    }
}

// ---------------- M2M (one depth, parents gather their two children) ----------------
__device__ __forceinline__ void m2m_add(double dx, double dy, double dz, const double *Mc, double *out)
{
    double mono[PH_NMULTI];
    scaled_monomials(dx, dy, dz, mono);
#pragma unroll
    for (int a = 0; a < PH_NMULTI; a++) {
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < PH_NMULTI; b++) {
            const int g0 = h_mi.e[a][0] - h_mi.e[b][0], g1 = h_mi.e[a][1] - h_mi.e[b][1],
                      g2 = h_mi.e[a][2] - h_mi.e[b][2];
            if (g0 < 0 || g1 < 0 || g2 < 0) continue;
            s += Mc[b] * mono[h_mi.idx[g0][g1][g2]];
        }
        out[a] += s;
    }
}

__global__ void k_m2m_depth(const int *list, const int *depth_off, int d, const int *tree_cnt, const int *son0,
                            const int *son1, const double *cx, const double *cy, const double *cz, double *M,
                            const int *gate)
{
    if (gate && !*gate) return;
    const int begin = depth_off[d], end = depth_off[d + 1], nleaf = tree_cnt[BC_LEAVES];
    for (int i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
        int u = list[i];
        if (u < nleaf) continue;
        double out[PH_NMULTI];
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) out[a] = 0.0;
        double c0 = cx[u], c1 = cy[u], c2 = cz[u];
        int ch[2] = {son0[u], son1[u]};
        for (int k = 0; k < 2; k++) {
            int c = ch[k];
            double Mc[PH_NMULTI];
#pragma unroll
            for (int a = 0; a < PH_NMULTI; a++) Mc[a] = M[(size_t)c * PH_NMULTI + a];
            m2m_add(c0 - cx[c], c1 - cy[c], c2 - cz[c], Mc, out);
        }
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) M[(size_t)u * PH_NMULTI + a] = out[a];
    }
}

// ---------------- M2L ----------------
// radial factors of erfc(r/2rs)/r; with a = 1/(2rs), E = exp(-a^2 r^2), c = 2/sqrt(pi):
//   f0 = erfc/r, f1 = -erfc/r^3 - c a E/r^2,
//   f2 = 3 erfc/r^5 + c E (3a/r^4 + 2a^3/r^2),
//   f3 = -15 erfc/r^7 - c E (15a/r^6 + 10a^3/r^4 + 4a^5/r^2)
__device__ __forceinline__ void m2l_add(double dx, double dy, double dz, const double *Ms, double rs, double *L)
{
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    double a = 0.5 / rs, a2 = a * a;
    double u = a * r;
    double ce = 1.1283791670955126 * exp(-u * u);
    double er = erfc(u);
    double ir = 1.0 / r, ir2 = ir * ir;
    double f[4];
    f[0] = er * ir;
    f[1] = -er * ir * ir2 - ce * a * ir2;
    f[2] = 3.0 * er * ir * ir2 * ir2 + ce * (3.0 * a * ir2 * ir2 + 2.0 * a * a2 * ir2);
    f[3] = -15.0 * er * ir * ir2 * ir2 * ir2 - ce * (15.0 * a * ir2 * ir2 * ir2 + 10.0 * a * a2 * ir2 * ir2 +
                                                    4.0 * a * a2 * a2 * ir2);
    double x[3] = {dx, dy, dz};
    double pw[3][4];
#pragma unroll
    for (int d = 0; d < 3; d++) { pw[d][0] = 1.0; pw[d][1] = x[d]; pw[d][2] = x[d] * x[d]; pw[d][3] = x[d] * x[d] * x[d]; }
    double D[PH_NMULTI];
#pragma unroll
    for (int g = 0; g < PH_NMULTI; g++) {
        const int e0 = h_mi.e[g][0], e1 = h_mi.e[g][1], e2 = h_mi.e[g][2], k = h_mi.ord[g];
        double v = f[k] * pw[0][e0] * pw[1][e1] * pw[2][e2];
        if (k >= 2) {
            if (e0 >= 2) v += f[k - 1] * (double)(e0 * (e0 - 1) / 2) * pw[0][e0 - 2] * pw[1][e1] * pw[2][e2];
            if (e1 >= 2) v += f[k - 1] * (double)(e1 * (e1 - 1) / 2) * pw[0][e0] * pw[1][e1 - 2] * pw[2][e2];
            if (e2 >= 2) v += f[k - 1] * (double)(e2 * (e2 - 1) / 2) * pw[0][e0] * pw[1][e1] * pw[2][e2 - 2];
        }
        D[g] = v;
    }
#pragma unroll
    for (int b = 0; b < PH_NMULTI; b++) {
        double s = 0.0;
#pragma unroll
        for (int aa = 0; aa < PH_NMULTI; aa++) {
            if (h_mi.ord[aa] + h_mi.ord[b] > 3) continue;
            s += Ms[aa] * D[h_mi.idx[h_mi.e[aa][0] + h_mi.e[b][0]][h_mi.e[aa][1] + h_mi.e[b][1]]
                                     [h_mi.e[aa][2] + h_mi.e[b][2]]];
        }
        L[b] += s;
    }
}

__global__ void k_m2l(const int *tree_cnt, const unsigned long long *walk_flags, const uint32_t *pool,
                      const long long *off, const int *cnt, const double *cx, const double *cy, const double *cz,
                      const double *M, double *Lout, const int *boxid, const BoxParams *boxes)
{
    const int nunified = *walk_flags ? 0 : tree_cnt[BC_LEAVES] + tree_cnt[BC_NODES];
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nunified; u += gridDim.x * blockDim.x) {
        int n = cnt[u];
        if (n == 0) continue;
        double L[PH_NMULTI];
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) L[a] = Lout[(size_t)u * PH_NMULTI + a];
        double c0 = cx[u], c1 = cy[u], c2 = cz[u];
        const BoxParams &B = boxes[boxid[u]];
        const double rs = B.rs, boxsize = B.boxsize;
        long long o = off[u];
        for (int k = 0; k < n; k++) {
            uint32_t e = pool[o + k];
            int s = PH_ENTRY_ID(e), img = PH_ENTRY_IMG(e);
            double s0 = cx[s], s1 = cy[s], s2 = cz[s];
            if (img) {
                int mi, mj, mk;
                image_offsets(img, mi, mj, mk);
                s0 += mi * boxsize; s1 += mj * boxsize; s2 += mk * boxsize;
            }
            double Ms[PH_NMULTI];
#pragma unroll
            for (int a = 0; a < PH_NMULTI; a++) Ms[a] = M[(size_t)s * PH_NMULTI + a];
            m2l_add(c0 - s0, c1 - s1, c2 - s2, Ms, rs, L);
        }
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) Lout[(size_t)u * PH_NMULTI + a] = L[a];
    }
}

// ---------------- L2L (one depth: each member adds its parent's expansion) ----------------
__global__ void k_l2l_depth(const int *list, const int *depth_off, int d, const int *parent, const double *cx,
                            const double *cy, const double *cz, double *L, const int *gate)
{
    if (gate && !*gate) return;
    const int begin = depth_off[d], end = depth_off[d + 1];
    for (int i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
        int u = list[i];
        int p = parent[u];
        if (p < 0) continue;
        double mono[PH_NMULTI];
        scaled_monomials(cx[u] - cx[p], cy[u] - cy[p], cz[u] - cz[p], mono);
        double Lp[PH_NMULTI];
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) Lp[a] = L[(size_t)p * PH_NMULTI + a];
#pragma unroll
        for (int b = 0; b < PH_NMULTI; b++) {
            double s = 0.0;
#pragma unroll
            for (int g = 0; g < PH_NMULTI; g++) {
                if (h_mi.ord[b] + h_mi.ord[g] > 3) continue;
                s += Lp[h_mi.idx[h_mi.e[b][0] + h_mi.e[g][0]][h_mi.e[b][1] + h_mi.e[g][1]][h_mi.e[b][2] + h_mi.e[g][2]]] *
                     mono[g];
            }
            L[(size_t)u * PH_NMULTI + b] += s;
        }
    }
}

// ---------------- L2P ----------------
__global__ void k_l2p(const double *px, const double *py, const double *pz, const int *ipart, const int *npart,
                      const double *cx, const double *cy, const double *cz, const int *tree_cnt, const double *L,
                      double *ax, double *ay, double *az, const int *gate)
{
    if (gate && !*gate) return;
    const int nleaf = tree_cnt[BC_LEAVES];
    int lane = warp_lane();
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int l = gw; l < nleaf; l += nw) {
        int ip = ipart[l], np = npart[l];
        const double *Ll = L + (size_t)l * PH_NMULTI;
        for (int j = lane; j < np; j += 32) {
            int p = ip + j;
            double mono[PH_NMULTI];
            scaled_monomials(px[p] - cx[l], py[p] - cy[l], pz[p] - cz[l], mono);
            double F[3];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                double s = 0.0;
#pragma unroll
                for (int g = 0; g < PH_NMULTI; g++) {
                    if (h_mi.ord[g] > 2) continue;
                    int e0 = h_mi.e[g][0] + (i == 0), e1 = h_mi.e[g][1] + (i == 1), e2 = h_mi.e[g][2] + (i == 2);
                    s += Ll[h_mi.idx[e0][e1][e2]] * mono[g];
                }
                F[i] = s;
            }
            ax[p] += F[0];
            ay[p] += F[1];
            az[p] += F[2];
        }
    }
}

// ---------------- split-precision far field ----------------
// M2L in FP32: centre differences from the FP32 hi/lo centres (the side
// near the far face takes off the box length, so the subtraction is
// exact), multipoles rounded to FP32, radial factors from
// erfc(u) = exp(-u^2) t P(t) (the fit of fit_split_kernel.py), L
// accumulated per target in FP32 and added to the FP64 expansion.
__device__ __forceinline__ float rsqrt_f(float x) { float y; asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
__device__ __forceinline__ float rcp_f(float x) { float y; asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
__device__ __forceinline__ float ex2_f(float x) { float y; asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }

struct FarConsts {
    float a, pa, Lhi, Llo;
    float c[SPLIT_NA];
};

__device__ __forceinline__ float cdiff(float ht, float lt, float hs, float ls, int o, float Lhi, float Llo)
{
    // (c_t) - (c_s + shift)
    if (o > 0) { ht -= Lhi; lt -= Llo; }
    else if (o < 0) { hs -= Lhi; ls -= Llo; }
    return (ht - hs) + (lt - ls);
}

__device__ __forceinline__ void m2l_add_f32(float dx, float dy, float dz, const float *Ms, const FarConsts &F,
                                            float *L)
{
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float ir = rsqrt_f(r2);
    const float r = r2 * ir;
    const float a = F.a, a2 = a * a;
    const float u = a * r;
    const float E = ex2_f(-u * u * 1.44269504f);
    const float t = rcp_f(fmaf(F.pa, r, 1.0f));
    float P = F.c[SPLIT_NA - 1];
#pragma unroll
    for (int k = SPLIT_NA - 2; k >= 0; k--) P = fmaf(P, t, F.c[k]);
    const float er = E * t * P;
    const float ce = 1.12837917f * E;
    const float ir2 = ir * ir;
    float f[4];
    f[0] = er * ir;
    f[1] = -er * ir * ir2 - ce * a * ir2;
    f[2] = 3.0f * er * ir * ir2 * ir2 + ce * (3.0f * a * ir2 * ir2 + 2.0f * a * a2 * ir2);
    f[3] = -15.0f * er * ir * ir2 * ir2 * ir2 - ce * (15.0f * a * ir2 * ir2 * ir2 + 10.0f * a * a2 * ir2 * ir2 +
                                                      4.0f * a * a2 * a2 * ir2);
    const float x[3] = {dx, dy, dz};
    float pw[3][4];
#pragma unroll
    for (int d = 0; d < 3; d++) { pw[d][0] = 1.0f; pw[d][1] = x[d]; pw[d][2] = x[d] * x[d]; pw[d][3] = x[d] * x[d] * x[d]; }
    float D[PH_NMULTI];
#pragma unroll
    for (int g = 0; g < PH_NMULTI; g++) {
        const int e0 = h_mi.e[g][0], e1 = h_mi.e[g][1], e2 = h_mi.e[g][2], k = h_mi.ord[g];
        float v = f[k] * pw[0][e0] * pw[1][e1] * pw[2][e2];
        if (k >= 2) {
            if (e0 >= 2) v += f[k - 1] * (float)(e0 * (e0 - 1) / 2) * pw[0][e0 - 2] * pw[1][e1] * pw[2][e2];
            if (e1 >= 2) v += f[k - 1] * (float)(e1 * (e1 - 1) / 2) * pw[0][e0] * pw[1][e1 - 2] * pw[2][e2];
            if (e2 >= 2) v += f[k - 1] * (float)(e2 * (e2 - 1) / 2) * pw[0][e0] * pw[1][e1] * pw[2][e2 - 2];
        }
        D[g] = v;
    }
#pragma unroll
    for (int b = 0; b < PH_NMULTI; b++) {
        float acc = 0.0f;
#pragma unroll
        for (int aa = 0; aa < PH_NMULTI; aa++) {
            if (h_mi.ord[aa] + h_mi.ord[b] > 3) continue;
            acc = fmaf(Ms[aa], D[h_mi.idx[h_mi.e[aa][0] + h_mi.e[b][0]][h_mi.e[aa][1] + h_mi.e[b][1]]
                                       [h_mi.e[aa][2] + h_mi.e[b][2]]], acc);
        }
        L[b] += acc;
    }
}

__global__ void k_m_to_f32(const double *M, float *M32, const int *tree_cnt, const int *gate)
{
    if (gate && !*gate) return;
    const long long n = (long long)(tree_cnt[BC_LEAVES] + tree_cnt[BC_NODES]) * PH_NMULTI;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        M32[i] = (float)M[i];
}

// one warp per target (lists differ in length by orders of magnitude on
// clustered input; targets are handed out one at a time): lanes take the
// entries k = lane, lane + 32, ...; their partial expansions are combined
// by a fixed butterfly (lane 0's result) and added to the FP64 L
__global__ void k_m2l_f32(const int *tree_cnt, const unsigned long long *walk_flags, const uint32_t *pool,
                          const long long *off, const int *cnt, const float4 *chi, const float4 *clo, const float *M32,
                          double *Lout, const int *boxid, const BoxParams *boxes, FarConsts F, int *work,
                          const int *gate)
{
    if (gate && !*gate) return;  // no M2L task in this pass
    const int nunified = *walk_flags ? 0 : tree_cnt[BC_LEAVES] + tree_cnt[BC_NODES];
    const int lane = threadIdx.x & 31;
    for (;;) {
        int u = 0;
        if (lane == 0) u = atomicAdd(work, 1);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= nunified) break;
        const int n = cnt[u];
        if (n == 0) continue;
        float L[PH_NMULTI];
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) L[a] = 0.0f;
        const float4 th = chi[u], tl = clo[u];
        const BoxParams &B = boxes[boxid[u]];
        F.a = B.far_a;
        F.pa = B.far_pa;
        F.Lhi = B.Lhi;
        F.Llo = B.Llo;
        const long long o = off[u];
        for (int k = lane; k < n; k += 32) {
            const uint32_t e = pool[o + k];
            const int s = PH_ENTRY_ID(e), img = PH_ENTRY_IMG(e);
            int mi, mj, mk;
            image_offsets(img, mi, mj, mk);
            const float4 sh = chi[s], sl = clo[s];
            const float dx = cdiff(th.x, tl.x, sh.x, sl.x, mi, F.Lhi, F.Llo);
            const float dy = cdiff(th.y, tl.y, sh.y, sl.y, mj, F.Lhi, F.Llo);
            const float dz = cdiff(th.z, tl.z, sh.z, sl.z, mk, F.Lhi, F.Llo);
            float Ms[PH_NMULTI];
#pragma unroll
            for (int a = 0; a < PH_NMULTI; a++) Ms[a] = M32[(size_t)s * PH_NMULTI + a];
            m2l_add_f32(dx, dy, dz, Ms, F, L);
        }
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) {
            float v = L[a];
#pragma unroll
            for (int w = 16; w > 0; w >>= 1) v += __shfl_xor_sync(0xffffffffu, v, w);
            L[a] = v;
        }
        if (lane == 0) {
#pragma unroll
            for (int a = 0; a < PH_NMULTI; a++) Lout[(size_t)u * PH_NMULTI + a] += (double)L[a];
        }
    }
}

// L2P in FP32 on the leaf-centre offsets, added to the FP64 accelerations
__global__ void k_l2p_f32(const float4 *pos4, const int *ipart, const int *npart, const int *tree_cnt,
                          const double *L, double *ax, double *ay, double *az, const int *gate)
{
    if (gate && !*gate) return;
    const int nleaf = tree_cnt[BC_LEAVES];
    const int lane = warp_lane();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int l = gw; l < nleaf; l += nw) {
        const int ip = ipart[l], np = npart[l];
        float Ll[PH_NMULTI];
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) Ll[a] = (float)L[(size_t)l * PH_NMULTI + a];
        for (int j = lane; j < np; j += 32) {
            const float4 o = pos4[ip + j];
            const float px[4] = {1.f, o.x, o.x * o.x, 0.f}, py[4] = {1.f, o.y, o.y * o.y, 0.f},
                        pz[4] = {1.f, o.z, o.z * o.z, 0.f};
            float F[3];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                float acc = 0.0f;
#pragma unroll
                for (int g = 0; g < PH_NMULTI; g++) {
                    if (h_mi.ord[g] > 2) continue;
                    const int e0 = h_mi.e[g][0] + (i == 0), e1 = h_mi.e[g][1] + (i == 1), e2 = h_mi.e[g][2] + (i == 2);
                    const float mono = px[h_mi.e[g][0]] * py[h_mi.e[g][1]] * pz[h_mi.e[g][2]] * (float)h_mi.invf[g];
                    acc = fmaf(Ll[h_mi.idx[e0][e1][e2]], mono, acc);
                }
                F[i] = acc;
            }
            ax[ip + j] += F[0];
            ay[ip + j] += F[1];
            az[ip + j] += F[2];
        }
    }
}

// zero the local expansions of every unified id
__global__ void k_zero_L(double *L, const int *tree_cnt, const int *gate)
{
    if (gate && !*gate) return;
    const long long n = (long long)(tree_cnt[BC_LEAVES] + tree_cnt[BC_NODES]) * PH_NMULTI;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        L[i] = 0.0;
}

// far-field switches of a captured pass: gate[0] multipoles (M2L work or
// kept multipoles), gate[1] M2L / L2L / L2P (any M2L task)
__global__ void k_far_gate(const unsigned long long *walk_ctr, int keep_multipoles, int *gate)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const bool m2l = walk_ctr[WC_M2L_LOCAL] + walk_ctr[WC_M2L_IMAGE] > 0;
        gate[0] = m2l || keep_multipoles;
        gate[1] = m2l;
    }
}

inline int grid_cap() { return device_sm_count() * 16; }

inline int grid_for(long long n, int tpb)
{
    long long g = (n + tpb - 1) / tpb;
    if (g < 1) g = 1;
    return (int)(g < grid_cap() ? g : grid_cap());
}

}  // namespace

// All launches below read the tree sizes and depth slices on the device;
// depths past the tree's deepest have empty slices.
int run_m2l(const MultipoleArgs &a, cudaStream_t st)
{
    ph::note_launch(), k_m2l<<<grid_cap(), MP_TB, 0, st>>>(a.tree_cnt, a.walk_flags, a.m2l_pool, a.m2l_off, a.m2l_cnt,
                                                             a.cx, a.cy, a.cz, a.M, a.L, a.boxid, a.boxes);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

static void launch_l2l(const MultipoleArgs &a, cudaStream_t st)
{
    for (int d = 1; d < a.ndepth; d++)
        ph::note_launch(), k_l2l_depth<<<grid_cap(), MP_TB, 0, st>>>(a.depth_list, a.depth_off, d, a.parent, a.cx, a.cy,
                                                                       a.cz, a.L, a.gate_l);
}

int run_downward(const MultipoleArgs &a, cudaStream_t st)
{
    launch_l2l(a, st);
    ph::note_launch(), k_l2p<<<grid_cap(), 256, 0, st>>>(a.px, a.py, a.pz, a.ipart, a.npart, a.cx, a.cy, a.cz,
                                                           a.tree_cnt, a.L, a.ax, a.ay, a.az, a.gate_l);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int run_m2l_f32(const MultipoleArgs &a, float *M32, cudaStream_t st)
{
    ph::note_launch(), k_m_to_f32<<<grid_cap(), 256, 0, st>>>(a.M, M32, a.tree_cnt, a.gate_l);
    FarConsts F;  // per-box fields are filled per target from the box table
    F.a = F.pa = F.Lhi = F.Llo = 0.f;
    for (int i = 0; i < SPLIT_NA; i++) F.c[i] = (float)SPLIT_A[i];
    PH_CUDA_CHECK(cudaMemsetAsync(a.work, 0, sizeof(int), st));
    ph::note_launch(), k_m2l_f32<<<grid_cap(), MP_TB, 0, st>>>(a.tree_cnt, a.walk_flags, a.m2l_pool, a.m2l_off,
                                                                 a.m2l_cnt, a.chi, a.clo, M32, a.L, a.boxid, a.boxes, F,
                                                                 a.work, a.gate_l);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int run_downward_f32(const MultipoleArgs &a, cudaStream_t st)
{
    launch_l2l(a, st);
    ph::note_launch(), k_l2p_f32<<<grid_cap(), 256, 0, st>>>(a.pos4, a.ipart, a.npart, a.tree_cnt, a.L, a.ax, a.ay,
                                                               a.az, a.gate_l);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int run_p2m_m2m(const MultipoleArgs &a, cudaStream_t st)
{
    ph::note_launch(), k_p2m<<<grid_cap(), MP_TB, 0, st>>>(a.px, a.py, a.pz, a.ipart, a.npart, a.cx, a.cy, a.cz,
                                                             a.tree_cnt, a.boxid, a.boxes, a.M, a.gate_m);
    for (int d = a.ndepth - 1; d >= 0; d--)
        ph::note_launch(), k_m2m_depth<<<grid_cap(), MP_TB, 0, st>>>(a.depth_list, a.depth_off, d, a.tree_cnt, a.son0,
                                                                       a.son1, a.cx, a.cy, a.cz, a.M, a.gate_m);
    ph::note_launch(), k_zero_L<<<grid_cap(), 256, 0, st>>>(a.L, a.tree_cnt, a.gate_m);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_far_gate(const unsigned long long *walk_ctr, int keep_multipoles, int *gate, cudaStream_t st)
{
    ph::note_launch(), k_far_gate<<<1, 1, 0, st>>>(walk_ctr, keep_multipoles, gate);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// batched single operators (operator-level tests and the operator C-ABI)
namespace {
__global__ void k_op_m2l(int n, const double *d, const double *M, double *L, double rs)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double Ms[PH_NMULTI], Lo[PH_NMULTI];
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) { Ms[a] = M[(size_t)i * PH_NMULTI + a]; Lo[a] = L[(size_t)i * PH_NMULTI + a]; }
        m2l_add(d[3 * i], d[3 * i + 1], d[3 * i + 2], Ms, rs, Lo);
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) L[(size_t)i * PH_NMULTI + a] = Lo[a];
    }
}
__global__ void k_op_m2m(int n, const double *d, const double *M, double *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double Ms[PH_NMULTI], o[PH_NMULTI];
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) { Ms[a] = M[(size_t)i * PH_NMULTI + a]; o[a] = out[(size_t)i * PH_NMULTI + a]; }
        m2m_add(d[3 * i], d[3 * i + 1], d[3 * i + 2], Ms, o);
#pragma unroll
        for (int a = 0; a < PH_NMULTI; a++) out[(size_t)i * PH_NMULTI + a] = o[a];
    }
}
__global__ void k_op_l2l(int n, const double *d, const double *L, double *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double mono[PH_NMULTI];
        scaled_monomials(d[3 * i], d[3 * i + 1], d[3 * i + 2], mono);
        for (int b = 0; b < PH_NMULTI; b++) {
            double s = 0.0;
#pragma unroll
            for (int g = 0; g < PH_NMULTI; g++) {
                if (h_mi.ord[b] + h_mi.ord[g] > 3) continue;
                s += L[(size_t)i * PH_NMULTI + h_mi.idx[h_mi.e[b][0] + h_mi.e[g][0]][h_mi.e[b][1] + h_mi.e[g][1]]
                                                     [h_mi.e[b][2] + h_mi.e[g][2]]] * mono[g];
            }
            out[(size_t)i * PH_NMULTI + b] += s;
        }
    }
}
}  // namespace

int launch_op_batch(int op, int n, const double *d, const double *in, double *inout, double rs, cudaStream_t st)
{
    if (n <= 0) return 0;
    int g = grid_for(n, MP_TB);
    if (op == 0) ph::note_launch(), k_op_m2l<<<g, MP_TB, 0, st>>>(n, d, in, inout, rs);
    else if (op == 1) ph::note_launch(), k_op_m2m<<<g, MP_TB, 0, st>>>(n, d, in, inout);
    else ph::note_launch(), k_op_l2l<<<g, MP_TB, 0, st>>>(n, d, in, inout);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace ph
