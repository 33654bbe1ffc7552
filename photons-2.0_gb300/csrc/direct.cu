// Measurement helpers that run on the GPU:
//  * photons_direct_sum: FP64 direct sum of the untruncated short-range
//    kernel m g(r/2rs) dx / max(r,eps)^3 over all sources within rmax
//    (minimum image), for a subset of targets.  This is the error
//    reference for the force pass (the pass truncates by tree cells, this
//    does not).  Sources are binned into cells of side >= rmax on the host.
//  * photons_fp32_fma_peak: FFMA throughput probe, the denominator of the
//    P2P roofline fraction; photons_fp64_fma_peak: the DFMA one, for the
//    FP64 drop-in pass.
#include <cmath>
#include <cstring>
#include <vector>

#include "api_internal.cuh"

namespace {

__global__ void k_direct(const double *__restrict__ sx, const double *__restrict__ sy, const double *__restrict__ sz,
                         const int *__restrict__ cell_start, int ncell, double cellw, const double *__restrict__ tx,
                         const double *__restrict__ ty, const double *__restrict__ tz, const int *__restrict__ tself,
                         int nt, double L, double rmax2, double eps, double mass, double rs, double *out)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const double coeff = 2.0 / sqrt(M_PI);
    const double soft3 = mass / (eps * eps * eps);
    for (int t = gw; t < nt; t += nw) {
        double px = tx[t], py = ty[t], pz = tz[t];
        int self = tself[t];
        int ci[3] = {(int)(px / cellw), (int)(py / cellw), (int)(pz / cellw)};
        for (int d = 0; d < 3; d++) ci[d] = min(max(ci[d], 0), ncell - 1);
        double ax = 0, ay = 0, az = 0;
        int span = ncell >= 3 ? 1 : 0;
        for (int ox = -span; ox <= span; ox++)
            for (int oy = -span; oy <= span; oy++)
                for (int oz = -span; oz <= span; oz++) {
                    int cx = (ci[0] + ox + ncell) % ncell, cy = (ci[1] + oy + ncell) % ncell,
                        cz = (ci[2] + oz + ncell) % ncell;
                    int c = ncell >= 3 ? (cx * ncell + cy) * ncell + cz : 0;
                    int b = ncell >= 3 ? cell_start[c] : 0;
                    int e = ncell >= 3 ? cell_start[c + 1] : cell_start[ncell * ncell * ncell];
                    for (int j = b + lane; j < e; j += 32) {
                        if (j == self) continue;
                        double dx = sx[j] - px, dy = sy[j] - py, dz = sz[j] - pz;
                        if (dx > 0.5 * L) dx -= L; else if (dx < -0.5 * L) dx += L;
                        if (dy > 0.5 * L) dy -= L; else if (dy < -0.5 * L) dy += L;
                        if (dz > 0.5 * L) dz -= L; else if (dz < -0.5 * L) dz += L;
                        double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 >= rmax2) continue;
                        double dr = sqrt(r2);
                        double ir3 = dr < eps ? soft3 : mass / (dr * dr * dr);
                        double u = 0.5 * dr / rs;
                        ir3 *= erfc(u) + coeff * u * exp(-u * u);
                        ax += dx * ir3;
                        ay += dy * ir3;
                        az += dz * ir3;
                    }
                }
        ax = warp_sum_d(ax);
        ay = warp_sum_d(ay);
        az = warp_sum_d(az);
        if (lane == 0) {
            out[3 * t] = ax;
            out[3 * t + 1] = ay;
            out[3 * t + 2] = az;
        }
    }
}

__global__ void k_fma_probe(float *out, int iters, float seed)
{
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f, a4 = a0 + 4.f, a5 = a0 + 5.f,
          a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 1234.5f) out[0] = s;  // keeps the chains live
}

__global__ void k_dfma_probe(double *out, int iters, double seed)
{
    double a0 = seed + threadIdx.x, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0, a4 = a0 + 4.0, a5 = a0 + 5.0,
           a6 = a0 + 6.0, a7 = a0 + 7.0;
    const double m = 0.999999999, c = 1e-12;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
            a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
        }
    }
    double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 1234.5) out[0] = s;  // keeps the chains live
}

__global__ void k_fma2_probe(float *out, int iters, float seed)
{
    float2 a0 = make_float2(seed + threadIdx.x, seed - threadIdx.x), a1 = make_float2(a0.x + 1.f, a0.y + 1.f),
           a2 = make_float2(a0.x + 2.f, a0.y + 2.f), a3 = make_float2(a0.x + 3.f, a0.y + 3.f);
    float2 a4 = make_float2(a0.x + 4.f, a0.y + 4.f), a5 = make_float2(a0.x + 5.f, a0.y + 5.f),
           a6 = make_float2(a0.x + 6.f, a0.y + 6.f), a7 = make_float2(a0.x + 7.f, a0.y + 7.f);
    const float2 m = make_float2(0.999999f, 0.999999f), c = make_float2(1e-7f, 1e-7f);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            a0 = __ffma2_rn(a0, m, c); a1 = __ffma2_rn(a1, m, c); a2 = __ffma2_rn(a2, m, c); a3 = __ffma2_rn(a3, m, c);
            a4 = __ffma2_rn(a4, m, c); a5 = __ffma2_rn(a5, m, c); a6 = __ffma2_rn(a6, m, c); a7 = __ffma2_rn(a7, m, c);
        }
    }
    float s = a0.x + a1.x + a2.x + a3.x + a4.x + a5.x + a6.x + a7.x + a0.y + a1.y + a2.y + a3.y + a4.y + a5.y +
              a6.y + a7.y;
    if (s == 1234.5f) out[0] = s;
}

}  // namespace

extern "C" int photons_direct_sum(const photons_params *p, int n, const double *pos, int nt, const int *targets,
                                  double rmax, double *acc)
{
    photons_gpu_clear_error();
    if (!p || n < 1 || nt < 0 || !pos || (nt > 0 && (!targets || !acc)) || !(rmax > 0))
        return ph_set_error(PH_ERR_ARG, "bad direct-sum arguments");
    if (nt == 0) return 0;
    const double L = p->boxsize;
    int ncell = (int)(L / rmax);
    if (ncell > 512) ncell = 512;
    if (ncell < 3) ncell = 1;
    const double cw = L / ncell;
    const size_t nc3 = (size_t)ncell * ncell * ncell;
    std::vector<int> cnt(nc3 + 1, 0), cellof(n);
    for (int j = 0; j < n; j++) {
        int c[3];
        for (int d = 0; d < 3; d++) {
            c[d] = (int)(pos[3 * (size_t)j + d] / cw);
            if (c[d] < 0) c[d] = 0;
            if (c[d] >= ncell) c[d] = ncell - 1;
        }
        cellof[j] = (int)(((size_t)c[0] * ncell + c[1]) * ncell + c[2]);
        cnt[cellof[j] + 1]++;
    }
    for (size_t c = 0; c < nc3; c++) cnt[c + 1] += cnt[c];
    std::vector<int> fill(cnt.begin(), cnt.end() - 1), slot(n);
    std::vector<double> sx(n), sy(n), sz(n);
    for (int j = 0; j < n; j++) {
        int s = fill[cellof[j]]++;
        slot[j] = s;
        sx[s] = pos[3 * (size_t)j];
        sy[s] = pos[3 * (size_t)j + 1];
        sz[s] = pos[3 * (size_t)j + 2];
    }
    std::vector<double> tx(nt), ty(nt), tz(nt);
    std::vector<int> ts(nt);
    for (int t = 0; t < nt; t++) {
        int j = targets[t];
        if (j < 0 || j >= n) return ph_set_error(PH_ERR_ARG, "target index out of range");
        tx[t] = pos[3 * (size_t)j];
        ty[t] = pos[3 * (size_t)j + 1];
        tz[t] = pos[3 * (size_t)j + 2];
        ts[t] = slot[j];
    }
    double *d_sx = nullptr, *d_sy = nullptr, *d_sz = nullptr, *d_tx = nullptr, *d_ty = nullptr, *d_tz = nullptr,
           *d_out = nullptr;
    int *d_cell = nullptr, *d_ts = nullptr;
    int rc = 0;
    auto al = [&](void **ptr, size_t bytes) {
        if (rc) return;
        if (cudaMalloc(ptr, bytes) != cudaSuccess) {
            cudaGetLastError();
            rc = ph_set_error(PH_ERR_NOMEM, "direct-sum allocation failed");
        }
    };
    al((void **)&d_sx, sizeof(double) * n); al((void **)&d_sy, sizeof(double) * n); al((void **)&d_sz, sizeof(double) * n);
    al((void **)&d_tx, sizeof(double) * nt); al((void **)&d_ty, sizeof(double) * nt); al((void **)&d_tz, sizeof(double) * nt);
    al((void **)&d_out, sizeof(double) * 3 * nt); al((void **)&d_cell, sizeof(int) * (nc3 + 1));
    al((void **)&d_ts, sizeof(int) * nt);
    if (!rc) {
        cudaMemcpy(d_sx, sx.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(d_sy, sy.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(d_sz, sz.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(d_tx, tx.data(), sizeof(double) * nt, cudaMemcpyHostToDevice);
        cudaMemcpy(d_ty, ty.data(), sizeof(double) * nt, cudaMemcpyHostToDevice);
        cudaMemcpy(d_tz, tz.data(), sizeof(double) * nt, cudaMemcpyHostToDevice);
        cudaMemcpy(d_ts, ts.data(), sizeof(int) * nt, cudaMemcpyHostToDevice);
        cudaMemcpy(d_cell, cnt.data(), sizeof(int) * (nc3 + 1), cudaMemcpyHostToDevice);
        int blocks = ph::device_sm_count() * 8;
        ph::note_launch(), k_direct<<<blocks, 256>>>(d_sx, d_sy, d_sz, d_cell, ncell, cw, d_tx, d_ty, d_tz, d_ts, nt, L, rmax * rmax,
                                  p->eps, p->mass, p->rs, d_out);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(acc, d_out, sizeof(double) * 3 * nt, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = ph_set_cuda_error(e, "direct sum", __FILE__, __LINE__);
    }
    cudaFree(d_sx); cudaFree(d_sy); cudaFree(d_sz); cudaFree(d_tx); cudaFree(d_ty); cudaFree(d_tz);
    cudaFree(d_out); cudaFree(d_cell); cudaFree(d_ts);
    return rc;
}

static double fma_probe(int iters, bool packed)
{
    photons_gpu_clear_error();
    if (iters < 1) iters = 4096;
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float)) != cudaSuccess) { cudaGetLastError(); return -1.0; }
    int blocks = ph::device_sm_count() * 8, threads = 256;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    if (packed) ph::note_launch(), k_fma2_probe<<<blocks, threads>>>(d, iters / 8 + 1, 1.0f);  // warm-up
    else ph::note_launch(), k_fma_probe<<<blocks, threads>>>(d, iters / 8 + 1, 1.0f);
    cudaEventRecord(a);
    if (packed) ph::note_launch(), k_fma2_probe<<<blocks, threads>>>(d, iters, 1.0f);
    else ph::note_launch(), k_fma_probe<<<blocks, threads>>>(d, iters, 1.0f);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    double flops = (packed ? 2.0 : 1.0) * 2.0 * 8.0 * 16.0 * (double)iters * blocks * threads;
    return flops / (ms * 1e-3) / 1e12;
}

extern "C" double photons_fp32_fma_peak(int iters)
{
    photons_gpu_clear_error();
    if (iters < 1) iters = 4096;
    return fma_probe(iters, false);
}

// TFLOP/s of DFMA chains (2 flops each) over the whole device
extern "C" double photons_fp64_fma_peak(int iters)
{
    photons_gpu_clear_error();
    if (iters < 1) iters = 256;
    double *d = nullptr;
    if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) { cudaGetLastError(); return -1.0; }
    const int blocks = ph::device_sm_count() * 8, threads = 256;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    ph::note_launch(), k_dfma_probe<<<blocks, threads>>>(d, iters / 8 + 1, 1.0);  // warm-up
    cudaEventRecord(a);
    ph::note_launch(), k_dfma_probe<<<blocks, threads>>>(d, iters, 1.0);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    const double flops = 2.0 * 8.0 * 16.0 * (double)iters * blocks * threads;
    return flops / (ms * 1e-3) / 1e12;
}

extern "C" double photons_fp32x2_fma_peak(int iters)
{
    photons_gpu_clear_error();
    if (iters < 1) iters = 4096;
    return fma_probe(iters, true);
}

// the FP64 pair factor's split term erfc(u) + (2/sqrt(pi)) u exp(-u^2) at n
// host points: the piecewise polynomials of the FP64 kernels, or (exact)
// erfc and exp as src/fmm.c:846-848 writes them
extern "C" int photons_split_factor_fp64(const double *u, int n, int exact, double *g)
{
    photons_gpu_clear_error();
    if (n < 0 || (n > 0 && (!u || !g))) return ph_set_error(PH_ERR_ARG, "bad split-factor arguments");
    if (n == 0) return 0;
    double *d = nullptr;
    PH_CUDA_CHECK(cudaMalloc(&d, sizeof(double) * 2 * (size_t)n));
    int rc = 0;
    cudaError_t e = cudaMemcpy(d, u, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        rc = ph::launch_split_factor_fp64(d, n, exact, d + n, 0);
        if (!rc) e = cudaMemcpy(g, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    }
    if (!rc && e != cudaSuccess) rc = ph_set_cuda_error(e, "split factor", __FILE__, __LINE__);
    cudaFree(d);
    return rc;
}
