// PM long-range force on an N^3 periodic mesh, the other half of the
// reference's force split (src/partmesh.c:18-800 for one rank,
// src/conv.f90:128-247 for the convolution):
//   1. cloud-in-cell deposit of the particle mass, scaled to a density by
//      (N/L)^3 (src/partmesh.c:86-180);
//   2. FFT, multiplication by the long-range Green's function
//      G(k) = L^2 / (pi N^3) exp(-|k|^2 (2 pi rs / L)^2) / |k|^2 / W(k)^2,
//      W = prod sinc(pi k_d / N) (the CIC window, deconvolved twice), and the
//      inverse FFT: the potential psi with G-free units (conv.f90:171-227);
//   3. a 4-point finite-difference gradient of psi per mesh cell
//      (src/partmesh.c:524-735) and its CIC interpolation to the particles:
//      acc_pm = grad psi (src/partmesh.c:574-587).
// The mesh arithmetic is FP64 in the reference's order, every product and
// sum rounded on its own except the interpolation sums (fused multiply-adds);
// the constant pi is the reference's: conv.f90 declares
// `real*8, parameter :: M_PI = 3.1415926`, a default (single-precision)
// real literal, so its value is 3.1415926 rounded to FP32 (3.141592502593994).
// The deposit adds with FP64 atomics, so its summation order (and the last
// bits of the density) varies from run to run.
#include <cufft.h>

#include <cmath>

#include "api_internal.cuh"

namespace {

constexpr double PM_PI = (double)3.1415926f;  // src/conv.f90:171

struct Cic {
    int i, j, k, ii, jj, kk;
    double wi, wj, wk, win, wjn, wkn;
};

__device__ __forceinline__ int wrap(int a, int N) { return a < 0 ? a + N : (a >= N ? a - N : a); }

// nearest cell, neighbour cell on the particle's side and the two weights
// per axis (src/partmesh.c:91-132)
__device__ __forceinline__ void cic_axis(double x, double norm, double delta, int N, int &c, int &cn, double &w,
                                         double &wn)
{
    c = (int)__dmul_rn(x, norm);
    w = __dmul_rn(__dsub_rn(x, __dmul_rn((double)c + 0.5, delta)), norm);
    if (w > 0) {
        cn = c + 1;
    } else {
        w = -w;
        cn = c - 1;
    }
    wn = __dsub_rn(1.0, w);
    c = wrap(c, N);
    cn = wrap(cn, N);
}

__device__ __forceinline__ Cic cic(const double *pos, int p, double norm, double delta, int N)
{
    Cic s;
    cic_axis(pos[3 * (size_t)p], norm, delta, N, s.i, s.ii, s.wi, s.win);
    cic_axis(pos[3 * (size_t)p + 1], norm, delta, N, s.j, s.jj, s.wj, s.wjn);
    cic_axis(pos[3 * (size_t)p + 2], norm, delta, N, s.k, s.kk, s.wk, s.wkn);
    return s;
}

__device__ __forceinline__ size_t cell(int i, int j, int k, int N) { return ((size_t)i * N + j) * N + k; }


__global__ void k_pm_deposit(const double *__restrict__ pos, int n, int N, double norm, double delta, double mass,
                             double *rho)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const Cic s = cic(pos, p, norm, delta, N);
        // ((m wx) wy) wz with the shared leading products formed once
        const double mn = __dmul_rn(mass, s.win), mi = __dmul_rn(mass, s.wi);
        const double nn = __dmul_rn(mn, s.wjn), in = __dmul_rn(mi, s.wjn);
        const double nj = __dmul_rn(mn, s.wj), ij = __dmul_rn(mi, s.wj);
        atomicAdd(rho + cell(s.i, s.j, s.k, N), __dmul_rn(nn, s.wkn));
        atomicAdd(rho + cell(s.ii, s.j, s.k, N), __dmul_rn(in, s.wkn));
        atomicAdd(rho + cell(s.i, s.jj, s.k, N), __dmul_rn(nj, s.wkn));
        atomicAdd(rho + cell(s.i, s.j, s.kk, N), __dmul_rn(nn, s.wk));
        atomicAdd(rho + cell(s.ii, s.jj, s.k, N), __dmul_rn(ij, s.wkn));
        atomicAdd(rho + cell(s.ii, s.j, s.kk, N), __dmul_rn(in, s.wk));
        atomicAdd(rho + cell(s.i, s.jj, s.kk, N), __dmul_rn(nj, s.wk));
        atomicAdd(rho + cell(s.ii, s.jj, s.kk, N), __dmul_rn(ij, s.wk));
    }
}

__global__ void k_pm_scale(double *a, size_t m, double s)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x)
        a[i] = __dmul_rn(a[i], s);
}

// sinc(pi q / N), 1 at q = 0, as the reference forms it
__device__ __forceinline__ double pm_sinc(int q, int N)
{
    if (q == 0) return 1.0;
    const double f = __ddiv_rn(__dmul_rn(PM_PI, (double)q), (double)N);
    return __ddiv_rn(sin(f), f);
}

// the Green's function on the half spectrum [N][N][N/2+1]; it depends only
// on the mesh size, L and rs, so a context computes it once per set
__global__ void k_pm_green_table(double *G, int N, double pref, double ismth2)
{
    const int nz = N / 2 + 1, nhalf = N / 2;
    const size_t m = (size_t)N * N * nz;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < m; t += (size_t)gridDim.x * blockDim.x) {
        int a = (int)(t / ((size_t)N * nz)), b = (int)((t / nz) % N), c = (int)(t % nz);
        if (a > nhalf) a -= N;
        if (b > nhalf) b -= N;
        if (c > nhalf) c -= N;
        double gf;
        if (a == 0 && b == 0 && c == 0) {
            gf = pref;
        } else {
            const double fx = pm_sinc(a, N), fy = pm_sinc(b, N), fz = pm_sinc(c, N);
            const double k2 = (double)(a * a + b * b + c * c);
            const double ff = __ddiv_rn(1.0, __dmul_rn(__dmul_rn(fx, fy), fz));
            gf = __dmul_rn(pref, exp(__dmul_rn(-k2, ismth2)));
            gf = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(gf, ff), ff), ff), ff);
            gf = __ddiv_rn(gf, k2);
        }
        G[t] = gf;
    }
}

// the half spectrum times the Green's function
__global__ void k_pm_green(cufftDoubleComplex *rk, const double *__restrict__ G, size_t m)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < m; t += (size_t)gridDim.x * blockDim.x) {
        const double gf = G[t];
        rk[t].x = __dmul_rn(rk[t].x, gf);
        rk[t].y = __dmul_rn(rk[t].y, gf);
    }
}

// 4-point derivative along each axis (src/partmesh.c:524-531):
// f1 invx (psi+1 - psi-1) - f2 invx (psi+2 - psi-2), f1 = 4/3, f2 = 1/6, invx = N / (2 L)
// (x, y, z, 0) per cell, one 32-byte record, so that the interpolation's
// eight corners are eight sector loads
__global__ void k_pm_gradient(const double *__restrict__ psi, int N, double invx, double4_32a *g4)
{
    const double f1 = 4.0 / 3.0, f2 = 1.0 / 6.0;
    const double c1 = __dmul_rn(f1, invx), c2 = __dmul_rn(f2, invx);
    const size_t m = (size_t)N * N * N;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < m; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / ((size_t)N * N)), j = (int)((t / N) % N), k = (int)(t % N);
        double d, gx, gy, gz;
        d = __dmul_rn(c1, __dsub_rn(psi[cell(wrap(i + 1, N), j, k, N)], psi[cell(wrap(i - 1, N), j, k, N)]));
        gx = __dsub_rn(d, __dmul_rn(c2, __dsub_rn(psi[cell(wrap(i + 2, N), j, k, N)], psi[cell(wrap(i - 2, N), j, k, N)])));
        d = __dmul_rn(c1, __dsub_rn(psi[cell(i, wrap(j + 1, N), k, N)], psi[cell(i, wrap(j - 1, N), k, N)]));
        gy = __dsub_rn(d, __dmul_rn(c2, __dsub_rn(psi[cell(i, wrap(j + 2, N), k, N)], psi[cell(i, wrap(j - 2, N), k, N)])));
        d = __dmul_rn(c1, __dsub_rn(psi[cell(i, j, wrap(k + 1, N), N)], psi[cell(i, j, wrap(k - 1, N), N)]));
        gz = __dsub_rn(d, __dmul_rn(c2, __dsub_rn(psi[cell(i, j, wrap(k + 2, N), N)], psi[cell(i, j, wrap(k - 2, N), N)])));
        g4[t] = make_double4_32a(gx, gy, gz, 0.0);
    }
}

// one corner's weighted gradient added to the three running sums.  The
// adds are fused multiply-adds (one rounding instead of two): the kernel is
// bound by GB300's FP64 pipe, and this halves its work in the sums.
__device__ __forceinline__ void corner(double3 &a, double w, const double4_32a &g, bool first)
{
    if (first) {
        a = make_double3(__dmul_rn(w, g.x), __dmul_rn(w, g.y), __dmul_rn(w, g.z));
    } else {
        a.x = __fma_rn(w, g.x, a.x);
        a.y = __fma_rn(w, g.y, a.y);
        a.z = __fma_rn(w, g.z, a.z);
    }
}

// the eight weighted cell values summed in the reference's order, for the
// three components at once
__global__ void k_pm_interp(const double *__restrict__ pos, int n, int N, double norm, double delta,
                            const double4_32a *__restrict__ g4, double *acc)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const Cic s = cic(pos, p, norm, delta, N);
        // (wx wy) wz with the four leading products formed once
        const double nn = __dmul_rn(s.win, s.wjn), in = __dmul_rn(s.wi, s.wjn);
        const double nj = __dmul_rn(s.win, s.wj), ij = __dmul_rn(s.wi, s.wj);
        double3 a;
        corner(a, __dmul_rn(nn, s.wkn), g4[cell(s.i, s.j, s.k, N)], true);
        corner(a, __dmul_rn(in, s.wkn), g4[cell(s.ii, s.j, s.k, N)], false);
        corner(a, __dmul_rn(nj, s.wkn), g4[cell(s.i, s.jj, s.k, N)], false);
        corner(a, __dmul_rn(ij, s.wkn), g4[cell(s.ii, s.jj, s.k, N)], false);
        corner(a, __dmul_rn(nn, s.wk), g4[cell(s.i, s.j, s.kk, N)], false);
        corner(a, __dmul_rn(in, s.wk), g4[cell(s.ii, s.j, s.kk, N)], false);
        corner(a, __dmul_rn(nj, s.wk), g4[cell(s.i, s.jj, s.kk, N)], false);
        corner(a, __dmul_rn(ij, s.wk), g4[cell(s.ii, s.jj, s.kk, N)], false);
        acc[3 * (size_t)p] = a.x;
        acc[3 * (size_t)p + 1] = a.y;
        acc[3 * (size_t)p + 2] = a.z;
    }
}

int cufft_error(cufftResult r, const char *what)
{
    return ph_set_error(PH_ERR_CUDA, "%s failed (cuFFT status %d)", what, (int)r);
}

}  // namespace

// mesh buffers and FFT plans of one mesh size, kept in the context
int ph_pm_prepare(photons_ctx *c, int N)
{
    if (c->pm_n == N) return 0;
    if (c->pm_plan_r2c) cufftDestroy(c->pm_plan_r2c);
    if (c->pm_plan_c2r) cufftDestroy(c->pm_plan_c2r);
    c->pm_plan_r2c = c->pm_plan_c2r = 0;
    cudaFree(c->pm_rho); cudaFree(c->pm_rk); cudaFree(c->pm_grad); cudaFree(c->pm_green);
    c->pm_rho = nullptr; c->pm_rk = nullptr; c->pm_grad = nullptr; c->pm_green = nullptr;
    c->pm_n = 0;
    c->pm_green_pref = c->pm_green_ismth2 = 0.0;
    const size_t m = (size_t)N * N * N, mk = (size_t)N * N * (N / 2 + 1);
    cudaError_t e = cudaMalloc(&c->pm_rho, sizeof(double) * m);
    if (e == cudaSuccess) e = cudaMalloc(&c->pm_rk, sizeof(cufftDoubleComplex) * mk);
    if (e == cudaSuccess) e = cudaMalloc(&c->pm_grad, 4 * sizeof(double) * m);
    if (e == cudaSuccess) e = cudaMalloc(&c->pm_green, sizeof(double) * mk);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return ph_set_error(PH_ERR_NOMEM, "PM mesh of %d^3 cells does not fit", N);
    }
    cufftResult r = cufftPlan3d(&c->pm_plan_r2c, N, N, N, CUFFT_D2Z);
    if (r != CUFFT_SUCCESS) return cufft_error(r, "cufftPlan3d (forward)");
    r = cufftPlan3d(&c->pm_plan_c2r, N, N, N, CUFFT_Z2D);
    if (r != CUFFT_SUCCESS) return cufft_error(r, "cufftPlan3d (inverse)");
    c->pm_n = N;
    return 0;
}

void ph_pm_release(photons_ctx *c)
{
    if (c->pm_plan_r2c) cufftDestroy(c->pm_plan_r2c);
    if (c->pm_plan_c2r) cufftDestroy(c->pm_plan_c2r);
    cudaFree(c->pm_rho); cudaFree(c->pm_rk); cudaFree(c->pm_grad); cudaFree(c->pm_green);
    c->pm_plan_r2c = c->pm_plan_c2r = 0;
    c->pm_rho = nullptr; c->pm_rk = nullptr; c->pm_grad = nullptr; c->pm_green = nullptr;
    c->pm_n = 0;
    c->pm_green_pref = c->pm_green_ismth2 = 0.0;
}

// enqueue the PM force on device positions pos[3n] into acc_pm[3n]
int ph_pm_enqueue(photons_ctx *c, const photons_params *p, int N, int n, const double *pos, double *acc_pm)
{
    PH_TRY(ph_pm_prepare(c, N));
    cudaStream_t st = c->stream;
    const size_t m = (size_t)N * N * N, mk = (size_t)N * N * (N / 2 + 1);
    const int blocks = ph::device_sm_count() * 8;
    const double L = p->boxsize;
    const double norm = (double)N / L, delta = 1.0 / norm;  // src/partmesh.c:85-86
    PH_CUDA_CHECK(cudaMemsetAsync(c->pm_rho, 0, sizeof(double) * m, st));
    ph::note_launch(), k_pm_deposit<<<blocks, 256, 0, st>>>(pos, n, N, norm, delta, p->mass, c->pm_rho);
    double renormal = (double)N / L;
    renormal = renormal * renormal * renormal;
    ph::note_launch(), k_pm_scale<<<blocks, 256, 0, st>>>(c->pm_rho, m, renormal);
    cufftResult r = cufftSetStream(c->pm_plan_r2c, st);
    if (r == CUFFT_SUCCESS) r = cufftSetStream(c->pm_plan_c2r, st);
    if (r == CUFFT_SUCCESS) r = cufftExecD2Z(c->pm_plan_r2c, c->pm_rho, c->pm_rk);
    if (r != CUFFT_SUCCESS) return cufft_error(r, "cufftExecD2Z");
    // conv.f90:175-177: ismth2 = (2 pi rs / L)^2, pref = L^2 / (pi N^3)
    double ismth2 = 2 * PM_PI * p->rs / L;
    ismth2 = ismth2 * ismth2;
    const double pref = L * L / (PM_PI * (double)N * (double)N * (double)N);
    if (c->pm_green_pref != pref || c->pm_green_ismth2 != ismth2) {
        ph::note_launch(), k_pm_green_table<<<blocks, 256, 0, st>>>(c->pm_green, N, pref, ismth2);
        c->pm_green_pref = pref;
        c->pm_green_ismth2 = ismth2;
    }
    ph::note_launch(), k_pm_green<<<blocks, 256, 0, st>>>(c->pm_rk, c->pm_green, mk);
    r = cufftExecZ2D(c->pm_plan_c2r, c->pm_rk, c->pm_rho);
    if (r != CUFFT_SUCCESS) return cufft_error(r, "cufftExecZ2D");
    const double invx = 0.5 * N / L;  // src/partmesh.c:458
    double4_32a *g4 = reinterpret_cast<double4_32a *>(c->pm_grad);
    ph::note_launch(), k_pm_gradient<<<blocks, 256, 0, st>>>(c->pm_rho, N, invx, g4);
    ph::note_launch(), k_pm_interp<<<blocks, 256, 0, st>>>(pos, n, N, norm, delta, g4, acc_pm);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

extern "C" int photons_pm_force(photons_ctx *c, const photons_params *p, int nside, int n, const double *pos,
                                double *acc_pm)
{
    photons_gpu_clear_error();
    if (!c || !p || !pos || !acc_pm) return ph_set_error(PH_ERR_ARG, "null argument");
    if (n < 1 || nside < 4 || nside > 2048) return ph_set_error(PH_ERR_ARG, "bad PM arguments (n %d, mesh %d)", n, nside);
    if (!(p->boxsize > 0) || !(p->rs > 0)) return ph_set_error(PH_ERR_ARG, "invalid PM parameters");
    cudaSetDevice(c->device);
    cudaStream_t st = c->stream;
    const int dio = p->flags & PHOTONS_F_DEVICE_IO;
    const double *dpos = pos;
    double *dacc = acc_pm;
    if (!dio) {
        if (n > c->pm_cap_io) {
            cudaFree(c->pm_io);
            c->pm_io = nullptr;
            c->pm_cap_io = 0;
            if (cudaMalloc(&c->pm_io, sizeof(double) * 6 * (size_t)n) != cudaSuccess) {
                cudaGetLastError();
                return ph_set_error(PH_ERR_NOMEM, "PM staging for %d particles does not fit", n);
            }
            c->pm_cap_io = n;
        }
        PH_CUDA_CHECK(cudaMemcpyAsync(c->pm_io, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, st));
        dpos = c->pm_io;
        dacc = c->pm_io + 3 * (size_t)n;
    }
    PH_TRY(ph_pm_enqueue(c, p, nside, n, dpos, dacc));
    if (!dio)
        PH_CUDA_CHECK(cudaMemcpyAsync(acc_pm, dacc, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    return 0;
}
