/*
 * One-rank stand-in for the reference's Fortran convolution
 * (src/conv.f90:128-247, subroutine `convolution`), so that the reference's
 * own PM (src/partmesh.c, compiled in place by oracle/Makefile) runs here
 * without 2DECOMP&FFT.  TEST INFRASTRUCTURE ONLY: it lets the reference's
 * CIC deposit, halo exchange, 4-point gradient and interpolation pin the
 * PM restatement (oracle/pm_oracle.py).
 *
 * What it restates, in place on data[(i N + j) N + k] (the layout
 * partmesh.c hands over, the Fortran's in(i, j, k)):
 *   forward 3-D transform of the density (unnormalised);
 *   multiplication by the Green's function
 *     pref exp(-k^2 ismth2) ff ff ff ff / k^2,  ff = 1 / (fx fy fz),
 *     pref = L^2 / (pi N^3), ismth2 = (2 pi rs / L)^2, DC term = pref,
 *   in the Fortran's operation order;
 *   inverse transform (unnormalised), real part back into data.
 * The Fortran declares `real*8, parameter :: M_PI = 3.1415926`, a
 * default-kind (single-precision) literal, so its pi is 3.1415926f.
 * The transform is a direct separable DFT, exact to rounding, for the small
 * meshes the tests use: the FFT library is the one part of the reference's
 * PM this does not reproduce.
 */
#include <math.h>
#include <stdlib.h>

static const double CONV_PI = (double)3.1415926f;

/* one axis of an N^3 complex array held as re/im, C order (axis 0 slowest) */
static void dft_axis(double *re, double *im, int N, int axis, double sign, const double *cs, const double *sn,
                     double *tr, double *ti)
{
    const long NN = (long)N * N;
    const long stride = axis == 0 ? NN : axis == 1 ? N : 1;
    for (int a = 0; a < N; a++)
        for (int b = 0; b < N; b++) {
            const long base = axis == 0 ? (long)a * N + b : axis == 1 ? (long)a * NN + b : ((long)a * N + b) * N;
            for (int q = 0; q < N; q++) {
                double sr = 0.0, si = 0.0;
                for (int p = 0; p < N; p++) {
                    const int t = (int)(((long)p * q) % N);
                    const double c = cs[t], s = sign * sn[t];
                    const double xr = re[base + p * stride], xi = im[base + p * stride];
                    sr += xr * c - xi * s;
                    si += xr * s + xi * c;
                }
                tr[q] = sr;
                ti[q] = si;
            }
            for (int q = 0; q < N; q++) {
                re[base + q * stride] = tr[q];
                im[base + q * stride] = ti[q];
            }
        }
}

static void dft3(double *re, double *im, int N, double sign)
{
    double *cs = malloc(sizeof(double) * N), *sn = malloc(sizeof(double) * N);
    double *tr = malloc(sizeof(double) * N), *ti = malloc(sizeof(double) * N);
    for (int t = 0; t < N; t++) {
        cs[t] = cos(2.0 * M_PI * t / N);
        sn[t] = sin(2.0 * M_PI * t / N);
    }
    for (int axis = 0; axis < 3; axis++) dft_axis(re, im, N, axis, sign, cs, sn, tr, ti);
    free(cs); free(sn); free(tr); free(ti);
}

/* the sinc factor of one signed wavenumber (src/conv.f90:196-225) */
static double sinc_factor(int w, int n)
{
    if (w == 0) return 1.0;
    double f = CONV_PI * w / n;
    return sin(f) / f;
}

/* Fortran calling convention: every argument by reference */
void convolution_(double *data, int *nside, double *param)
{
    const int N = nside[0];
    const long n3 = (long)N * N * N;
    double *re = malloc(sizeof(double) * n3), *im = calloc((size_t)n3, sizeof(double));
    for (long c = 0; c < n3; c++) re[c] = data[c];
    dft3(re, im, N, -1.0);

    const int nhalf = N / 2;
    const double smooth = param[0], box = param[1];
    double ismth2 = 2 * CONV_PI * smooth / box;
    ismth2 = ismth2 * ismth2;
    const double pref = box * box / (CONV_PI * nside[0] * nside[1] * nside[2]);
    for (int i = 0; i < N; i++) {
        const int l = i > nhalf ? i - N : i;
        const double fx = sinc_factor(l, nside[0]);
        for (int j = 0; j < N; j++) {
            const int m = j > nhalf ? j - N : j;
            const double fy = sinc_factor(m, nside[1]);
            for (int k = 0; k < N; k++) {
                const int n = k > nhalf ? k - N : k;
                const double fz = sinc_factor(n, nside[2]);
                const double k2 = (double)(float)(n * n + m * m + l * l);  /* REAL(...): default kind */
                const double ff = 1.0 / (fx * fy * fz);
                double gf = pref * exp(-k2 * ismth2) * ff * ff * ff * ff / k2;
                if (l == 0 && m == 0 && n == 0) gf = pref;
                const long c = ((long)i * N + j) * N + k;
                re[c] *= gf;
                im[c] *= gf;
            }
        }
    }
    dft3(re, im, N, 1.0);
    for (long c = 0; c < n3; c++) data[c] = re[c];
    free(re);
    free(im);
}
