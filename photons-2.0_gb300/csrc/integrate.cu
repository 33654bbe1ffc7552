// Kick-drift-kick time integration on device-resident particles.
//
// Restates the reference's step (src/photoNs.c:141-196 and 257-268):
//   dk = kick_loga(loga_i, loga_f), dd = drift_loga(loga_i, loga_f),
//   dkh = dk G / 2;  vel += acc dkh;  pos += vel dd;  wrap into [0, L);
//   forces at the new positions;  vel += acc dkh.
// Every update is a separately rounded product and sum, as the reference's
// loops compute them, so a step matches the reference bit for bit given the
// same accelerations.  The kernels stream the 3N-double arrays and are HBM
// bound: a kick moves 24 bytes per coordinate, a drift 24 bytes; each does
// one FP64 multiply and one add per coordinate.
#include <cmath>

#include "api_internal.cuh"

namespace {

// the reference's factor integrands, Simpson's rule over 128 intervals of
// log a (src/initial.c:639-683): z/h for the kick, z^2/h for the drift,
// h = 0.1 sqrt(Om z^3 + OL), z = 1/a.  Summation order as in the reference.
double loga_integral(double om, double ox, double loga_i, double loga_f, int zpow)
{
    const int nblock = 128;
    const double dloga = (loga_f - loga_i) / nblock;
    auto term = [&](double z) {
        const double h = 0.1 * sqrt(om * z * z * z + ox);
        return zpow == 1 ? dloga * z / h : dloga * z * z / h;
    };
    double s = term(1.0 / exp(loga_i));
    for (int n = 1; n < nblock; n++) {
        const double z = 1.0 / (exp(loga_i + dloga * n));
        const double h = 0.1 * sqrt(om * z * z * z + ox);
        s += zpow == 1 ? 2.0 * (1 + n % 2) * dloga * z / h : 2.0 * (1 + n % 2) * dloga * z * z / h;
    }
    s += term(1.0 / exp(loga_f));
    return s / 3.0;
}

// vel[i] += acc[i] * dkh over the flat 3n arrays, two doubles per access
__global__ void k_kick(double *__restrict__ vel, const double *__restrict__ acc, double dkh, long long m)
{
    const long long m2 = m >> 1;
    double2 *v2 = reinterpret_cast<double2 *>(vel);
    const double2 *a2 = reinterpret_cast<const double2 *>(acc);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m2; i += (long long)gridDim.x * blockDim.x) {
        double2 v = v2[i];
        const double2 a = a2[i];
        v.x = __dadd_rn(v.x, __dmul_rn(a.x, dkh));
        v.y = __dadd_rn(v.y, __dmul_rn(a.y, dkh));
        v2[i] = v;
    }
    if ((m & 1) && blockIdx.x == 0 && threadIdx.x == 0) vel[m - 1] = __dadd_rn(vel[m - 1], __dmul_rn(acc[m - 1], dkh));
}

// The reference's wrap: add L while below 0, then subtract L while >= L;
// bounded, so a non-finite coordinate is left as it is.  The common case
// 0 <= x < L is decided on the bit pattern (for non-negative doubles the
// integer order is the numeric order; -0.0, negatives, infinities and NaN
// all fail it) so that it costs no FP64 compare.
__device__ __forceinline__ double wrap_coord(double x, double L, long long Lbits)
{
    const long long b = __double_as_longlong(x);
    if (b >= 0 && b < Lbits) return x;
    int k = 0;
    while (x < 0.0 && k < 64) { x = __dadd_rn(x, L); k++; }
    while (x >= L && k < 128) { x = __dsub_rn(x, L); k++; }
    return x;
}

__global__ void k_drift(double *__restrict__ pos, const double *__restrict__ vel, double dd, double L, long long m)
{
    const long long m2 = m >> 1;
    const long long Lb = __double_as_longlong(L);
    double2 *p2 = reinterpret_cast<double2 *>(pos);
    const double2 *v2 = reinterpret_cast<const double2 *>(vel);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m2; i += (long long)gridDim.x * blockDim.x) {
        double2 p = p2[i];
        const double2 v = v2[i];
        p.x = wrap_coord(__dadd_rn(p.x, __dmul_rn(v.x, dd)), L, Lb);
        p.y = wrap_coord(__dadd_rn(p.y, __dmul_rn(v.y, dd)), L, Lb);
        p2[i] = p;
    }
    if ((m & 1) && blockIdx.x == 0 && threadIdx.x == 0)
        pos[m - 1] = wrap_coord(__dadd_rn(pos[m - 1], __dmul_rn(vel[m - 1], dd)), L, Lb);
}

// The same kick and drift with the factor read from device memory, for a
// step captured once as a graph and launched with new factors each time;
// a nonzero *skip (the pass before it failed to fit) leaves vel as it is.
__global__ void k_kick_dev(double *__restrict__ vel, const double *__restrict__ acc, const double *f,
                           const int *skip, long long m)
{
    if (skip && *skip) return;
    const double dkh = *f;
    const long long m2 = m >> 1;
    double2 *v2 = reinterpret_cast<double2 *>(vel);
    const double2 *a2 = reinterpret_cast<const double2 *>(acc);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m2; i += (long long)gridDim.x * blockDim.x) {
        double2 v = v2[i];
        const double2 a = a2[i];
        v.x = __dadd_rn(v.x, __dmul_rn(a.x, dkh));
        v.y = __dadd_rn(v.y, __dmul_rn(a.y, dkh));
        v2[i] = v;
    }
    if ((m & 1) && blockIdx.x == 0 && threadIdx.x == 0) vel[m - 1] = __dadd_rn(vel[m - 1], __dmul_rn(acc[m - 1], dkh));
}

__global__ void k_drift_dev(double *__restrict__ pos, const double *__restrict__ vel, const double *f, double L,
                            long long m)
{
    const double dd = *f;
    const long long m2 = m >> 1;
    const long long Lb = __double_as_longlong(L);
    double2 *p2 = reinterpret_cast<double2 *>(pos);
    const double2 *v2 = reinterpret_cast<const double2 *>(vel);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m2; i += (long long)gridDim.x * blockDim.x) {
        double2 p = p2[i];
        const double2 v = v2[i];
        p.x = wrap_coord(__dadd_rn(p.x, __dmul_rn(v.x, dd)), L, Lb);
        p.y = wrap_coord(__dadd_rn(p.y, __dmul_rn(v.y, dd)), L, Lb);
        p2[i] = p;
    }
    if ((m & 1) && blockIdx.x == 0 && threadIdx.x == 0)
        pos[m - 1] = wrap_coord(__dadd_rn(pos[m - 1], __dmul_rn(vel[m - 1], dd)), L, Lb);
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

int enqueue_kick(int n, double *vel, const double *acc, double dkh, cudaStream_t st)
{
    if (n < 0 || (n > 0 && (!vel || !acc))) return ph_set_error(PH_ERR_ARG, "bad kick arguments");
    if (!aligned16(vel) || !aligned16(acc)) return ph_set_error(PH_ERR_ARG, "kick arrays must be 16-byte aligned");
    if (n == 0) return 0;
    ph::note_launch(), k_kick<<<ph::device_sm_count() * 8, 256, 0, st>>>(vel, acc, dkh, 3LL * n);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int enqueue_drift(int n, double *pos, const double *vel, double dd, double L, cudaStream_t st)
{
    if (n < 0 || (n > 0 && (!pos || !vel)) || !(L > 0)) return ph_set_error(PH_ERR_ARG, "bad drift arguments");
    if (!aligned16(pos) || !aligned16(vel)) return ph_set_error(PH_ERR_ARG, "drift arrays must be 16-byte aligned");
    if (n == 0) return 0;
    ph::note_launch(), k_drift<<<ph::device_sm_count() * 8, 256, 0, st>>>(pos, vel, dd, L, 3LL * n);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace

namespace {

// positions in tree order from the build's FP64 copies (the same values)
__global__ void k_pos_from_tree(const double *__restrict__ x, const double *__restrict__ y,
                                const double *__restrict__ z, int n, double *pos)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        pos[3 * (size_t)i] = x[i];
        pos[3 * (size_t)i + 1] = y[i];
        pos[3 * (size_t)i + 2] = z[i];
    }
}

// out[i] = in[perm[i]], for records of w 8-byte words
__global__ void k_permute(const int *__restrict__ perm, const long long *__restrict__ in, int n, int w,
                          long long *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t s = (size_t)perm[i] * w, d = (size_t)i * w;
        for (int k = 0; k < w; k++) out[d + k] = in[s + k];
    }
}

// after a pass with PHOTONS_F_TREE_ORDER: positions, velocities and ids
// (optional) into the pass's tree order, as the reference keeps part[]
// (src/fmm.c:30-78 permutes whole Body records); acc is already in it
int reorder_state(photons_ctx *c, int n, double *pos, double *vel, long long *ids, cudaStream_t st)
{
    const int blocks = ph::device_sm_count() * 8;
    ph::note_launch(), k_pos_from_tree<<<blocks, 256, 0, st>>>(c->b.x, c->b.y, c->b.z, n, pos);
    long long *scratch = reinterpret_cast<long long *>(c->io);  // 3n words, free between passes
    ph::note_launch(), k_permute<<<blocks, 256, 0, st>>>(c->b.perm, reinterpret_cast<const long long *>(vel), n, 3,
                                                      scratch);
    PH_CUDA_CHECK(cudaMemcpyAsync(vel, scratch, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    if (ids) {
        ph::note_launch(), k_permute<<<blocks, 256, 0, st>>>(c->b.perm, ids, n, 1, scratch);
        PH_CUDA_CHECK(cudaMemcpyAsync(ids, scratch, sizeof(long long) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    }
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace

extern "C" double photons_kick_loga(double omega_m, double omega_x, double loga_i, double loga_f)
{
    return loga_integral(omega_m, omega_x, loga_i, loga_f, 1);
}

extern "C" double photons_drift_loga(double omega_m, double omega_x, double loga_i, double loga_f)
{
    return loga_integral(omega_m, omega_x, loga_i, loga_f, 2);
}

extern "C" int photons_kick(int n, double *vel, const double *acc, double dkh, void *cuda_stream)
{
    photons_gpu_clear_error();
    return enqueue_kick(n, vel, acc, dkh, (cudaStream_t)cuda_stream);
}

extern "C" int photons_drift(int n, double *pos, const double *vel, double dd, double boxsize, void *cuda_stream)
{
    photons_gpu_clear_error();
    return enqueue_drift(n, pos, vel, dd, boxsize, (cudaStream_t)cuda_stream);
}

// launchers of the device-factor kernels (the captured step in api.cu)
int ph_enqueue_kick_dev(int n, double *vel, const double *acc, const double *dkh, const int *skip, cudaStream_t st)
{
    if (n < 0 || (n > 0 && (!vel || !acc || !dkh))) return ph_set_error(PH_ERR_ARG, "bad kick arguments");
    if (!aligned16(vel) || !aligned16(acc)) return ph_set_error(PH_ERR_ARG, "kick arrays must be 16-byte aligned");
    if (n == 0) return 0;
    ph::note_launch(), k_kick_dev<<<ph::device_sm_count() * 8, 256, 0, st>>>(vel, acc, dkh, skip, 3LL * n);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int ph_enqueue_drift_dev(int n, double *pos, const double *vel, const double *dd, double L, cudaStream_t st)
{
    if (n < 0 || (n > 0 && (!pos || !vel || !dd)) || !(L > 0)) return ph_set_error(PH_ERR_ARG, "bad drift arguments");
    if (!aligned16(pos) || !aligned16(vel)) return ph_set_error(PH_ERR_ARG, "drift arrays must be 16-byte aligned");
    if (n == 0) return 0;
    ph::note_launch(), k_drift_dev<<<ph::device_sm_count() * 8, 256, 0, st>>>(pos, vel, dd, L, 3LL * n);
    PH_CUDA_CHECK(cudaGetLastError());
    return 0;
}

extern "C" int photons_kdk_step(photons_ctx *c, const photons_params *p, int n, double *pos, double *vel,
                                double *acc, double dkh, double dd)
{
    photons_gpu_clear_error();
    if (!c || !p) return ph_set_error(PH_ERR_ARG, "null argument");
    cudaSetDevice(c->device);
    cudaStream_t st = c->stream;
    photons_params q = *p;
    q.flags |= PHOTONS_F_DEVICE_IO;
    q.flags &= ~PHOTONS_F_TREE_ORDER;
    // the whole step as one captured graph once this pass's own graph fits
    // (ph_kdk_graph_step); otherwise, or to repeat a pass that did not fit
    // after the graph's kick and drift, the steps one by one
    int done = 0;
    PH_TRY(ph_kdk_graph_step(c, &q, n, pos, vel, acc, dkh, dd, &done));
    if (done == KDK_DONE) return 0;
    if (done == KDK_NOT_RUN) {
        PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
        PH_TRY(enqueue_drift(n, pos, vel, dd, p->boxsize, st));
    }
    PH_TRY(photons_force_pass(c, &q, n, pos, acc));
    PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    return 0;
}

extern "C" int photons_kdk_step_pm(photons_ctx *c, const photons_params *p, int nside, int n, double *pos,
                                   double *vel, double *acc, double *acc_pm, double dkh, double dd)
{
    photons_gpu_clear_error();
    if (!c || !p || !acc_pm) return ph_set_error(PH_ERR_ARG, "null argument");
    cudaSetDevice(c->device);
    cudaStream_t st = c->stream;
    // src/photoNs.c:158-196: PM kick, short-range kick, drift and wrap
    PH_TRY(enqueue_kick(n, vel, acc_pm, dkh, st));
    PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
    PH_TRY(enqueue_drift(n, pos, vel, dd, p->boxsize, st));
    // forces at the new positions: the short-range pass and the PM mesh
    photons_params q = *p;
    q.flags |= PHOTONS_F_DEVICE_IO;
    q.flags &= ~PHOTONS_F_TREE_ORDER;
    PH_TRY(photons_force_pass(c, &q, n, pos, acc));
    PH_TRY(ph_pm_enqueue(c, &q, nside, n, pos, acc_pm));
    // src/photoNs.c:257-268: short-range kick, then PM kick
    PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
    PH_TRY(enqueue_kick(n, vel, acc_pm, dkh, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    return 0;
}

// The same steps with the state kept in the order of the last pass's tree:
// after the short-range pass, pos, vel (and ids, if given) are permuted
// into tree order and acc comes back in it, so every array stays in one
// order and the next build starts from nearly sorted particles, as the
// reference's driver does with part[].  The caller follows particles by ids.
extern "C" int photons_kdk_step_ordered(photons_ctx *c, const photons_params *p, int n, double *pos, double *vel,
                                        double *acc, long long *ids, double dkh, double dd)
{
    photons_gpu_clear_error();
    if (!c || !p) return ph_set_error(PH_ERR_ARG, "null argument");
    cudaSetDevice(c->device);
    cudaStream_t st = c->stream;
    PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
    PH_TRY(enqueue_drift(n, pos, vel, dd, p->boxsize, st));
    photons_params q = *p;
    q.flags |= PHOTONS_F_DEVICE_IO | PHOTONS_F_TREE_ORDER;
    PH_TRY(photons_force_pass(c, &q, n, pos, acc));
    PH_TRY(reorder_state(c, n, pos, vel, ids, st));
    PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    return 0;
}

extern "C" int photons_kdk_step_pm_ordered(photons_ctx *c, const photons_params *p, int nside, int n, double *pos,
                                           double *vel, double *acc, double *acc_pm, long long *ids, double dkh,
                                           double dd)
{
    photons_gpu_clear_error();
    if (!c || !p || !acc_pm) return ph_set_error(PH_ERR_ARG, "null argument");
    cudaSetDevice(c->device);
    cudaStream_t st = c->stream;
    PH_TRY(enqueue_kick(n, vel, acc_pm, dkh, st));
    PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
    PH_TRY(enqueue_drift(n, pos, vel, dd, p->boxsize, st));
    photons_params q = *p;
    q.flags |= PHOTONS_F_DEVICE_IO | PHOTONS_F_TREE_ORDER;
    PH_TRY(photons_force_pass(c, &q, n, pos, acc));
    PH_TRY(reorder_state(c, n, pos, vel, ids, st));
    // the PM force at the reordered positions comes out in the same order
    PH_TRY(ph_pm_enqueue(c, &q, nside, n, pos, acc_pm));
    PH_TRY(enqueue_kick(n, vel, acc, dkh, st));
    PH_TRY(enqueue_kick(n, vel, acc_pm, dkh, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    return 0;
}
