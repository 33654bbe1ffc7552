// photons_direct_sum_noalloc: the FP64 direct sum of photons_direct_sum for
// callers that cannot allocate device memory while they run.  A production
// run budgets HBM up front (particle arrays, the PM mesh, the force pass's
// pools), so a cudaMalloc issued between two steps may fail, and
// cudaMalloc/cudaFree synchronise the device and stall the caller's other
// streams.  Such a caller checks forces against this sum (e.g. every few
// steps) with device-resident inputs and outputs and no allocation at all.
//
// The scratch (cell lists and the binned source copy) lives in one
// file-scope __device__ array of fixed size, NA_SCRATCH_BYTES (about
// 10.8 MB), that every device loading this library holds until the process
// exits.  Limits: NA_MAX_SOURCES sources, NA_MAX_TARGETS targets, at most
// NA_MAX_CELL_SIDE^3 cells.  Every call reuses the same array: the cell
// counts and the error flag are cleared at the start of each call, and two
// calls that overlap on the GPU (different streams, different host threads)
// race on it.
//
// Host code must not pass g_direct_scratch itself to a kernel: on the host
// that name is a stand-in, not a device address.  The first call on each
// device looks the address up with cudaGetSymbolAddress while that device is
// current and keeps it for that device's CUDA context (a new context, e.g.
// after cudaDeviceReset, is looked up again); that first call should come
// before any stream capture.  The library's device code is loaded lazily, so
// the array itself is placed in device memory by that first lookup: a caller
// that budgets all of HBM makes one warm-up call first (nt = 0 does only
// the set-up and launches nothing).
#include <cuda.h>

#include <cmath>
#include <mutex>

#include "api_internal.cuh"

namespace {

constexpr int NA_MAX_SOURCES = 1 << 18;
constexpr int NA_MAX_TARGETS = 1 << 16;
constexpr int NA_MAX_CELL_SIDE = 64;
constexpr int NA_MAX_CELLS = NA_MAX_CELL_SIDE * NA_MAX_CELL_SIDE * NA_MAX_CELL_SIDE;
constexpr int NA_MAX_DEVICES = 64;

constexpr size_t na_align(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets of the scratch regions (each 256-byte aligned)
constexpr size_t NA_OFF_FLAG = 0;                                                        // int error flag
constexpr size_t NA_OFF_START = 256;                                                     // int[cells+1]
constexpr size_t NA_OFF_FILL = NA_OFF_START + na_align(sizeof(int) * (NA_MAX_CELLS + 1));  // int[cells]
constexpr size_t NA_OFF_SX = NA_OFF_FILL + na_align(sizeof(int) * NA_MAX_CELLS);          // double[sources] x3
constexpr size_t NA_OFF_SY = NA_OFF_SX + sizeof(double) * NA_MAX_SOURCES;
constexpr size_t NA_OFF_SZ = NA_OFF_SY + sizeof(double) * NA_MAX_SOURCES;
constexpr size_t NA_OFF_SLOT = NA_OFF_SZ + sizeof(double) * NA_MAX_SOURCES;                // int[sources]
constexpr size_t NA_OFF_TX = NA_OFF_SLOT + na_align(sizeof(int) * NA_MAX_SOURCES);         // double[targets] x3
constexpr size_t NA_OFF_TY = NA_OFF_TX + sizeof(double) * NA_MAX_TARGETS;
constexpr size_t NA_OFF_TZ = NA_OFF_TY + sizeof(double) * NA_MAX_TARGETS;
constexpr size_t NA_OFF_TSELF = NA_OFF_TZ + sizeof(double) * NA_MAX_TARGETS;               // int[targets]
constexpr size_t NA_SCRATCH_BYTES = NA_OFF_TSELF + na_align(sizeof(int) * NA_MAX_TARGETS);

static __device__ __align__(256) unsigned char g_direct_scratch[NA_SCRATCH_BYTES];

struct NaView {
    int *flag, *start, *fill, *slot, *tself;
    double *sx, *sy, *sz, *tx, *ty, *tz;
};

__device__ __forceinline__ NaView na_view(unsigned char *s)
{
    NaView v;
    v.flag = (int *)(s + NA_OFF_FLAG);
    v.start = (int *)(s + NA_OFF_START);
    v.fill = (int *)(s + NA_OFF_FILL);
    v.sx = (double *)(s + NA_OFF_SX);
    v.sy = (double *)(s + NA_OFF_SY);
    v.sz = (double *)(s + NA_OFF_SZ);
    v.slot = (int *)(s + NA_OFF_SLOT);
    v.tx = (double *)(s + NA_OFF_TX);
    v.ty = (double *)(s + NA_OFF_TY);
    v.tz = (double *)(s + NA_OFF_TZ);
    v.tself = (int *)(s + NA_OFF_TSELF);
    return v;
}

// cell of a position: the same clamped binning as photons_direct_sum
__device__ __forceinline__ int na_cell(const double *pos, int j, int ncell, double cw)
{
    int c[3];
    for (int d = 0; d < 3; d++) c[d] = min(max((int)(pos[3 * (size_t)j + d] / cw), 0), ncell - 1);
    return (c[0] * ncell + c[1]) * ncell + c[2];
}

__global__ void k_na_clear(unsigned char *s, int ncells)
{
    NaView v = na_view(s);
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 == 0) *v.flag = 0;
    for (int i = i0; i <= ncells; i += gridDim.x * blockDim.x) v.start[i] = 0;
}

__global__ void k_na_count(unsigned char *s, const double *pos, int n, int ncell, double cw)
{
    NaView v = na_view(s);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        atomicAdd(v.start + na_cell(pos, j, ncell, cw) + 1, 1);
}

// one block: inclusive scan of start[0..ncells] in place (start[0] is 0,
// start[c+1] the count of cell c), giving each cell's first slot; fill = start
__global__ void __launch_bounds__(1024) k_na_scan(unsigned char *s, int ncells)
{
    __shared__ int warp_tot[32];
    NaView v = na_view(s);
    const int m = ncells + 1;
    const int seg = (m + blockDim.x - 1) / blockDim.x;
    const int b = min(m, (int)threadIdx.x * seg), e = min(m, b + seg);
    int sum = 0;
    for (int i = b; i < e; i++) sum += v.start[i];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = sum;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    int run = inc - sum + (wid > 0 ? warp_tot[wid - 1] : 0);
    for (int i = b; i < e; i++) {
        run += v.start[i];
        v.start[i] = run;
        if (i < ncells) v.fill[i] = run;
    }
}

// with start holding each cell's first slot, fill is rewound to it above;
// the slot order inside a cell depends on atomic arrival
__global__ void k_na_place(unsigned char *s, const double *pos, int n, int ncell, double cw)
{
    NaView v = na_view(s);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int c = na_cell(pos, j, ncell, cw);
        // fill[c] starts at the cell's exclusive start: start[c] after the
        // inclusive scan is the end of cell c-1, i.e. the start of cell c
        const int slot = atomicAdd(v.fill + c, 1);
        v.sx[slot] = pos[3 * (size_t)j];
        v.sy[slot] = pos[3 * (size_t)j + 1];
        v.sz[slot] = pos[3 * (size_t)j + 2];
        v.slot[j] = slot;
    }
}

__global__ void k_na_targets(unsigned char *s, const double *pos, int n, const int *targets, int nt)
{
    NaView v = na_view(s);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
        const int j = targets[t];
        if (j < 0 || j >= n) {
            atomicOr(v.flag, 1);
            v.tx[t] = v.ty[t] = v.tz[t] = 0.0;
            v.tself[t] = -1;
            continue;
        }
        v.tx[t] = pos[3 * (size_t)j];
        v.ty[t] = pos[3 * (size_t)j + 1];
        v.tz[t] = pos[3 * (size_t)j + 2];
        v.tself[t] = v.slot[j];
    }
}

// warp per target over the 27 neighbouring cells; the arithmetic of the
// allocating direct sum, sources and targets read from the scratch
__global__ void k_na_direct(unsigned char *s, int ncell, double cellw, int nt, double L, double rmax2, double eps,
                            double mass, double rs, double *out)
{
    NaView v = na_view(s);
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const double coeff = 2.0 / sqrt(M_PI);
    const double soft3 = mass / (eps * eps * eps);
    const int nc3 = ncell * ncell * ncell;
    for (int t = gw; t < nt; t += nw) {
        const int self = v.tself[t];
        double ax = 0, ay = 0, az = 0;
        if (self >= 0) {
            const double px = v.tx[t], py = v.ty[t], pz = v.tz[t];
            int ci[3] = {(int)(px / cellw), (int)(py / cellw), (int)(pz / cellw)};
            for (int d = 0; d < 3; d++) ci[d] = min(max(ci[d], 0), ncell - 1);
            const int span = ncell >= 3 ? 1 : 0;
            for (int ox = -span; ox <= span; ox++)
                for (int oy = -span; oy <= span; oy++)
                    for (int oz = -span; oz <= span; oz++) {
                        const int cx = (ci[0] + ox + ncell) % ncell, cy = (ci[1] + oy + ncell) % ncell,
                                  cz = (ci[2] + oz + ncell) % ncell;
                        const int c = ncell >= 3 ? (cx * ncell + cy) * ncell + cz : 0;
                        const int b = ncell >= 3 ? v.start[c] : 0;
                        const int e = ncell >= 3 ? v.start[c + 1] : v.start[nc3];
                        for (int j = b + lane; j < e; j += 32) {
                            if (j == self) continue;
                            double dx = v.sx[j] - px, dy = v.sy[j] - py, dz = v.sz[j] - pz;
                            if (dx > 0.5 * L) dx -= L; else if (dx < -0.5 * L) dx += L;
                            if (dy > 0.5 * L) dy -= L; else if (dy < -0.5 * L) dy += L;
                            if (dz > 0.5 * L) dz -= L; else if (dz < -0.5 * L) dz += L;
                            const double r2 = dx * dx + dy * dy + dz * dz;
                            if (r2 >= rmax2) continue;
                            const double dr = sqrt(r2);
                            double ir3 = dr < eps ? soft3 : mass / (dr * dr * dr);
                            const double u = 0.5 * dr / rs;
                            ir3 *= erfc(u) + coeff * u * exp(-u * u);
                            ax += dx * ir3;
                            ay += dy * ir3;
                            az += dz * ir3;
                        }
                    }
        }
        ax = warp_sum_d(ax);
        ay = warp_sum_d(ay);
        az = warp_sum_d(az);
        if (lane == 0) {
            out[3 * (size_t)t] = ax;
            out[3 * (size_t)t + 1] = ay;
            out[3 * (size_t)t + 2] = az;
        }
    }
}

std::mutex g_na_mutex;
unsigned char *g_na_ptr[NA_MAX_DEVICES];  // device address of g_direct_scratch, per device
CUcontext g_na_ctx[NA_MAX_DEVICES];       // the context that address belongs to

// the current thread's CUDA context, through the runtime's driver entry
// point (the library does not link the driver library itself)
CUcontext na_current_context()
{
    typedef CUresult (*GetCurrent)(CUcontext *);
    static GetCurrent fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (GetCurrent)f;
        cudaGetLastError();
    });
    CUcontext ctx = nullptr;
    if (fn) fn(&ctx);
    return ctx;
}

// device address of the scratch on the current device, looked up once per
// device and context
int na_scratch(unsigned char **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ph_set_cuda_error(e, "cudaGetDevice", __FILE__, __LINE__);
    if (dev < 0 || dev >= NA_MAX_DEVICES)
        return ph_set_error(PH_ERR_UNSUPPORTED, "device %d beyond the %d devices the no-allocation scratch tracks", dev,
                            NA_MAX_DEVICES);
    const CUcontext ctx = na_current_context();  // null before the runtime has set up this thread's context
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev] || !ctx || ctx != g_na_ctx[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_direct_scratch);
        if (e != cudaSuccess) return ph_set_cuda_error(e, "cudaGetSymbolAddress(no-allocation scratch)", __FILE__, __LINE__);
        g_na_ptr[dev] = (unsigned char *)ptr;
        g_na_ctx[dev] = na_current_context();
    }
    *out = g_na_ptr[dev];
    return 0;
}

// device memory (or managed memory) that the current device can use directly
bool na_device_pointer(const void *ptr, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" int photons_direct_sum_noalloc(const photons_params *p, int n, const double *pos, int nt, const int *targets,
                                          double rmax, double *acc, void *cuda_stream)
{
    photons_gpu_clear_error();
    if (!p || n < 1 || nt < 0 || !pos || (nt > 0 && (!targets || !acc)) || !(rmax > 0) || !(p->boxsize > 0))
        return ph_set_error(PH_ERR_ARG, "bad no-allocation direct-sum arguments");
    if (n > NA_MAX_SOURCES)
        return ph_set_error(PH_ERR_ARG, "no-allocation direct sum: %d sources exceed the maximum %d", n, NA_MAX_SOURCES);
    if (nt > NA_MAX_TARGETS)
        return ph_set_error(PH_ERR_ARG, "no-allocation direct sum: %d targets exceed the maximum %d", nt, NA_MAX_TARGETS);
    unsigned char *s = nullptr;
    if (int rc = na_scratch(&s)) return rc;  // with nt = 0 the call is the warm-up: set-up only
    if (nt == 0) return 0;
    int dev = -1;
    cudaGetDevice(&dev);
    if (!na_device_pointer(pos, dev) || !na_device_pointer(targets, dev) || !na_device_pointer(acc, dev))
        return ph_set_error(PH_ERR_ARG, "no-allocation direct sum: pos, targets and acc must be device pointers "
                                        "on the current device (%d)", dev);

    const double L = p->boxsize;
    int ncell = (int)(L / rmax);
    if (ncell > NA_MAX_CELL_SIDE) ncell = NA_MAX_CELL_SIDE;
    if (ncell < 3) ncell = 1;
    const double cw = L / ncell;
    const int nc3 = ncell * ncell * ncell;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    const int blocks = ph::device_sm_count() * 8;

    ph::note_launch(), k_na_clear<<<blocks, 256, 0, st>>>(s, nc3);
    ph::note_launch(), k_na_count<<<blocks, 256, 0, st>>>(s, pos, n, ncell, cw);
    ph::note_launch(), k_na_scan<<<1, 1024, 0, st>>>(s, nc3);
    ph::note_launch(), k_na_place<<<blocks, 256, 0, st>>>(s, pos, n, ncell, cw);
    ph::note_launch(), k_na_targets<<<blocks, 256, 0, st>>>(s, pos, n, targets, nt);
    ph::note_launch(), k_na_direct<<<blocks, 256, 0, st>>>(s, ncell, cw, nt, L, rmax * rmax, p->eps, p->mass, p->rs, acc);
    cudaError_t e = cudaGetLastError();
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, s + NA_OFF_FLAG, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return ph_set_cuda_error(e, "no-allocation direct sum", __FILE__, __LINE__);
    if (flag) return ph_set_error(PH_ERR_ARG, "no-allocation direct sum: target index out of range [0, %d)", n);
    return 0;
}
