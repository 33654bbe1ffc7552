// Device-wide exclusive scan with the element count held in device memory,
// so the launches do not depend on host-side sizes (tree levels and
// interaction counts are only known on the device).
//
// Three phases over tiles of SCAN_TILE elements: per-tile sums, a
// single-block scan of the tile sums, and per-tile scans with the tile
// offsets added; counts known to stay small run in one block instead.
// Deterministic (integer arithmetic, fixed order).
#include "fmm_internal.cuh"

#define SCAN_THREADS 256
#define SCAN_ITEMS 8
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)

namespace {

template <typename T>
__device__ __forceinline__ T warp_incl_scan_t(T v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

template <typename T, int NT = SCAN_THREADS>
__device__ __forceinline__ T block_excl_scan(T v, T *smem_warp, T &total)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T incl = warp_incl_scan_t(v);
    if (lane == 31) smem_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T w = (lane < NT / 32) ? smem_warp[lane] : T(0);
        T wi = warp_incl_scan_t(w);
        if (lane < NT / 32) smem_warp[lane] = wi - w;
        if (lane == NT / 32 - 1) smem_warp[NT / 32] = wi;
    }
    __syncthreads();
    T r = incl - v + smem_warp[wid];
    total = smem_warp[NT / 32];
    __syncthreads();
    return r;
}

// The whole scan in one block of 1,024 threads, for counts of at most
// SCAN_ONE_BLOCK_MAX: one launch instead of three (a tree level's node
// scans are a few thousand elements, bound by launches, not bandwidth)
#define SCAN_ONE_THREADS 1024
#define SCAN_ONE_ITEMS 16
#define SCAN_ONE_BLOCK_MAX (1 << 16)

template <typename T>
__global__ void __launch_bounds__(SCAN_ONE_THREADS) k_scan_one_block(const T *__restrict__ in, T *__restrict__ out,
                                                                     const int *n_ptr, T *total_out)
{
    __shared__ T sw[SCAN_ONE_THREADS / 32 + 1];
    const int n = *n_ptr;
    T carry = 0;
    for (int base = 0; base < n; base += SCAN_ONE_THREADS * SCAN_ONE_ITEMS) {
        const int i0 = base + threadIdx.x * SCAN_ONE_ITEMS;
        T v[SCAN_ONE_ITEMS];
        T s = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ONE_ITEMS; i++) {
            v[i] = (i0 + i < n) ? in[i0 + i] : T(0);
            s += v[i];
        }
        T total;
        T ex = block_excl_scan<T, SCAN_ONE_THREADS>(s, sw, total) + carry;
#pragma unroll
        for (int i = 0; i < SCAN_ONE_ITEMS; i++) {
            if (i0 + i < n) out[i0 + i] = ex;
            ex += v[i];
        }
        carry += total;
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

template <typename T>
__global__ void k_tile_sums(const T *__restrict__ in, const int *n_ptr, T *__restrict__ tile_sum)
{
    __shared__ T sw[SCAN_THREADS / 32 + 1];
    int n = *n_ptr;
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int base = t * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
        T s = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            int idx = base + i;
            s += (idx < n) ? in[idx] : T(0);
        }
        T total;
        block_excl_scan(s, sw, total);
        if (threadIdx.x == 0) tile_sum[t] = total;
    }
}

template <typename T>
__global__ void k_scan_tile_sums(T *tile_sum, const int *n_ptr, T *total_out)
{
    __shared__ T sw[SCAN_THREADS / 32 + 1];
    int n = *n_ptr;
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    T carry = 0;
    for (int base = 0; base < ntiles; base += SCAN_THREADS) {
        int idx = base + threadIdx.x;
        T v = (idx < ntiles) ? tile_sum[idx] : T(0);
        T total;
        T ex = block_excl_scan(v, sw, total);
        if (idx < ntiles) tile_sum[idx] = ex + carry;
        carry += total;
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

template <typename T>
__global__ void k_tile_scan(const T *__restrict__ in, T *__restrict__ out, const int *n_ptr,
                            const T *__restrict__ tile_off)
{
    __shared__ T sw[SCAN_THREADS / 32 + 1];
    int n = *n_ptr;
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int base = t * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
        T v[SCAN_ITEMS];
        T s = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            int idx = base + i;
            v[i] = (idx < n) ? in[idx] : T(0);
            s += v[i];
        }
        T total;
        T ex = block_excl_scan(s, sw, total) + tile_off[t];
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            int idx = base + i;
            if (idx < n) out[idx] = ex;
            ex += v[i];
        }
    }
}

template <typename T>
void scan_exclusive(const T *in, T *out, const int *n_ptr, int cap, T *total, T *scratch, cudaStream_t st)
{
    if (cap <= SCAN_ONE_BLOCK_MAX) {
        ph::note_launch(), k_scan_one_block<T><<<1, SCAN_ONE_THREADS, 0, st>>>(in, out, n_ptr, total);
        return;
    }
    int ntiles_cap = (cap + SCAN_TILE - 1) / SCAN_TILE;
    int grid = ntiles_cap < 4 * ph::device_sm_count() ? (ntiles_cap > 0 ? ntiles_cap : 1) : 4 * ph::device_sm_count();
    ph::note_launch(), k_tile_sums<T><<<grid, SCAN_THREADS, 0, st>>>(in, n_ptr, scratch);
    ph::note_launch(), k_scan_tile_sums<T><<<1, SCAN_THREADS, 0, st>>>(scratch, n_ptr, total);
    ph::note_launch(), k_tile_scan<T><<<grid, SCAN_THREADS, 0, st>>>(in, out, n_ptr, scratch);
}

}  // namespace

namespace ph {

size_t scan_scratch_elems(int cap) { return (size_t)(cap + SCAN_TILE - 1) / SCAN_TILE + 1; }

void scan_exclusive_i32(const int *in, int *out, const int *n_ptr, int cap, int *total, int *scratch,
                        size_t scratch_elems, cudaStream_t st)
{
    (void)scratch_elems;
    scan_exclusive<int>(in, out, n_ptr, cap, total, scratch, st);
}

void scan_exclusive_i32_bounded(const int *in, int *out, const int *n_ptr, int cap, int nmax, int *total,
                                int *scratch, size_t scratch_elems, cudaStream_t st)
{
    (void)scratch_elems;
    scan_exclusive<int>(in, out, n_ptr, nmax < cap ? nmax : cap, total, scratch, st);
}

void scan_exclusive_i64(const long long *in, long long *out, const int *n_ptr, int cap, long long *total,
                        long long *scratch, cudaStream_t st)
{
    scan_exclusive<long long>(in, out, n_ptr, cap, total, scratch, st);
}

}  // namespace ph
