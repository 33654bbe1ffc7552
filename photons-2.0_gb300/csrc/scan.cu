// Device-wide exclusive scan with the element count held in device memory,
// so the launches do not depend on host-side sizes (tree levels and
// interaction counts are only known on the device).
//
// Three phases over tiles of SCAN_TILE elements: per-tile sums, a
// single-block scan of the tile sums, and per-tile scans with the tile
// offsets added.  Deterministic (integer arithmetic, fixed order).
#include "fmm_internal.cuh"

#define SCAN_THREADS 256
#define SCAN_ITEMS 8
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)

namespace {

__device__ __forceinline__ int block_excl_scan(int v, int *smem_warp, int &total)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = warp_incl_scan(v);
    if (lane == 31) smem_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < SCAN_THREADS / 32) ? smem_warp[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) smem_warp[lane] = wi - w;
        if (lane == SCAN_THREADS / 32 - 1) smem_warp[SCAN_THREADS / 32] = wi;
    }
    __syncthreads();
    int r = incl - v + smem_warp[wid];
    total = smem_warp[SCAN_THREADS / 32];
    __syncthreads();
    return r;
}

__global__ void k_tile_sums(const int *__restrict__ in, const int *n_ptr, int *__restrict__ tile_sum)
{
    __shared__ int sw[SCAN_THREADS / 32 + 1];
    int n = *n_ptr;
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int base = t * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
        int s = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            int idx = base + i;
            s += (idx < n) ? in[idx] : 0;
        }
        int total;
        block_excl_scan(s, sw, total);
        if (threadIdx.x == 0) tile_sum[t] = total;
    }
}

__global__ void k_scan_tile_sums(int *tile_sum, const int *n_ptr, int *total_out)
{
    __shared__ int sw[SCAN_THREADS / 32 + 1];
    int n = *n_ptr;
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    int carry = 0;
    for (int base = 0; base < ntiles; base += SCAN_THREADS) {
        int idx = base + threadIdx.x;
        int v = (idx < ntiles) ? tile_sum[idx] : 0;
        int total;
        int ex = block_excl_scan(v, sw, total);
        if (idx < ntiles) tile_sum[idx] = ex + carry;
        carry += total;
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

__global__ void k_tile_scan(const int *__restrict__ in, int *__restrict__ out, const int *n_ptr,
                            const int *__restrict__ tile_off)
{
    __shared__ int sw[SCAN_THREADS / 32 + 1];
    int n = *n_ptr;
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int base = t * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        int s = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            int idx = base + i;
            v[i] = (idx < n) ? in[idx] : 0;
            s += v[i];
        }
        int total;
        int ex = block_excl_scan(s, sw, total) + tile_off[t];
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            int idx = base + i;
            if (idx < n) out[idx] = ex;
            ex += v[i];
        }
    }
}

}  // namespace

namespace ph {

size_t scan_scratch_elems(int cap) { return (size_t)(cap + SCAN_TILE - 1) / SCAN_TILE + 1; }

void scan_exclusive_i32(const int *in, int *out, const int *n_ptr, int cap, int *total, int *scratch,
                        size_t scratch_elems, cudaStream_t st)
{
    (void)scratch_elems;
    int ntiles_cap = (cap + SCAN_TILE - 1) / SCAN_TILE;
    int grid = ntiles_cap < 4 * device_sm_count() ? (ntiles_cap > 0 ? ntiles_cap : 1) : 4 * device_sm_count();
    ph::note_launch(), k_tile_sums<<<grid, SCAN_THREADS, 0, st>>>(in, n_ptr, scratch);
    ph::note_launch(), k_scan_tile_sums<<<1, SCAN_THREADS, 0, st>>>(scratch, n_ptr, total);
    ph::note_launch(), k_tile_scan<<<grid, SCAN_THREADS, 0, st>>>(in, out, n_ptr, scratch);
}

}  // namespace ph
