// Internal definitions shared by the force-pass translation units.
//
// Index spaces on the device:
//   particles  [0, N)       in tree order after the build (perm[] maps back)
//   leaves     [0, NL)      numbered as src/fmm.c:101-118 numbers them
//   nodes      [0, NN)      preorder, as src/fmm.c:111-114 numbers them
//   unified id u: u < NL is leaf u, otherwise node u - NL.
// The reference's own index space (leaves from N, nodes from N+NLEAF,
// src/fmm.c:211-212) is used only at the C-ABI boundary.
#pragma once
#include <atomic>

#include <cuda_runtime.h>
#include <stdint.h>

#define PH_NMULTI 20
#define PH_NIMG 27
// image tag of entries whose source lies in a received tree (another
// rank's exported tree, possibly shifted by a periodic image): the received
// centres already carry the sender's shift
#define PH_IMG_IMPORT 27

// interaction entry: unified source id (27 bits) | image index (5 bits)
#define PH_ENTRY(u, img) ((uint32_t)(u) | ((uint32_t)(img) << 27))
#define PH_ENTRY_ID(e) ((int)((e) & 0x07FFFFFFu))
#define PH_ENTRY_IMG(e) ((int)((e) >> 27))
#define PH_MAX_UNIFIED (1 << 27)
// largest leaf the P2P kernels stage (shared-memory stage of 128 FP64 sources)
#define PH_MAX_LEAF 128

// child encoding inside the build: >= 0 node, < 0 leaf (~leaf)
#define PH_IS_LEAF_CODE(c) ((c) < 0)

// error bits reported by kernels through Work::flags
#define PH_FLAG_STACK_OVERFLOW 1u
#define PH_FLAG_STAGE_OVERFLOW 2u
#define PH_FLAG_POOL_OVERFLOW 4u
#define PH_FLAG_LEAF_CAPACITY 8u
#define PH_FLAG_NODE_CAPACITY 16u
#define PH_FLAG_DEPTH 32u
#define PH_FLAG_TOP 64u  // wide nodes left after the launched levels of the tree build

struct PassParams {
    double boxsize, theta, rs, rcut, eps, mass;
    int maxleaf;
    int images;  // unused by the kernels; the walk takes an image mask
    int axis0;   // the first split axis (direct_local_start; 0 but for a rank's domain tree)
};

// One periodic box of a pass.  A pass covers one box or many independent
// boxes (their particles concatenated, one tree root each); every kernel
// reads the constants of the box its target belongs to from this table.
struct BoxParams {
    double boxsize, rs, rcut, eps, mass;
    double rcut2;       // rcut^2
    double acc_scale;   // packed FP32 P2P: m sig^2
    float Lhi, Llo;     // box side as an FP32 pair
    float c2f;          // rcut^2 in FP32 (walk filter)
    float sig, e2s, pias, cs;  // packed FP32 P2P: coordinate scale, eps'^2, p ia / sig, (2/sqrt(pi)) ia / sig
    float far_a, far_pa;       // FP32 M2L: ia = 1/(2 rs) and p ia
    int first, count;   // particle range in the concatenated input
    int root;           // unified id of the box's root node (written by the build)
    int domain;         // 1: the root's box is dom_lo..dom_hi (a rank's domain), else [0, boxsize]^3
    double dom_lo[3], dom_hi[3];
};

// ------------------------------------------------------------------
// device helpers
// ------------------------------------------------------------------
__device__ __forceinline__ int warp_lane() { return threadIdx.x & 31; }

template <typename T>
__device__ __forceinline__ T shfl(T v, int src) { return __shfl_sync(0xffffffffu, v, src); }

__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// inclusive warp scan of ints
__device__ __forceinline__ int warp_incl_scan(int v)
{
    int lane = warp_lane();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ long long warp_sum_ll(long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// fixed-order (deterministic) warp sum of doubles: xor butterfly
__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// image shift for image index img (1..26) in the loop order of
// src/fmm.c:1029-1044 (mi, mj, mk from -1 to 1, skipping 0,0,0); img 0 = none
__host__ __device__ __forceinline__ void image_offsets(int img, int &mi, int &mj, int &mk)
{
    if (img == 0 || img >= PH_NIMG) { mi = mj = mk = 0; return; }
    int c = img - 1;
    if (c >= 13) c += 1;  // skip the centre cell (index 13 of the 27)
    mi = c / 9 - 1;
    mj = (c / 3) % 3 - 1;
    mk = c % 3 - 1;
}

// ------------------------------------------------------------------
// host helpers shared by the translation units
// ------------------------------------------------------------------
namespace ph {

int device_sm_count();

// number of kernels this library has launched (reported by photons_launch_count)
// kernels launched by this library (photons_launch_count).  Host threads
// (the PM thread beside the force pass) add to it concurrently; a thread
// that is capturing a graph counts into its own tally instead, and the
// graph's kernels are added each time the graph is launched.
extern std::atomic<unsigned long long> g_launches;
extern thread_local unsigned long long *t_capture_tally;
inline void note_launch()
{
    if (t_capture_tally) ++*t_capture_tally;
    else g_launches.fetch_add(1, std::memory_order_relaxed);
}

// exclusive scan of n int32 values (n read on the device from n_ptr, at most
// cap elements); writes total to *total (device) if total != nullptr.
void scan_exclusive_i32(const int *in, int *out, const int *n_ptr, int cap, int *total, int *scratch,
                        size_t scratch_elems, cudaStream_t st);
// the same for a count the host knows is at most nmax (<= cap): counts of
// at most 65,536 are scanned in one block, one launch
void scan_exclusive_i32_bounded(const int *in, int *out, const int *n_ptr, int cap, int nmax, int *total,
                                int *scratch, size_t scratch_elems, cudaStream_t st);
size_t scan_scratch_elems(int cap);
// the same over 64-bit values; scratch holds scan_scratch_elems(cap) values
void scan_exclusive_i64(const long long *in, long long *out, const int *n_ptr, int cap, long long *total,
                        long long *scratch, cudaStream_t st);

}  // namespace ph

#define PH_CUDA_CHECK(call)                                                                   \
    do {                                                                                      \
        cudaError_t e__ = (call);                                                             \
        if (e__ != cudaSuccess) return ph_set_cuda_error(e__, #call, __FILE__, __LINE__);     \
    } while (0)

int ph_set_cuda_error(cudaError_t e, const char *what, const char *file, int line);
int ph_set_error(int code, const char *fmt, ...);
