/*
 * photoNs-2.0 FMM short-range force pass on one GB300 GPU: C ABI.
 *
 * Two layers:
 *
 *  1. The reference's own entry points, unchanged names and signatures, so
 *     the reference driver (src/photoNs.c) links this library in place of
 *     src/fmm.c, src/operator.c and src/remotes.c.  They communicate
 *     through the reference's globals (part, NPART, MAXLEAF, open_angle,
 *     splitRadius, cutoffRadius, SoftenScale, MASSPART, BOXSIZE, toptree,
 *     btree, leaf, ...), which this library also defines so that it can be
 *     loaded on its own.  Like the reference they print a message and exit
 *     on a fatal error; photons_gpu_status()/photons_gpu_error() report the
 *     last error without exiting.
 *
 *  2. photons_* extensions: a context-based pass on plain arrays (the call
 *     benchmarks and tests use), inspection of the tree and lists, batched
 *     operators, an FP64 direct-sum reference, and timing.
 *
 * Only one rank is supported (the reference's single-GPU case); with
 * PROC_SIZE > 1 the legacy entry points fail.
 */
#ifndef PHOTONS_FMM_H
#define PHOTONS_FMM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* 1. reference entry points                                           */
/* ------------------------------------------------------------------ */

/* inc/fmm.h:16 -- top-tree geometry of the domain (src/fmm.c:329-360) */
void fmm_construct(void);
/* inc/fmm.h:19 -- tree build, multipoles, top-tree connect (src/fmm.c:719-770);
   permutes part[] into tree order and fills btree/leaf like the reference */
void fmm_prepare(void);
/* inc/fmm.h:20 -- local P2P and M2L lists and their evaluation (src/fmm.c:909-984) */
void fmm_task(void);
/* inc/fmm.h:21 -- 26 periodic images, L2L and L2P (src/fmm.c:987-1075) */
void fmm_ext(void);
/* inc/fmm.h:17 -- release the tree (src/fmm.c:1077-1087) */
void fmm_deconstruct(void);
/* inc/fmm.h:10 -- tree build only (src/fmm.c:180-264) */
void build_localtree(void);

/* inc/operator.h:6-19 -- operators on host data, FP64 (src/operator.c) */
void p2m(int iPart, int npart, double center[3], double M[]);
void m2m(double dx, double dy, double dz, double M[], double tM[]);
void m2l(double dx, double dy, double dz, double M[], double toL[]);
void l2l(double dx, double dy, double dz, double L[], double toL[]);
void l2p(int ileaf);
void walk_m2m(int iNode);
void walk_l2l(int inode);

/* inc/photoNs.h:325 -- MAC (src/fmm.c:266-326) */
int acceptance(double wi[3], double wj[3], double dist[3]);

/* inc/remotes.h:16 -- interactions with one shifted copy of the local tree
   (src/remotes.c:684-751); at one rank idx must be 0 */
void fmm_remote(int idx, double shift[3]);

/* inc/kernels.h:4-8 -- one local P2P task on the GPU in FP64: the particles
   of leaf inode from those of leaf jnode (reference leaf ids, after
   fmm_prepare), added to part[].acc as src/fmm.c:823-868 adds a task.  The
   reference declares these but never defines them.  p2p_kernel evaluates
   the pair force as src/fmm.c:834-852 writes it; p2p_kernel_rinvsqrt the
   same force with 1/r from the reciprocal square root and the split
   factor erfc(u) + (2/sqrt(pi)) u exp(-u^2) from piecewise polynomials
   (within 5.3e-17 of it), the FP64 pass's form;
   p2p_kernel_inleaf a leaf with itself (jnode == inode), self pairs skipped. */
void p2p_kernel(int inode, int jnode);
void p2p_kernel_rinvsqrt(int inode, int jnode);
void p2p_kernel_inleaf(int inode, int jnode);

/* inc/partmesh.h:16-17, 22 -- the PM long-range force at one rank, on the
   GPU (src/partmesh.c:18-795 in the -DPMTHREAD build, :800-1582 without):
   part[].acc_pm from part[].pos on an NSIDE^3 mesh with splitRadius,
   BOXSIZE and MASSPART.  pm_thread is the entry of the driver's PM thread
   (src/partmesh.c:11-16, src/photoNs.c:104); the PM uses a GPU context of
   its own, so it runs beside the FMM calls of the driver's main thread. */
void partmesh_thread(void);
void partmesh(void);
void *pm_thread(void *arg);
/* src/conv.f90:3-23, called as decomp_2d_init by src/initial.c:226, 468: the
   pencil of one rank is the whole mesh (0-based start and end) */
void get_local_size_(int *global_size, int *vproc, int *local_start, int *local_end, int *local_size);

/* ------------------------------------------------------------------ */
/* 2. extensions                                                       */
/* ------------------------------------------------------------------ */

/* last error of the calling thread: 0 = none */
int photons_gpu_status(void);
const char *photons_gpu_error(void);
void photons_gpu_clear_error(void);

typedef struct photons_params {
    double boxsize;  /* periodic box side (BOXSIZE) */
    double theta;    /* opening angle (open_angle) */
    double rs;       /* split radius (splitRadius) */
    double rcut;     /* cutoff radius (cutoffRadius) */
    double eps;      /* softening length (SoftenScale) */
    double mass;     /* particle mass (MASSPART) */
    int maxleaf;     /* MAXLEAF */
    int precision;   /* PHOTONS_FP32_SPLIT or PHOTONS_FP64 */
    unsigned image_mask; /* bit 0: local tree, bit k (1..26): image k; 0 means all */
    int flags;       /* PHOTONS_F_* */
} photons_params;

#define PHOTONS_FP32_SPLIT 0
#define PHOTONS_FP64 1

/* flags */
#define PHOTONS_F_DEVICE_IO 1       /* pos/acc pointers are device memory */
#define PHOTONS_F_TREE_ORDER 2      /* acc returned in tree order (see photons_get_perm) */
#define PHOTONS_F_NO_FARFIELD 4     /* skip P2M/M2M/M2L/L2L/L2P */
#define PHOTONS_F_MULTIPOLES 8      /* compute P2M/M2M even when no M2L task exists */
#define PHOTONS_F_KEEP_LISTS 16     /* keep lists for photons_list_* */
#define PHOTONS_F_ONE_WAY 32        /* FP32: every pair one way (no mutual pairs, no reaction slots) */
#define PHOTONS_F_P2P_BULK 64      /* FP32 mutual kernel: source leaves staged by TMA bulk copies */
/* FP32 mutual P2P kernel build (bits 8-11): 0 the default (build 2); 1
   three blocks per SM, two dependency chains; 2 four blocks, one chain,
   6-target path; 3 three blocks, one chain; 4 four blocks, two chains.  The
   builds give the same forces to FP32 rounding, either source staging
   (PHOTONS_F_P2P_BULK) the same bits; the autotuner times them. */
#define PHOTONS_F_P2P_SHAPE(s) ((s) << 8)
#define PHOTONS_F_SHAPE_OF(f) (((f) >> 8) & 15)
#define PHOTONS_P2P_SHAPES 5

typedef struct photons_ctx photons_ctx;

photons_ctx *photons_create(int device);
void photons_destroy(photons_ctx *ctx);
/* launch on this cudaStream_t (NULL: the context's own stream) */
int photons_set_stream(photons_ctx *ctx, void *cuda_stream);

/* One force pass over n particles: pos[3n] in, acc[3n] out (overwritten).
   Host or device pointers per PHOTONS_F_DEVICE_IO. */
int photons_force_pass(photons_ctx *ctx, const photons_params *p, int n, const double *pos, double *acc);

/* One pass over nbox independent periodic boxes in one launch per operator:
   box b holds counts[b] particles, stored after those of boxes 0..b-1 in
   pos[3 sum(counts)] (acc likewise).  params[b] gives each box's side, rs,
   rcut, softening and mass; theta, maxleaf, precision, image_mask and flags
   must be the same in every entry.  Each box is its own tree and periodic
   domain (one root per box; images shift by that box's side), so the
   result equals nbox separate passes.  No counterpart in the reference,
   which evaluates one domain per rank. */
int photons_force_pass_boxes(photons_ctx *ctx, int nbox, const photons_params *params, const int *counts,
                             const double *pos, double *acc);

/* counters[32] after a pass: idxP2P, idxM2L, walk_m2l_count, p2p_count_remote,
   NLEAF, NNODE, nleaf, nnode, first_leaf, first_node, direct_local_start,
   n_p2p, n_m2l, n_p2p_ext, n_m2l_ext, n_images, local pairs, image pairs,
   depth, max stack, max stage, pd peak, p2p entries, m2l entries */
int photons_get_counters(photons_ctx *ctx, long long *counters, int n);
/* milliseconds of the last pass: total, upload, tree, walk, p2p, farfield, download */
int photons_get_timings(photons_ctx *ctx, float *ms, int n);
/* tree-order -> input index */
int photons_get_perm(photons_ctx *ctx, int *perm);
/* tree-order positions */
int photons_get_positions(photons_ctx *ctx, double *pos);

/* the tree in the reference's layout and index space:
   leaves: ip_np[2*nleaf], geom[6*nleaf] (centre, width), M/L[20*nleaf];
   nodes: info[3*nnode] (npart, son0, son1), geom[7*nnode] (split, centre, width), M/L */
int photons_copy_leaves(photons_ctx *ctx, int *ip_np, double *geom, double *M, double *L);
int photons_copy_nodes(photons_ctx *ctx, int *info, double *geom, double *M, double *L);

/* lists of the last pass (PHOTONS_F_KEEP_LISTS), reference index space;
   kind 0 local P2P, 1 local M2L, 2 image P2P, 3 image M2L */
long long photons_list_size(photons_ctx *ctx, int kind);
int photons_list_copy(photons_ctx *ctx, int kind, int *target, int *source, int *image);

/* batched operators on host arrays, evaluated on the GPU:
   op 0: L[i] += M2L(d[i], M[i]) with split radius rs
   op 1: out[i] += M2M(d[i], in[i]);  op 2: out[i] += L2L(d[i], in[i]) */
int photons_op_batch(int op, int n, const double *d, const double *in, double *inout, double rs);

/* FP64 direct sum of the untruncated split kernel over all sources within
   rmax (minimum image) for nt targets (input indices); host arrays */
int photons_direct_sum(const photons_params *p, int n, const double *pos, int nt, const int *targets,
                       double rmax, double *acc);

/* The same FP64 direct sum, allocating nothing (no cudaMalloc, cudaFree or
   allocating library call).  It has no counterpart in the reference.  It is
   for callers that cannot allocate device memory mid-run: a run that has
   budgeted all of HBM up front (particles, PM mesh, force-pass pools), where
   a cudaMalloc between steps fails, or whose other streams must not be
   stalled by the device-wide synchronisation of cudaMalloc/cudaFree.
   pos[3n], targets[nt] and acc[3nt] are DEVICE pointers on the current
   device (host pointers and other devices' buffers are rejected).  At most
   262144 sources and 65536 targets; larger sizes return error 1 with a
   message.  Scratch is one fixed array of about 10.8 MB per device.  The
   library's device code is loaded lazily, so that array is placed in device
   memory by the first call on a device, which also looks up its address
   (with the device current; again after the device's context is replaced):
   make that first call before HBM is budgeted and before any stream
   capture.  A call with nt = 0 does only this set-up (a warm-up; nothing is
   launched).  From then on the array stays until the process exits.  All
   calls share it, so calls that overlap on the GPU (other streams or host
   threads) race.  Runs on cuda_stream (NULL: the default stream) and
   returns after that stream has finished the call's work. */
int photons_direct_sum_noalloc(const photons_params *p, int n, const double *pos, int nt, const int *targets,
                               double rmax, double *acc, void *cuda_stream);

/* ---- several ranks, one GPU each: the reference's domain decomposition
   (src/domains.c, src/toptree.c) and its locally essential trees
   (src/remotes.c:60-169, 684-751).  Each rank builds its tree over its own
   domain, exports for every other rank (and for every periodic image) its
   tree shifted and pruned against the receiver's domain, and walks its tree
   against the trees it receives.  The transport between ranks is the
   caller's (MPI, NCCL or torch.distributed); the library builds and uses
   the messages, in the reference's RemoteNode / RemoteBody layouts. ---- */
/* inc/photoNs.h:177-183 (RemoteNode): a node of an exported tree; son[] are
   the children's indices in the same array, -1 where the sender pruned
   them, and for a leaf (npart <= MAXLEAF) the range of its bodies */
typedef struct {
    int npart;
    int son[2];
    double width[3];
    double center[3];
    double M[20];
} photons_remote_node;
/* inc/photoNs.h:185-189 (RemoteBody): a body of an exported leaf, shifted */
typedef struct {
    double pos[3];
    double replenish;
} photons_remote_body;
/* a rank's domain: its box (the split planes around it) and the axis its
   local tree splits first (direct_local_start) */
typedef struct {
    double lo[3], hi[3];
    int axis;
} photons_domain;

/* The first decomposition of the periodic box over nrank ranks, equal work
   per rank (src/domains.c:400-459, src/toptree.c:157-182, domain ids of
   src/initial.c:197-222): domains[r] for every rank; split[nrank-1] the
   domain tree's split planes in heap order (may be NULL).  Host function. */
int photons_domain_split(int nrank, double boxsize, photons_domain *domains, double *split);
/* rank[i] of each position pos[3i] under split planes split[nrank-1]
   (src/domains.c:263-298: above a plane goes to the upper side).  Host. */
int photons_domain_assign(int nrank, const double *split, int n, const double *pos, int *rank);
/* Load balance (src/domains.c:22-156): moves the split planes by the
   measured work time of each rank, relaxed as the reference relaxes them,
   and writes the new domains (may be NULL).  Host function. */
int photons_domain_rebalance(int nrank, double boxsize, double *split, const double *rank_time,
                             photons_domain *domains);
/* Start this rank's pass (src/fmm.c:719-770 for a domain): the tree of the
   n positions of this rank's domain, built over the domain box from its
   first axis, and its multipoles.  Host or device positions per
   PHOTONS_F_DEVICE_IO; they must stay valid until photons_domain_finish. */
int photons_domain_prepare(photons_ctx *ctx, const photons_params *p, const photons_domain *dom, int n,
                           const double *pos);
/* The tree prepared in ctx shifted by shift[3] and pruned against the
   receiving rank's domain (src/remotes.c:60-169), in depth-first preorder.
   Host buffers; *nnode and *nbody receive the sizes.  With nodes and bodies
   NULL only the sizes; if node_cap or body_cap is too small nothing is
   written and error 4 (capacity) is returned with the sizes set. */
int photons_let_export(photons_ctx *ctx, const photons_domain *receiver, const double shift[3],
                       photons_remote_node *nodes, int node_cap, photons_remote_body *bodies, int body_cap,
                       int *nnode, int *nbody);
/* A tree received from another rank (or this rank's own, shifted), kept
   for photons_domain_finish; host buffers, copied.  Checked: child and body
   indices must lie in the message. */
int photons_let_import(photons_ctx *ctx, const photons_remote_node *nodes, int nnode,
                       const photons_remote_body *bodies, int nbody);
/* Finish the pass (src/fmm.c:909-1075 with fmm_remote over the received
   trees): local walk, the 26 periodic images of the local tree, the walks
   against every received tree (P2P with its bodies, M2L with its pruned
   nodes), L2L, L2P; acc[3n] in the prepared positions' order (host or
   device as prepared).  Counters and lists as photons_force_pass leaves
   them; the image counters include the received trees. */
int photons_domain_finish(photons_ctx *ctx, double *acc);

/* ---- kick-drift-kick integration on device arrays (src/photoNs.c:141-196,
   257-268).  Products and sums are rounded separately, as in the reference's
   loops, so a step matches it bit for bit given the same accelerations. ---- */
/* the reference's kick and drift factors: Simpson's rule over 128 intervals
   of log a (src/initial.c:639-683); omega_m, omega_x stand for its OmegaM0
   and OmegaX0 globals.  Host functions. */
double photons_kick_loga(double omega_m, double omega_x, double loga_i, double loga_f);
double photons_drift_loga(double omega_m, double omega_x, double loga_i, double loga_f);
/* vel[3n] += acc[3n] * dkh (src/photoNs.c:164-174); device arrays, 16-byte
   aligned; enqueued on cuda_stream (NULL: default stream) */
int photons_kick(int n, double *vel, const double *acc, double dkh, void *cuda_stream);
/* pos[3n] += vel[3n] * dd, each coordinate then wrapped into [0, boxsize)
   as src/photoNs.c:176-196 does; enqueued on cuda_stream */
int photons_drift(int n, double *pos, const double *vel, double dd, double boxsize, void *cuda_stream);
/* one step on device arrays: kick with acc, drift, force pass into acc (the
   short-range force; PHOTONS_F_DEVICE_IO implied), kick with the new acc.
   dkh = kick factor x G / 2, dd = drift factor.  Returns after the step. */
int photons_kdk_step(photons_ctx *ctx, const photons_params *p, int n, double *pos, double *vel, double *acc,
                     double dkh, double dd);

/* ---- PM long-range force (src/partmesh.c:18-800 at one rank, the
   convolution of src/conv.f90:128-247): CIC deposit of the particle mass on
   an nside^3 periodic mesh, FFT, the long-range Green's function
   exp(-k^2 rs^2)/k^2 with the CIC window deconvolved, inverse FFT, 4-point
   gradient and CIC interpolation: acc_pm[3n] (G-free, like the short-range
   acc).  Uses boxsize, rs and mass of p; host or device pointers per
   PHOTONS_F_DEVICE_IO.  Returns after the work is done. ---- */
int photons_pm_force(photons_ctx *ctx, const photons_params *p, int nside, int n, const double *pos, double *acc_pm);

/* ---- Gadget-2 snapshots (the reference's SnapFormat 2, src/snapshot.c:5-22,
   64-293, 397-549): header block, FP32 position and velocity blocks.  Host
   functions. ---- */
typedef struct photons_gadget_header {
    int npart[6];
    double mass[6];
    double time, redshift;
    int flag_sfr, flag_feedback;
    int npart_total[6];
    int flag_cooling, num_files;
    double boxsize, omega0, omega_lambda, hubble;
} photons_gadget_header;
int photons_gadget_read_header(const char *path, photons_gadget_header *h);
/* particles [first, first+count) of the file (species in order) as FP64:
   pos[3 count]; vel[3 count] (may be NULL) multiplied by (1/(1+z))^1.5 as
   src/snapshot.c:163-181 does */
int photons_gadget_read(const char *path, long long first, long long count, double *pos, double *vel);
/* one file of n particles (positions and velocities rounded to FP32,
   velocities divided by (1/(1+z))^1.5 as src/snapshot.c:470-481) */
int photons_gadget_write(const char *path, const photons_gadget_header *h, long long n, const double *pos,
                         const double *vel);

/* the reference's whole step with both halves of the force, on device
   arrays: kick with acc_pm then acc, drift and wrap, short-range pass into
   acc and PM (nside^3 mesh) into acc_pm, kick with acc then acc_pm
   (src/photoNs.c:158-196, 229-268) */
int photons_kdk_step_pm(photons_ctx *ctx, const photons_params *p, int nside, int n, double *pos, double *vel,
                        double *acc, double *acc_pm, double dkh, double dd);

/* the two steps above with the particle state kept in tree order, as the
   reference's driver keeps part[] (src/fmm.c:30-78): after the short-range
   pass pos, vel and ids (optional, may be NULL; the caller's particle
   identities) are permuted into the pass's tree order and acc (and acc_pm)
   come back in it, so the next step's build starts from nearly sorted
   particles.  No counterpart function in the reference; device arrays. */
int photons_kdk_step_ordered(photons_ctx *ctx, const photons_params *p, int n, double *pos, double *vel, double *acc,
                             long long *ids, double dkh, double dd);
int photons_kdk_step_pm_ordered(photons_ctx *ctx, const photons_params *p, int nside, int n, double *pos,
                                double *vel, double *acc, double *acc_pm, long long *ids, double dkh, double dd);

/* kernels launched by this library so far (all contexts) */
unsigned long long photons_launch_count(void);

/* pinned host memory for the host-buffer pass: the pass's kernels read and
   write it over the host link (so do they any pinned memory the device
   addresses); NULL and an error message if it cannot be had */
void *photons_host_alloc(size_t bytes);
void photons_host_free(void *p);

/* FP32 FMA throughput probes: TFLOP/s of FFMA chains, and of the paired
   (float2) FFMA of sm_100+; ~iters x 128 FMAs per thread */
double photons_fp32_fma_peak(int iters);
double photons_fp32x2_fma_peak(int iters);
/* the FP64 one (DFMA chains), the denominator of the FP64 pass's roofline */
double photons_fp64_fma_peak(int iters);
/* the FP64 kernels' split factor erfc(u) + (2/sqrt(pi)) u exp(-u^2) at n
   host points u >= 0, evaluated on the device: their piecewise polynomials,
   or with exact != 0 erfc and exp as src/fmm.c:846-848 writes them (a check
   of the polynomials); 0 or an error code */
int photons_split_factor_fp64(const double *u, int n, int exact, double *g);

#ifdef __cplusplus
}
#endif
#endif
