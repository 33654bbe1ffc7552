/*
 * CPU restatement of the photoNs-2.0 FMM short-range force pass.
 * TEST INFRASTRUCTURE ONLY (the oracle): used by tests/, by
 * __graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline
 * leg.  The product never links it.
 *
 * Pinned against the reference sources compiled in place
 * (oracle/_ref/libphotons_ref.so) and the fixtures in tests/golden/.
 */
#ifndef PHOTONS_ORACLE_H
#define PHOTONS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define PO_NMULTI 20

typedef struct {
    double boxsize;   /* periodic box side (BOXSIZE) */
    double theta;     /* opening angle (open_angle) */
    double rs;        /* split radius (splitRadius) */
    double rcut;      /* cutoff radius (cutoffRadius) */
    double eps;       /* softening length (SoftenScale) */
    double mass;      /* particle mass (MASSPART) */
    int maxleaf;      /* MAXLEAF */
    int nthreads;     /* compute threads (>=1) */
    int capture;      /* keep the interaction lists for inspection */
    int images;       /* 1: 26 periodic images (PERIODIC_CONDITION), 0: none */
} po_params;

enum { PO_LIST_P2P = 0, PO_LIST_M2L = 1, PO_LIST_P2P_EXT = 2, PO_LIST_M2L_EXT = 3 };

enum {
    PO_OK = 0,
    PO_ERR_ARG = 1,
    PO_ERR_NOMEM = 2,
    PO_ERR_LEAF_CAPACITY = 3,   /* more leaves than 2N/MAXLEAF (reference writes past its array) */
    PO_ERR_NODE_CAPACITY = 4,
    PO_ERR_SMALL = 5            /* N <= MAXLEAF: the reference's image walk reads undefined memory */
};

typedef struct po_state po_state;

po_state *po_create(void);
void po_destroy(po_state *s);

/* One force pass.  Returns PO_OK or an error code; *seconds = wall time. */
int po_run(po_state *s, const po_params *p, int n, const double *pos_in, double *seconds);

/* The same pass with forces formed only for the particles targets[0..nt)
   (input indices): tree, walks, counters and multipoles are complete; the
   targets' accelerations are identical to the full pass's.  acc_out: nt*3;
   times[4]: tree build, multipoles, walks, sampled forces (seconds). */
int po_run_sample(po_state *s, const po_params *p, int n, const double *pos_in, int nt, const int *targets,
                  double *acc_out, double *times);
/* forces for another set of targets on the tree and lists of the last
   po_run_sample (or po_run), without rebuilding them; *seconds = wall time */
int po_forces_sample(po_state *s, int nt, const int *targets, double *acc_out, double *seconds);
/* pairs of the last pass's local and image P2P lists as the reference
   evaluates them (n_t n_s per task, minus a leaf's self pairs) */
void po_pairs(const po_state *s, long long *pairs_local, long long *pairs_image);

/* The reference's first domain decomposition at P ranks (src/domains.c:
   400-459, src/toptree.c:157-182): box[6 r..] = rank r's domain (lo, hi),
   axis[r] = its local tree's first split axis, split[P-1] = the domain
   tree's split planes (heap order). */
int po_domains(int P, double boxsize, double *box, int *axis, double *split);
/* One pass over P ranks emulated in this process (each rank's tree over its
   domain; other ranks' and periodic trees exported, pruned and walked as
   src/remotes.c:60-751 does).  acc_out[3n] in input order, counters[16 P]
   per rank, rank_out[n] each particle's rank; explicit_self sends a rank's
   own periodic images through the export too. */
int po_run_domains(int P, const po_params *p, int n, const double *pos_in, int explicit_self, double *acc_out,
                   long long *counters, int *rank_out);
/* fmm_prepare of one rank's domain (lo, hi: its top-tree box; axis: first split) */
int po_prepare_domain(po_state *s, const po_params *p, const double lo[3], const double hi[3], int axis, int n,
                      const double *pos_in);
/* the exported tree of the last pass (RemoteNode layout: int npart, son[2];
   double width[3], center[3], M[20]; bodies as x, y, z), pruned against the
   receiving root's centre and width; with nodes/bodies NULL only the sizes */
int po_export(const po_state *s, const double recv_center[3], const double recv_width[3], const double shift[3],
              int *nnode, int *nbody, int node_cap, int body_cap, void *nodes, double *bodies);

/* a received tree (po_export's layout), kept for po_finish_domain */
int po_import(po_state *s, int nnode, const void *nodes, int nbody, const double *bodies);
/* the prepared domain's pass over the received trees: acc_out[3n] in the
   prepared positions' order */
int po_finish_domain(po_state *s, double *acc_out);

/* counters[16]: idxP2P, idxM2L, walk_m2l_count, p2p_count_remote, NLEAF, NNODE,
   nleaf, nnode, first_leaf, first_node, direct_local_start(0), n_p2p, n_m2l,
   n_p2p_ext, n_m2l_ext, n_images, in the reference's index space. */
void po_counters(const po_state *s, long long *counters);
/* tree-ordered positions, accelerations after the local task phase and after
   the full pass, and perm[i] = input index of the particle at position i. */
void po_particles(const po_state *s, double *pos, double *acc_task, double *acc, int *perm);
long po_list_size(const po_state *s, int kind);
void po_list_copy(const po_state *s, int kind, int *target, int *source, int *image);
void po_copy_leaves(const po_state *s, int *ip_np, double *geom, double *M, double *L);
void po_copy_nodes(const po_state *s, int *info, double *geom, double *M, double *L);

/* scalar operators with the reference's conventions (operator.c) */
void po_p2m(int npart, const double *pos, double mass, const double center[3], double *M);
void po_m2m(double dx, double dy, double dz, const double *M, double *toM);
void po_m2l(double dx, double dy, double dz, const double *M, double *toL, double rs);
void po_l2l(double dx, double dy, double dz, const double *L, double *toL);
void po_l2p(int npart, const double *pos, const double center[3], const double *L, double *acc);
int po_acceptance(const double wi[3], const double wj[3], const double dist[3], double theta, double rcut);

/* FP64 direct sum of the untruncated split kernel, minimum image, over all
   sources within rmax of each listed target.  acc_out: nt*3. */
int po_direct_sum(const po_params *p, int n, const double *pos, int nt, const int *targets,
                  double rmax, double *acc_out);

/* time integration (src/photoNs.c:141-196, 257-268; src/initial.c:639-683):
   the kick and drift factors over [loga_i, loga_f], and the kick / drift
   updates of m = 3n coordinates (drift wraps into [0, L)) */
double po_kick_loga(double omega_m, double omega_x, double loga_i, double loga_f);
double po_drift_loga(double omega_m, double omega_x, double loga_i, double loga_f);
void po_kick(long long m, double *vel, const double *acc, double dkh);
void po_drift(long long m, double *pos, const double *vel, double dd, double L);

#ifdef __cplusplus
}
#endif
#endif
