/*
 * Harness around the reference photoNs-2.0 FMM sources, compiled in place
 * (src/fmm.c, src/operator.c, src/remotes.c, src/toptree.c,
 * src/domains.c, src/utility.c) into oracle/_ref/libphotons_ref.so by
 * oracle/Makefile.  TEST INFRASTRUCTURE ONLY: it is the checker that pins
 * the CPU restatement (oracle/photons_oracle.c) and generates the golden
 * fixtures; nothing in the product links it.
 *
 * What it does:
 *   - sets the reference's globals for a single rank the way
 *     src/initial.c:199-220 (setup_domain_index) and
 *     src/initial.c:316-345 (derived force parameters) would;
 *   - runs the reference's own driver sequence for one force pass
 *     (src/photoNs.c:83-116): domain_initialize, fmm_construct,
 *     fmm_prepare, fmm_task, fmm_ext;
 *   - captures every interaction list.  The reference sources are
 *     compiled with -Dpthread_create=oracle_pthread_create (and join), so
 *     each hand-off of a task batch to the compute thread
 *     (src/fmm.c:381-404, 543-565, 932-963; src/remotes.c:189-210,
 *     376-401, 642-670) arrives here.  At that moment the globals ts/tt
 *     (src/fmm.c:372-373) or ts_ex/tt_ex (src/remotes.c:179-180) point at
 *     the batch and argt[1] holds its length.  The batch is recorded and
 *     the worker is then run (synchronously when capturing, on a real
 *     thread otherwise).
 *   - maps image-tree indices back to local tree indices: the image tree
 *     is the preorder export of src/remotes.c:60-169, so exrtree node 0
 *     is first_node and an internal exported node's son[] indices pair up
 *     with the local node's son[] (leaves carry body ranges instead).
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include "photoNs.h"
#include "fmm.h"
#include "domains.h"

/* globals defined (non-static) by the reference sources */
extern int *ts, *tt, argt[2];
extern int *ts_ex, *tt_ex, argt_ex[2];
void *task_compute_p2p(void *);
void *task_compute_m2l(void *);
void *task_compute_p2p_ext(void *);
void *task_compute_m2l_ext(void *);

enum { K_P2P = 0, K_M2L = 1, K_P2P_EXT = 2, K_M2L_EXT = 3, NKIND = 4 };

typedef struct { int *t, *s, *img; long n, cap; } list_t;
static list_t lists[NKIND];
static int capture_on = 0;
static int image_index = -1;          /* advanced on every tree self-receive (tag 111) */
static int *ext_map = 0;              /* exrtree index -> local id, for the current image */
static long ext_map_cap = 0;

static void list_push(list_t *l, int t, int s, int img)
{
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 1 << 16;
        l->t = realloc(l->t, sizeof(int) * l->cap);
        l->s = realloc(l->s, sizeof(int) * l->cap);
        l->img = realloc(l->img, sizeof(int) * l->cap);
        if (!l->t || !l->s || !l->img) { fprintf(stderr, "harness: out of memory\n"); exit(5); }
    }
    l->t[l->n] = t; l->s[l->n] = s; l->img[l->n] = img; l->n++;
}

/* exported-tree index -> local id (leaf or node id in the reference's index space) */
static void map_ext(int e, int local)
{
    ext_map[e] = local;
    if (local < first_node) return;                 /* leaf: son[] hold body ranges */
    if (exrtree[e].son[0] < 0 || exrtree[e].son[1] < 0) return;   /* pruned by the sender */
    map_ext(exrtree[e].son[0], btree[local].son[0]);
    map_ext(exrtree[e].son[1], btree[local].son[1]);
}

static void recv_hook(int tag, void *buf, int count)
{
    (void)buf;
    if (tag != 111) return;
    image_index++;
    if (!capture_on) return;
    if (count > ext_map_cap) {
        ext_map_cap = count;
        ext_map = realloc(ext_map, sizeof(int) * ext_map_cap);
    }
    for (int i = 0; i < count; i++) ext_map[i] = -1;
    map_ext(0, first_node);
}

int oracle_pthread_create(pthread_t *tid, const pthread_attr_t *attr, void *(*fn)(void *), void *arg)
{
    if (capture_on) {
        int nt = ((int *)arg)[1];
        int kind;
        int *s, *t;
        if (fn == task_compute_p2p) { kind = K_P2P; s = ts; t = tt; }
        else if (fn == task_compute_m2l) { kind = K_M2L; s = ts; t = tt; }
        else if (fn == task_compute_p2p_ext) { kind = K_P2P_EXT; s = ts_ex; t = tt_ex; }
        else if (fn == task_compute_m2l_ext) { kind = K_M2L_EXT; s = ts_ex; t = tt_ex; }
        else { fprintf(stderr, "harness: unknown worker\n"); exit(5); }
        for (int n = 0; n < nt; n++) {
            int src = s[n];
            int img = 0;
            if (kind >= K_P2P_EXT) { img = image_index + 1; src = ext_map[src]; }
            list_push(&lists[kind], t[n], src, img);
        }
        fn(arg);
        *tid = (pthread_t)0;
        return 0;
    }
    return pthread_create(tid, attr, fn, arg);
}

int oracle_pthread_join(pthread_t tid, void **ret)
{
    if (capture_on) { if (ret) *ret = 0; return 0; }
    return pthread_join(tid, ret);
}

static double wall(void)
{
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

static int have_tree = 0;

/*
 * One force pass of the reference on npart particles (pos: npart*3 doubles).
 * Outputs are in the reference's tree order (it permutes part[] in place,
 * src/fmm.c:30-78): pos_out, acc_task_out (after fmm_task: local P2P + local
 * M2L, no L2L/L2P yet), acc_out (after fmm_ext).  counters[16]: see body.
 * Returns the wall time of fmm_construct..fmm_ext in seconds.
 */
double ref_run(int npart, const double *pos, double boxsize, int maxleaf, double theta,
               double rs, double rcut, double eps, double mass, int capture,
               double *pos_out, double *acc_task_out, double *acc_out, long long *counters)
{
    if (have_tree) { fmm_deconstruct(); domain_finalize(); have_tree = 0; }
    if (part) { free(part); part = 0; }

    for (int k = 0; k < NKIND; k++) lists[k].n = 0;
    capture_on = capture;
    image_index = -1;
    oracle_mpi_recv_hook = recv_hook;

    /* message types as src/initial.c:234-244 creates them */
    MPI_Type_contiguous(sizeof(MKey), MPI_CHAR, &strMKey);
    MPI_Type_contiguous(sizeof(RemoteNode), MPI_CHAR, &strReNode);
    MPI_Type_contiguous(sizeof(RemoteBody), MPI_CHAR, &strReBody);
    MPI_Type_contiguous(sizeof(Body), MPI_CHAR, &strBody);

    PROC_SIZE = 1; PROC_RANK = 0;
    mostleft = 0; this_domain = 0; first_domain = 0; last_domain = 0;
    NPART = npart; NPART_TOTAL = npart;
    BOXSIZE = boxsize; MAXLEAF = maxleaf; open_angle = theta;
    splitRadius = rs; cutoffRadius = rcut; SoftenScale = eps; MASSPART = mass;
    idxP2P = idxM2L = 0; walk_m2l_count = 0; p2p_count_remote = 0;

    part = (Body *)calloc((size_t)npart, sizeof(Body));
    for (int n = 0; n < npart; n++) {
        part[n].pos[0] = pos[3 * n + 0];
        part[n].pos[1] = pos[3 * n + 1];
        part[n].pos[2] = pos[3 * n + 2];
    }

    double t0 = wall();
    domain_initialize();
    fmm_construct();
    fmm_prepare();
    fmm_task();
    double t1 = wall();
    if (acc_task_out)
        for (int n = 0; n < npart; n++)
            for (int d = 0; d < 3; d++) acc_task_out[3 * n + d] = part[n].acc[d];
    double t2 = wall();
    fmm_ext();
    double t3 = wall();
    have_tree = 1;

    for (int n = 0; n < npart; n++)
        for (int d = 0; d < 3; d++) {
            if (pos_out) pos_out[3 * n + d] = part[n].pos[d];
            if (acc_out) acc_out[3 * n + d] = part[n].acc[d];
        }
    if (counters) {
        counters[0] = (long long)idxP2P;
        counters[1] = (long long)idxM2L;
        counters[2] = (long long)walk_m2l_count;
        counters[3] = (long long)p2p_count_remote;
        counters[4] = NLEAF;
        counters[5] = NNODE;
        counters[6] = last_leaf - first_leaf;
        counters[7] = last_node - first_node + 1;
        counters[8] = first_leaf;
        counters[9] = first_node;
        counters[10] = direct_local_start;
        counters[11] = lists[K_P2P].n;
        counters[12] = lists[K_M2L].n;
        counters[13] = lists[K_P2P_EXT].n;
        counters[14] = lists[K_M2L_EXT].n;
        counters[15] = image_index + 1;
    }
    capture_on = 0;
    return (t1 - t0) + (t3 - t2);
}

long ref_list_size(int kind) { return (kind >= 0 && kind < NKIND) ? lists[kind].n : -1; }

void ref_list_copy(int kind, int *t, int *s, int *img)
{
    list_t *l = &lists[kind];
    memcpy(t, l->t, sizeof(int) * l->n);
    memcpy(s, l->s, sizeof(int) * l->n);
    memcpy(img, l->img, sizeof(int) * l->n);
}

/* leaves: ipart,npart (int32 x2 per leaf), center/width (3+3 doubles), M/L (NMULTI each) */
void ref_copy_leaves(int *ip_np, double *geom, double *M, double *L)
{
    int nl = last_leaf - first_leaf;
    for (int i = 0; i < nl; i++) {
        Pack *p = &leaf[first_leaf + i];
        ip_np[2 * i] = p->ipart; ip_np[2 * i + 1] = p->npart;
        for (int d = 0; d < 3; d++) { geom[6 * i + d] = p->center[d]; geom[6 * i + 3 + d] = p->width[d]; }
        for (int m = 0; m < NMULTI; m++) { M[NMULTI * i + m] = p->M[m]; L[NMULTI * i + m] = p->L[m]; }
    }
}

/* nodes: npart, son0, son1 (int32 x3), split, center, width (7 doubles), M/L */
void ref_copy_nodes(int *info, double *geom, double *M, double *L)
{
    int nn = last_node - first_node + 1;
    for (int i = 0; i < nn; i++) {
        Node *p = &btree[first_node + i];
        info[3 * i] = p->npart; info[3 * i + 1] = p->son[0]; info[3 * i + 2] = p->son[1];
        geom[7 * i] = p->split;
        for (int d = 0; d < 3; d++) { geom[7 * i + 1 + d] = p->center[d]; geom[7 * i + 4 + d] = p->width[d]; }
        for (int m = 0; m < NMULTI; m++) { M[NMULTI * i + m] = p->M[m]; L[NMULTI * i + m] = p->L[m]; }
    }
}

/* The reference's scalar operators and MAC, for operator-level fixtures. */
void ref_m2l(double dx, double dy, double dz, double *M, double *L, double rs)
{
    splitRadius = rs;
    m2l(dx, dy, dz, M, L);
}
void ref_m2m(double dx, double dy, double dz, double *M, double *tM) { m2m(dx, dy, dz, M, tM); }
void ref_l2l(double dx, double dy, double dz, double *L, double *tL) { l2l(dx, dy, dz, L, tL); }
int ref_acceptance(double *wi, double *wj, double *dist, double theta, double rcut)
{
    open_angle = theta; cutoffRadius = rcut;
    return acceptance(wi, wj, dist);
}

/* The reference's time integrals (src/initial.c:639-683) read OmegaM0 and
   OmegaX0; initial.c and snapshot.c are compiled in only for them.  The
   2DECOMP&FFT call of initialize_nbody is never reached here. */
double kick_loga(double loga_i, double loga_f);
double drift_loga(double loga_i, double loga_f);
void get_local_size_(void) {}

double ref_kick_loga(double omega_m, double omega_x, double loga_i, double loga_f)
{
    OmegaM0 = omega_m;
    OmegaX0 = omega_x;
    return kick_loga(loga_i, loga_f);
}

double ref_drift_loga(double omega_m, double omega_x, double loga_i, double loga_f)
{
    OmegaM0 = omega_m;
    OmegaX0 = omega_x;
    return drift_loga(loga_i, loga_f);
}

/* Gadget-2 snapshots through the reference's own readers
   (src/snapshot.c:64-118, 209-293): header values and particles [0, n). */
void read_GadgetHeader(const char filename[]);
void read_Particle_Gadget2(char filename[], int n_start, int n_count);

void ref_gadget_header(const char *path, double *out)
{
    read_GadgetHeader(path);
    out[0] = BOXSIZE;
    out[1] = (double)NPART_TOTAL;
    out[2] = MASSPART;
    out[3] = OmegaM0;
    out[4] = OmegaX0;
    out[5] = Hubble0;
    out[6] = InitialTime;
}

void ref_gadget_read(const char *path, int n, double *pos, double *vel)
{
    Body *saved = part;
    part = (Body *)calloc((size_t)n, sizeof(Body));
    read_Particle_Gadget2((char *)path, 0, n);
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            pos[3 * i + d] = part[i].pos[d];
            vel[3 * i + d] = part[i].vel[d];
        }
    free(part);
    part = saved;
}

/*
 * The reference's PM at one rank: src/partmesh.c:18-795 (partmesh_thread,
 * the branch its Makefile builds with -DPMTHREAD -DMYALLTOALLV) on the
 * reference's globals, with the pencil decomposition of one rank and an
 * nside^3 mesh set up as src/initial.c:453-493 would (local start 0, end
 * nside - 1 as get_local_size returns them, size nside), and the Fortran
 * convolution replaced by oracle/pm_conv.c.  acc_pm[3n] out.
 */
void partmesh_thread(void);
extern MPI_Comm PM_COMM_WORLD;  /* inc/photoNs.h:311-313, declared under PMTHREAD */
void ref_pm_force(int npart, const double *pos, double boxsize, int nside, double rs, double mass, double *acc_pm)
{
    static int msize0, msize1;
    Body *saved = part;
    int saved_n = NPART;
    part = (Body *)calloc((size_t)npart, sizeof(Body));
    for (int n = 0; n < npart; n++)
        for (int d = 0; d < 3; d++) part[n].pos[d] = pos[3 * n + d];
    MPI_Type_contiguous(sizeof(MKey), MPI_CHAR, &strMKey);
    PM_COMM_WORLD = MPI_COMM_WORLD;
    PROC_SIZE = 1; PROC_RANK = 0;
    NPART = npart; BOXSIZE = boxsize; NSIDE = nside; splitRadius = rs; MASSPART = mass;
    vproc[0] = vproc[1] = 1;
    pside[0] = pside[1] = nside;
    for (int d = 0; d < 3; d++) {
        local_xstart[d] = 0;
        local_xend[d] = nside - 1;
        local_xsize[d] = nside;
    }
    data_length = (long)nside * nside * nside;
    msize0 = msize1 = nside - 1;  /* MPI_Allgather of local_xend[1], local_xend[2] over one rank */
    MSIZE0 = &msize0;
    MSIZE1 = &msize1;
    partmesh_thread();
    for (int n = 0; n < npart; n++)
        for (int d = 0; d < 3; d++) acc_pm[3 * n + d] = part[n].acc_pm[d];
    free(part);
    part = saved;
    NPART = saved_n;
}
