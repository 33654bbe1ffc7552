/*
 * The reference's data layouts and globals, as its headers define them
 * (inc/typesdef.h:25-57, inc/photoNs.h:170-189, 260-272).  The drop-in entry
 * points exchange data with the reference driver through exactly these
 * names and layouts, so they must be alike; this header restates them for
 * the library's own compilation.  NMULTI = 20 (OCTUPOLE, inc/typesdef.h:11).
 */
#ifndef PHOTONS_REF_ABI_H
#define PHOTONS_REF_ABI_H

#define REF_NMULTI 20
#define REF_NSON 2

typedef unsigned long REF_INT64;

typedef struct {
    int updated;
    int npart;
    int son[REF_NSON];
    double split;
    double width[3];
    double center[3];
    double M[REF_NMULTI];
    double L[REF_NMULTI];
} Node;

typedef struct {
    int npart;
    int ipart;
    double width[3];
    double center[3];
    double M[REF_NMULTI];
    double L[REF_NMULTI];
} Pack;

typedef struct {
    double pos[3];
    double acc[3];
    double vel[3];
    double acc_pm[3];
} Body;

typedef struct {
    int son[REF_NSON];
    double split;
    double M[REF_NMULTI];
    double center[3];
    double width[3];
} TopNode;

#ifdef __cplusplus
extern "C" {
#endif
/* globals read or written by the FMM entry points */
extern Body *part;
extern Node *btree;
extern Pack *leaf;
extern TopNode *toptree;
extern double open_angle;
extern int first_node, last_node, first_leaf, last_leaf, MAXLEAF;
extern int PROC_RANK, PROC_SIZE;
extern double BOXSIZE;
extern int NPART, NLEAF, NNODE;
extern long NPART_TOTAL;
extern double MASSPART, SoftenScale, cutoffRadius, splitRadius;
extern int first_domain, last_domain, this_domain, mostleft, direct_local_start;
extern double width_this_domain;
extern int *ExtDomain;
extern REF_INT64 idxP2P, idxM2L, walk_m2l_count, p2p_count_remote, m2l_count;
extern double dtime_p2p, dtime_m2l, dtime_fmm, dtime_task, dtime_ext, dtime_prep, dtime_fmm_remote;
extern double DTIME_THIS_DOMAIN;
#ifdef __cplusplus
}
#endif

#endif
