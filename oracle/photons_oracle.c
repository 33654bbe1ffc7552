/*
 * CPU restatement of the photoNs-2.0 FMM short-range force pass (the oracle).
 * TEST INFRASTRUCTURE ONLY -- see photons_oracle.h.
 *
 * Every step follows the reference's algorithm; each function names the
 * reference lines it restates.  Traversals visit pairs in the reference's
 * depth-first order and per-particle sums are formed in the reference's
 * order, so on the reference's own inputs this oracle reproduces its tree,
 * its interaction lists (same order) and, where no M2L occurs, its
 * accelerations bit for bit.  The multipole operators are written here in
 * multi-index form (the same Cartesian Taylor expansions as
 * src/operator.c, summed in a different order), so results that involve
 * M2L/L2L/L2P agree to rounding.
 *
 * Index space (src/fmm.c:200-212): particles [0,N), leaves
 * [N, N+NLEAF), nodes [N+NLEAF, N+NLEAF+NNODE).
 */
#define _GNU_SOURCE
#include "photons_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#define NM PO_NMULTI
#define NIMG 27

/* ------------------------------------------------------------------ */
/* multi-index tables for the order-3 Cartesian expansions             */
/* ------------------------------------------------------------------ */
/* Component order of inc/operator.h:24-60: 1, x, y, z, xx, xy, xz, yy, yz,
   zz, xxx, xxy, xxz, xyy, xyz, xzz, yyy, yyz, yzz, zzz -- graded, and inside
   a grade ordered by descending x then descending y exponent. */
static int mi_exp[NM][3];
static int mi_index[4][4][4];
static double mi_invfact[NM];    /* 1/(a! b! c!) */
static int mi_order[NM];
static int tables_ready = 0;

static void init_tables(void)
{
    if (tables_ready) return;
    static const double fact[4] = {1, 1, 2, 6};
    int i = 0;
    for (int k = 0; k <= 3; k++)
        for (int a = k; a >= 0; a--)
            for (int b = k - a; b >= 0; b--) {
                int c = k - a - b;
                mi_exp[i][0] = a; mi_exp[i][1] = b; mi_exp[i][2] = c;
                mi_index[a][b][c] = i;
                mi_invfact[i] = 1.0 / (fact[a] * fact[b] * fact[c]);
                mi_order[i] = k;
                i++;
            }
    tables_ready = 1;
}

/* d^g / g! for every multi-index g with |g| <= 3 */
static void scaled_monomials(double dx, double dy, double dz, double *out)
{
    double px[4] = {1, dx, dx * dx, dx * dx * dx};
    double py[4] = {1, dy, dy * dy, dy * dy * dy};
    double pz[4] = {1, dz, dz * dz, dz * dz * dz};
    for (int i = 0; i < NM; i++)
        out[i] = px[mi_exp[i][0]] * py[mi_exp[i][1]] * pz[mi_exp[i][2]] * mi_invfact[i];
}

/* P2M, src/operator.c:13-93: M_a = sum_p m (-(x_p - c))^a / a! */
void po_p2m(int npart, const double *pos, double mass, const double center[3], double *M)
{
    init_tables();
    double mono[NM];
    for (int i = 0; i < NM; i++) M[i] = 0.0;
    for (int p = 0; p < npart; p++) {
        scaled_monomials(-(pos[3 * p] - center[0]), -(pos[3 * p + 1] - center[1]),
                         -(pos[3 * p + 2] - center[2]), mono);
        for (int i = 0; i < NM; i++) M[i] += mass * mono[i];
    }
}

/* M2M, src/operator.c:96-160 (d = parent centre - child centre):
   toM_a += sum_{b <= a} M_b d^(a-b)/(a-b)! */
void po_m2m(double dx, double dy, double dz, const double *M, double *toM)
{
    init_tables();
    double mono[NM], out[NM];
    scaled_monomials(dx, dy, dz, mono);
    for (int a = 0; a < NM; a++) {
        double s = 0.0;
        for (int b = 0; b < NM; b++) {
            int g0 = mi_exp[a][0] - mi_exp[b][0], g1 = mi_exp[a][1] - mi_exp[b][1],
                g2 = mi_exp[a][2] - mi_exp[b][2];
            if (g0 < 0 || g1 < 0 || g2 < 0) continue;
            s += M[b] * mono[mi_index[g0][g1][g2]];
        }
        out[a] = s;
    }
    for (int a = 0; a < NM; a++) toM[a] += out[a];
}

/*
 * Radial derivative factors f_k = ((1/r) d/dr)^k phi of the short-range
 * Green's function phi(r) = erfc(r / (2 rs)) / r (the LONGSHORT branch of
 * src/operator.c:294-307).  With a = 1/(2 rs), E = exp(-a^2 r^2),
 * c = 2/sqrt(pi):
 *   f0 = erfc/r
 *   f1 = -erfc/r^3 - c a E/r^2
 *   f2 = 3 erfc/r^5 + 3 c a E/r^4 + 2 c a^3 E/r^2
 *   f3 = -15 erfc/r^7 - 15 c a E/r^6 - 10 c a^3 E/r^4 - 4 c a^5 E/r^2
 */
static void split_factors(double r, double rs, double f[4])
{
    double a = 0.5 / rs;
    double u = a * r;
    double ce = (2.0 / sqrt(M_PI)) * exp(-u * u);
    double er = erfc(u);
    double ir = 1.0 / r, ir2 = ir * ir;
    double a2 = a * a;
    f[0] = er * ir;
    f[1] = -er * ir * ir2 - ce * a * ir2;
    f[2] = 3.0 * er * ir * ir2 * ir2 + ce * (3.0 * a * ir2 * ir2 + 2.0 * a * a2 * ir2);
    f[3] = -15.0 * er * ir * ir2 * ir2 * ir2 - ce * (15.0 * a * ir2 * ir2 * ir2 + 10.0 * a * a2 * ir2 * ir2 +
                                                    4.0 * a * a2 * a2 * ir2);
}

/* derivative tensor D_g = d^g phi(x), |g| <= 3, from the radial factors:
   D_g = f_|g| x^g + f_(|g|-1) sum_i C(g_i,2) x^(g - 2 e_i) */
static void derivative_tensor(double dx, double dy, double dz, const double f[4], double *D)
{
    double x[3] = {dx, dy, dz};
    for (int g = 0; g < NM; g++) {
        int e0 = mi_exp[g][0], e1 = mi_exp[g][1], e2 = mi_exp[g][2];
        int k = mi_order[g];
        double mono = 1.0;
        for (int i = 0; i < e0; i++) mono *= x[0];
        for (int i = 0; i < e1; i++) mono *= x[1];
        for (int i = 0; i < e2; i++) mono *= x[2];
        double v = f[k] * mono;
        if (k >= 2) {
            int e[3] = {e0, e1, e2};
            for (int d = 0; d < 3; d++) {
                if (e[d] < 2) continue;
                double m2 = (double)(e[d] * (e[d] - 1) / 2);
                double rest = 1.0;
                for (int dd = 0; dd < 3; dd++) {
                    int p = e[dd] - (dd == d ? 2 : 0);
                    for (int i = 0; i < p; i++) rest *= x[dd];
                }
                v += f[k - 1] * m2 * rest;
            }
        }
        D[g] = v;
    }
}

/* M2L, src/operator.c:255-392 (d = target centre - source centre):
   toL_b += sum_{|a| <= 3-|b|} M_a D_(a+b) */
void po_m2l(double dx, double dy, double dz, const double *M, double *toL, double rs)
{
    init_tables();
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    double f[4], D[NM];
    split_factors(r, rs, f);
    derivative_tensor(dx, dy, dz, f, D);
    for (int b = 0; b < NM; b++) {
        double s = 0.0;
        for (int a = 0; a < NM; a++) {
            if (mi_order[a] + mi_order[b] > 3) continue;
            int i0 = mi_exp[a][0] + mi_exp[b][0], i1 = mi_exp[a][1] + mi_exp[b][1],
                i2 = mi_exp[a][2] + mi_exp[b][2];
            s += M[a] * D[mi_index[i0][i1][i2]];
        }
        toL[b] += s;
    }
}

/* L2L, src/operator.c:395-494 (d = child centre - parent centre):
   toL_b += sum_g L_(b+g) d^g/g!,  |b+g| <= 3 */
void po_l2l(double dx, double dy, double dz, const double *L, double *toL)
{
    init_tables();
    double mono[NM];
    scaled_monomials(dx, dy, dz, mono);
    for (int b = 0; b < NM; b++) {
        double s = 0.0;
        for (int g = 0; g < NM; g++) {
            if (mi_order[b] + mi_order[g] > 3) continue;
            int i0 = mi_exp[b][0] + mi_exp[g][0], i1 = mi_exp[b][1] + mi_exp[g][1],
                i2 = mi_exp[b][2] + mi_exp[g][2];
            s += L[mi_index[i0][i1][i2]] * mono[g];
        }
        toL[b] += s;
    }
}

/* L2P, src/operator.c:197-251: acc_i += sum_{|g|<=2} L_(e_i+g) d^g/g! */
void po_l2p(int npart, const double *pos, const double center[3], const double *L, double *acc)
{
    init_tables();
    double mono[NM];
    for (int p = 0; p < npart; p++) {
        scaled_monomials(pos[3 * p] - center[0], pos[3 * p + 1] - center[1], pos[3 * p + 2] - center[2], mono);
        for (int i = 0; i < 3; i++) {
            double s = 0.0;
            for (int g = 0; g < NM; g++) {
                if (mi_order[g] > 2) continue;
                int e[3] = {mi_exp[g][0], mi_exp[g][1], mi_exp[g][2]};
                e[i] += 1;
                s += L[mi_index[e[0]][e[1]][e[2]]] * mono[g];
            }
            acc[3 * p + i] += s;
        }
    }
}

/* MAC, src/fmm.c:266-326: 1 accept (M2L), 0 open, -1 drop (LONGSHORT). */
int po_acceptance(const double wi[3], const double wj[3], const double dist[3], double theta, double rcut)
{
    double w[3], gap[3];
    for (int d = 0; d < 3; d++) w[d] = (wi[d] + wj[d]) * 0.5;
    double dd2 = dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2];
    for (int d = 0; d < 3; d++) {
        gap[d] = fabs(dist[d]) - w[d];
        if (gap[d] <= 0.0) gap[d] = 0.0;
    }
    if (gap[0] + gap[1] + gap[2] < 0.0001) return 0;          /* touching boxes */
    double dm2 = gap[0] * gap[0] + gap[1] * gap[1] + gap[2] * gap[2];
    double c2 = rcut * rcut;
    if (dm2 >= c2) return -1;                                  /* beyond the cutoff */
    if (dd2 > c2) return 0;
    double wmax = w[0];
    if (w[1] > wmax) wmax = w[1];
    if (w[2] > wmax) wmax = w[2];
    wmax *= 2;
    return (wmax * wmax < theta * theta * dd2) ? 1 : 0;
}

/* ------------------------------------------------------------------ */
/* state                                                               */
/* ------------------------------------------------------------------ */
typedef struct { int npart, ipart; double width[3], center[3], M[NM], L[NM]; } o_leaf;
typedef struct { int npart, son[2]; double split, width[3], center[3], M[NM], L[NM]; } o_node;
typedef struct { int *t, *s, *img; long n, cap; } o_list;

struct po_state {
    po_params p;
    int n, nleaf_cap, nnode_cap, nleaf, nnode;
    int first_leaf, first_node;
    double *pos;      /* tree order, n*3 */
    int *perm;
    double *acc, *acc_task;
    o_leaf *leaf;
    o_node *node;
    o_list list[4];
    long long walk_m2l_count, p2p_count_remote;
    int err;
    int capture;
    /* sampled pass: forces only for these particles (tree order) and the
       leaves / nodes that hold them; NULL = every particle */
    unsigned char *part_on, *leaf_on, *node_on;    /* the domain this tree covers (src/fmm.c:189-197): the root's box and
       the first split axis (direct_local_start); the whole periodic box and
       axis 0 at one rank */
    int domain_set;
    double dom_lo[3], dom_hi[3];
    int axis0;
    /* trees received from other ranks (or from this one, shifted), walked
       as P2P/M2L "ext" lists with image tags PO_IMG_RECEIVED + k */
    struct o_rtree *rt;
    int nrt;
};

/* an exported (pruned, shifted) tree: src/remotes.c:60-169, the layout of
   RemoteNode (inc/photoNs.h:177-183); bodies as x, y, z */
typedef struct { int npart, son[2]; double width[3], center[3], M[NM]; } o_rnode;
typedef struct o_rtree { int nnode, nbody; o_rnode *node; double *body; } o_rtree;
#define PO_IMG_RECEIVED 100

/* One dual-tree traversal's output.  Walks are split into independent
   sub-walks (subtrees of the recursion) that run on separate threads and
   are concatenated in the order a sequential traversal would emit them. */
typedef struct { int kind, a, b; } o_item;   /* kind 0-3: list entry (t, s); 4: deferred sub-walk (im, jm) */
typedef struct {
    po_state *s;
    int image;              /* 0 local, 1..26 periodic image */
    double shift[3];
    o_list list[4];
    long long m2l;          /* contribution to walk_m2l_count */
    int err;
    int defer_depth;        /* >0: stop at this recursion depth and record the pair as an item */
    o_item *items;
    long nitems, capitems;
} o_walker;

po_state *po_create(void)
{
    init_tables();
    return (po_state *)calloc(1, sizeof(po_state));
}

static void free_run(po_state *s)
{
    free(s->pos); free(s->perm); free(s->acc); free(s->acc_task);
    free(s->leaf); free(s->node);
    free(s->part_on); free(s->leaf_on); free(s->node_on);
    s->pos = 0; s->perm = 0; s->acc = 0; s->acc_task = 0; s->leaf = 0; s->node = 0;
    s->part_on = 0; s->leaf_on = 0; s->node_on = 0;
}

void po_destroy(po_state *s)
{
    if (!s) return;
    for (int k = 0; k < s->nrt; k++) { free(s->rt[k].node); free(s->rt[k].body); }
    free(s->rt);
    free_run(s);
    for (int k = 0; k < 4; k++) { free(s->list[k].t); free(s->list[k].s); free(s->list[k].img); }
    free(s);
}

static int list_push(o_list *l, int t, int src, int img)
{
    if (l->n == l->cap) {
        long cap = l->cap ? 2 * l->cap : 1 << 10;
        int *a = realloc(l->t, sizeof(int) * cap), *b, *c;
        if (!a) return -1;
        l->t = a;
        b = realloc(l->s, sizeof(int) * cap);
        if (!b) return -1;
        l->s = b;
        c = realloc(l->img, sizeof(int) * cap);
        if (!c) return -1;
        l->img = c;
        l->cap = cap;
    }
    l->t[l->n] = t; l->s[l->n] = src; l->img[l->n] = img; l->n++;
    return 0;
}

#define IS_LEAF(S, id) ((id) < (S)->first_node)
#define LEAF(S, id) (&(S)->leaf[(id) - (S)->first_leaf])
#define NODE(S, id) (&(S)->node[(id) - (S)->first_node])

/* ------------------------------------------------------------------ */
/* kd-tree                                                             */
/* ------------------------------------------------------------------ */
static void swap_part(po_state *s, int i, int j)
{
    double t[3];
    memcpy(t, s->pos + 3 * i, sizeof t);
    memcpy(s->pos + 3 * i, s->pos + 3 * j, sizeof t);
    memcpy(s->pos + 3 * j, t, sizeof t);
    int q = s->perm[i]; s->perm[i] = s->perm[j]; s->perm[j] = q;
}

/*
 * Mean split of a segment along axis D, src/fmm.c:30-78.  Segments of
 * fewer than two particles go wholly to the upper side; a pair splits at
 * its midpoint, ordered.  Otherwise the mean is a sequential sum divided by
 * the count and the partition is the reference's two-ended swap: scanning
 * upward, each particle above the mean is exchanged with the next particle
 * (from the top) that is not above it; the lower part ends where the top
 * scan stopped.
 */
static void mean_split(po_state *s, int D, int start, int length, int cnt[2], double *split)
{
    double *x = s->pos;
    cnt[0] = cnt[1] = 0;
    if (length < 2) { cnt[1] = length; return; }
    if (length == 2) {
        cnt[0] = cnt[1] = 1;
        double a = x[3 * start + D], b = x[3 * (start + 1) + D];
        *split = 0.5 * (a + b);
        if (a > b) swap_part(s, start, start + 1);
        return;
    }
    double sum = 0.0;
    for (int i = 0; i < length; i++) sum += x[3 * (start + i) + D];
    double mean = sum / (double)length;
    int top = length - 1;
    for (int i = 0; i < top; i++) {
        if (x[3 * (start + i) + D] > mean) {
            while (top > i && x[3 * (start + top) + D] > mean) top--;
            swap_part(s, start + i, start + top);
        }
    }
    cnt[0] = top;
    cnt[1] = length - top;
    *split = mean;
}

/* src/fmm.c:81-120: depth-first build; leaves numbered as met, nodes preorder */
static void build(po_state *s, int D, int start, int length, int id, int *last_leaf, int *last_node)
{
    if (s->err || length == 0) return;
    o_node *nd = NODE(s, id);
    nd->npart = length;
    int cnt[2];
    double split = 0.0;
    mean_split(s, D, start, length, cnt, &split);
    nd->split = split;
    int ip = start;
    for (int c = 0; c < 2; c++) {
        if (cnt[c] <= s->p.maxleaf) {
            if (*last_leaf - s->first_leaf >= s->nleaf_cap) { s->err = PO_ERR_LEAF_CAPACITY; return; }
            o_leaf *lf = LEAF(s, *last_leaf);
            lf->npart = cnt[c];
            lf->ipart = ip;
            nd->son[c] = *last_leaf;
            (*last_leaf)++;
        } else {
            (*last_node)++;
            if (*last_node - s->first_node >= s->nnode_cap) { s->err = PO_ERR_NODE_CAPACITY; return; }
            nd->son[c] = *last_node;
            build(s, (D + 1) % 3, ip, cnt[c], *last_node, last_leaf, last_node);
            nd = NODE(s, id);
        }
        ip += cnt[c];
    }
}

/* src/fmm.c:123-177: boxes from the split planes */
static void geometry(po_state *s, int D, int id, double lo[3], double hi[3])
{
    o_node *nd = NODE(s, id);
    for (int d = 0; d < 3; d++) {
        nd->width[d] = hi[d] - lo[d];
        nd->center[d] = 0.5 * (hi[d] + lo[d]);
    }
    int nD = (D + 1) % 3;
    for (int c = 0; c < 2; c++) {
        int ch = nd->son[c];
        if (IS_LEAF(s, ch)) {
            o_leaf *lf = LEAF(s, ch);
            memcpy(lf->width, nd->width, sizeof lf->width);
            memcpy(lf->center, nd->center, sizeof lf->center);
            if (c == 0) {
                lf->width[D] = nd->split - lo[D];
                lf->center[D] = 0.5 * (lo[D] + nd->split);
            } else {
                lf->width[D] = hi[D] - nd->split;
                lf->center[D] = 0.5 * (hi[D] + nd->split);
            }
        } else if (c == 0) {
            double keep = hi[D];
            hi[D] = nd->split;
            geometry(s, nD, ch, lo, hi);
            hi[D] = keep;
        } else {
            double keep = lo[D];
            lo[D] = nd->split;
            geometry(s, nD, ch, lo, hi);
            lo[D] = keep;
        }
    }
}

/* src/operator.c:165-194: multipoles, children in order */
static void upward(po_state *s, int id)
{
    o_node *nd = NODE(s, id);
    for (int c = 0; c < 2; c++) {
        int ch = nd->son[c];
        if (IS_LEAF(s, ch)) {
            o_leaf *lf = LEAF(s, ch);
            po_m2m(nd->center[0] - lf->center[0], nd->center[1] - lf->center[1], nd->center[2] - lf->center[2],
                   lf->M, nd->M);
        } else {
            upward(s, ch);
            o_node *cn = NODE(s, ch);
            po_m2m(nd->center[0] - cn->center[0], nd->center[1] - cn->center[1], nd->center[2] - cn->center[2],
                   cn->M, nd->M);
        }
    }
}

/* src/operator.c:498-528: local expansions pushed to children */
static void downward(po_state *s, int id)
{
    o_node *nd = NODE(s, id);
    for (int c = 0; c < 2; c++) {
        int ch = nd->son[c];
        if (s->leaf_on && !(IS_LEAF(s, ch) ? s->leaf_on[ch - s->first_leaf] : s->node_on[ch - s->first_node]))
            continue;
        if (!IS_LEAF(s, ch)) {
            o_node *cn = NODE(s, ch);
            po_l2l(cn->center[0] - nd->center[0], cn->center[1] - nd->center[1], cn->center[2] - nd->center[2],
                   nd->L, cn->L);
            downward(s, ch);
        } else {
            o_leaf *lf = LEAF(s, ch);
            po_l2l(lf->center[0] - nd->center[0], lf->center[1] - nd->center[1], lf->center[2] - nd->center[2],
                   nd->L, lf->L);
        }
    }
}

/* ------------------------------------------------------------------ */
/* dual-tree walks                                                     */
/* ------------------------------------------------------------------ */
static const double *geom_center(po_state *s, int id)
{
    return IS_LEAF(s, id) ? LEAF(s, id)->center : NODE(s, id)->center;
}
static const double *geom_width(po_state *s, int id)
{
    return IS_LEAF(s, id) ? LEAF(s, id)->width : NODE(s, id)->width;
}
static double wsum(const double *w) { return w[0] + w[1] + w[2]; }

static int push_item(o_walker *w, int kind, int a, int b)
{
    if (w->nitems == w->capitems) {
        long cap = w->capitems ? 2 * w->capitems : 256;
        o_item *it = realloc(w->items, sizeof(o_item) * cap);
        if (!it) return -1;
        w->items = it;
        w->capitems = cap;
    }
    w->items[w->nitems].kind = kind;
    w->items[w->nitems].a = a;
    w->items[w->nitems].b = b;
    w->nitems++;
    return 0;
}

static void emit(o_walker *w, int kind, int t, int src)
{
    if (w->err) return;
    if (kind == PO_LIST_M2L || kind == PO_LIST_M2L_EXT) w->m2l++;
    int rc = w->defer_depth ? push_item(w, kind, t, src) : list_push(&w->list[kind], t, src, w->image);
    if (rc != 0) w->err = PO_ERR_NOMEM;
}

/* in a splitting walk, the pair (im, jm) at the split depth becomes a sub-walk */
static int deferred(o_walker *w, int depth, int im, int jm)
{
    if (!w->defer_depth || depth < w->defer_depth) return 0;
    if (push_item(w, 4, im, jm) != 0) w->err = PO_ERR_NOMEM;
    return 1;
}

/*
 * Local walk, src/fmm.c:406-538 (P2P) and src/fmm.c:569-712 (M2L) -- one
 * traversal, since both walks make identical decisions and differ only in
 * what they record: a leaf pair (or a leaf with itself) is a P2P task, an
 * accepted pair is an M2L task.  Node pairs that must be opened open the
 * side with the larger width sum (the source side on ties).
 */
static void walk_local(o_walker *w, int im, int jm, int depth)
{
    po_state *s = w->s;
    if (w->err || im < 0 || jm < 0) return;
    if (deferred(w, depth, im, jm)) return;
    int il = IS_LEAF(s, im), jl = IS_LEAF(s, jm);
    if (im == jm) {
        if (il) { emit(w, PO_LIST_P2P, im, jm); return; }
        o_node *a = NODE(s, im);
        walk_local(w, a->son[0], a->son[0], depth + 1);
        walk_local(w, a->son[0], a->son[1], depth + 1);
        walk_local(w, a->son[1], a->son[0], depth + 1);
        walk_local(w, a->son[1], a->son[1], depth + 1);
        return;
    }
    if (il && jl) { emit(w, PO_LIST_P2P, im, jm); return; }
    const double *ci = geom_center(s, im), *cj = geom_center(s, jm);
    double dist[3] = {ci[0] - cj[0], ci[1] - cj[1], ci[2] - cj[2]};
    /* the reference passes the leaf's width first in mixed pairs */
    int flag = jl ? po_acceptance(geom_width(s, jm), geom_width(s, im), dist, s->p.theta, s->p.rcut)
                  : po_acceptance(geom_width(s, im), geom_width(s, jm), dist, s->p.theta, s->p.rcut);
    if (flag == -1) return;
    if (flag == 1) { emit(w, PO_LIST_M2L, im, jm); return; }
    int open_target;
    if (il) open_target = 0;
    else if (jl) open_target = 1;
    else open_target = wsum(NODE(s, im)->width) > wsum(NODE(s, jm)->width);
    if (open_target) {
        o_node *a = NODE(s, im);
        walk_local(w, a->son[0], jm, depth + 1);
        walk_local(w, a->son[1], jm, depth + 1);
    } else {
        o_node *b = NODE(s, jm);
        walk_local(w, im, b->son[0], depth + 1);
        walk_local(w, im, b->son[1], depth + 1);
    }
}

/*
 * The exported (image) tree, src/remotes.c:60-169: the local tree shifted
 * by s->shift, with the children of an internal node dropped ("pruned")
 * when its shifted box is at least rcut from the receiving domain's box, or
 * when its largest width is below 0.95 theta times that distance.  Leaves
 * always ship their bodies.  The export is not materialised here: a node
 * of the image tree is a local node plus the shift, and its pruning is
 * evaluated where the walk needs it.  At one rank the receiving domain is
 * the local domain (toptree[0] after connect_local_toptree, i.e. the root
 * box).
 */
static int image_pruned(o_walker *w, int id)
{
    po_state *s = w->s;
    o_node *nd = NODE(s, id);
    o_node *root = NODE(s, s->first_node);
    double dr = 0.0;
    for (int d = 0; d < 3; d++) {
        double g = root->center[d] - nd->center[d] - w->shift[d];
        if (g < 0.0) g = -g;
        g -= (root->width[d] + nd->width[d]) * 0.5;
        if (g > 0.0) dr += g * g;
    }
    dr = sqrt(dr);
    double wmax = nd->width[0];
    if (wmax < nd->width[1]) wmax = nd->width[1];
    if (wmax < nd->width[2]) wmax = nd->width[2];
    if (dr >= s->p.rcut) return 1;
    return wmax < 0.95 * s->p.theta * dr;
}

/* src/remotes.c:213-372 (P2P) and 405-552 (M2L), one traversal.  The
   received node is a leaf iff it holds <= MAXLEAF particles; pruned
   received nodes are interacted by M2L unless dropped. */
static void walk_image(o_walker *w, int im, int jm, int depth)
{
    po_state *s = w->s;
    if (w->err) return;
    if (deferred(w, depth, im, jm)) return;
    int il = IS_LEAF(s, im);
    int jl = IS_LEAF(s, jm);
    if (il && jl) { emit(w, PO_LIST_P2P_EXT, im, jm); return; }
    const double *ci = geom_center(s, im), *cj = geom_center(s, jm);
    double cjs[3] = {cj[0] + w->shift[0], cj[1] + w->shift[1], cj[2] + w->shift[2]};
    double dist[3] = {ci[0] - cjs[0], ci[1] - cjs[1], ci[2] - cjs[2]};
    int flag = po_acceptance(geom_width(s, im), geom_width(s, jm), dist, s->p.theta, s->p.rcut);
    if (flag == -1) return;
    int pruned = jl ? 0 : image_pruned(w, jm);
    if (il) {
        if (flag == 1 || pruned) { emit(w, PO_LIST_M2L_EXT, im, jm); return; }
        o_node *b = NODE(s, jm);
        walk_image(w, im, b->son[0], depth + 1);
        walk_image(w, im, b->son[1], depth + 1);
        return;
    }
    if (flag == 1) { emit(w, PO_LIST_M2L_EXT, im, jm); return; }
    int open_target = jl || pruned || wsum(NODE(s, im)->width) > wsum(NODE(s, jm)->width);
    if (open_target) {
        o_node *a = NODE(s, im);
        walk_image(w, a->son[0], jm, depth + 1);
        walk_image(w, a->son[1], jm, depth + 1);
    } else {
        o_node *b = NODE(s, jm);
        walk_image(w, im, b->son[0], depth + 1);
        walk_image(w, im, b->son[1], depth + 1);
    }
}

/* The walk against a received tree (src/remotes.c:213-372 and 405-552,
   one traversal): source jm indexes the received RemoteNode array; a node
   is a leaf iff it holds <= MAXLEAF particles, and a node sent without its
   children (son = -1, pruned by the sender) is interacted by M2L unless
   dropped.  Entries carry the received tree's image tag. */
static void walk_received(o_walker *w, const o_rtree *rt, int im, int jm, int depth)
{
    po_state *s = w->s;
    if (w->err) return;
    if (deferred(w, depth, im, jm)) return;
    const o_rnode *J = &rt->node[jm];
    int il = IS_LEAF(s, im);
    int jl = J->npart <= s->p.maxleaf;
    if (il && jl) { emit(w, PO_LIST_P2P_EXT, im, jm); return; }
    const double *ci = geom_center(s, im);
    double dist[3] = {ci[0] - J->center[0], ci[1] - J->center[1], ci[2] - J->center[2]};
    int flag = po_acceptance(geom_width(s, im), J->width, dist, s->p.theta, s->p.rcut);
    if (flag == -1) return;
    int pruned = !jl && (J->son[0] < 0 || J->son[1] < 0);
    if (il) {
        if (flag == 1 || pruned) { emit(w, PO_LIST_M2L_EXT, im, jm); return; }
        walk_received(w, rt, im, J->son[0], depth + 1);
        walk_received(w, rt, im, J->son[1], depth + 1);
        return;
    }
    if (flag == 1) { emit(w, PO_LIST_M2L_EXT, im, jm); return; }
    int open_target = jl || pruned || wsum(NODE(s, im)->width) > wsum(J->width);
    if (open_target) {
        o_node *a = NODE(s, im);
        walk_received(w, rt, a->son[0], jm, depth + 1);
        walk_received(w, rt, a->son[1], jm, depth + 1);
    } else {
        walk_received(w, rt, im, J->son[0], depth + 1);
        walk_received(w, rt, im, J->son[1], depth + 1);
    }
}

/* The exported copy of a local tree (src/remotes.c:60-169): the tree
   shifted by `sh`, in depth-first preorder, an internal node's children
   left out when its shifted box lies at least rcut from the receiving
   domain's box (centre rc, width rw) or its largest width is below
   0.95 theta times that distance; leaves ship their bodies (shifted). */
static int export_node(const po_state *s, int id, const double rc[3], const double rw[3], const double sh[3],
                       o_rtree *out)
{
    int me = out->nnode++;
    o_rnode *E = &out->node[me];
    if (IS_LEAF(s, id)) {
        const o_leaf *lf = &s->leaf[id - s->first_leaf];
        E->npart = lf->npart;
        for (int d = 0; d < 3; d++) { E->center[d] = lf->center[d] + sh[d]; E->width[d] = lf->width[d]; }
        memcpy(E->M, lf->M, sizeof E->M);
        E->son[0] = out->nbody;
        for (int q = lf->ipart; q < lf->ipart + lf->npart; q++) {
            for (int d = 0; d < 3; d++) out->body[3 * (size_t)out->nbody + d] = s->pos[3 * (size_t)q + d] + sh[d];
            out->nbody++;
        }
        E->son[1] = out->nbody;
        return me;
    }
    const o_node *nd = &s->node[id - s->first_node];
    double dr = 0.0;
    for (int d = 0; d < 3; d++) {
        double g = rc[d] - nd->center[d] - sh[d];
        if (g < 0.0) g = -g;
        g -= (rw[d] + nd->width[d]) * 0.5;
        if (g > 0.0) dr += g * g;
    }
    dr = sqrt(dr);
    E->npart = nd->npart;
    for (int d = 0; d < 3; d++) { E->center[d] = nd->center[d] + sh[d]; E->width[d] = nd->width[d]; }
    memcpy(E->M, nd->M, sizeof E->M);
    double wmax = nd->width[0];
    if (wmax < nd->width[1]) wmax = nd->width[1];
    if (wmax < nd->width[2]) wmax = nd->width[2];
    if (dr >= s->p.rcut || wmax < 0.95 * s->p.theta * dr) {
        E->son[0] = E->son[1] = -1;
        return me;
    }
    for (int c = 0; c < 2; c++) {
        int k = export_node(s, nd->son[c], rc, rw, sh, out);
        out->node[me].son[c] = k;
    }
    return me;
}

int po_export(const po_state *s, const double recv_center[3], const double recv_width[3], const double shift[3],
              int *nnode, int *nbody, int node_cap, int body_cap, void *nodes, double *bodies)
{
    if (!s || !s->node || !nnode || !nbody) return PO_ERR_ARG;
    o_rtree t;
    t.nnode = t.nbody = 0;
    t.node = malloc(sizeof(o_rnode) * (size_t)(s->nleaf + s->nnode));
    t.body = malloc(sizeof(double) * 3 * (size_t)s->n);
    if (!t.node || !t.body) { free(t.node); free(t.body); return PO_ERR_NOMEM; }
    export_node(s, s->first_node, recv_center, recv_width, shift, &t);
    *nnode = t.nnode;
    *nbody = t.nbody;
    int rc = PO_OK;
    if (nodes && bodies) {
        if (t.nnode > node_cap || t.nbody > body_cap) rc = PO_ERR_ARG;
        else {
            memcpy(nodes, t.node, sizeof(o_rnode) * (size_t)t.nnode);
            memcpy(bodies, t.body, sizeof(double) * 3 * (size_t)t.nbody);
        }
    }
    free(t.node);
    free(t.body);
    return rc;
}

/* ------------------------------------------------------------------ */
/* pair kernel and list compute                                        */
/* ------------------------------------------------------------------ */
/* Softened, erfc-truncated pair force of src/fmm.c:834-852 and
   src/remotes.c:30-50, in the same operation order. */
static inline void pair_force(const double *pj, const double *pi, const po_params *p, double coeff, double *a)
{
    double dx0 = pj[0] - pi[0], dx1 = pj[1] - pi[1], dx2 = pj[2] - pi[2];
    double dr = sqrt(dx0 * dx0 + dx1 * dx1 + dx2 * dx2);
    double ir3 = (dr < p->eps) ? p->mass / (p->eps * p->eps * p->eps) : p->mass / (dr * dr * dr);
    double drs = 0.5 * dr / p->rs;
    ir3 *= (erfc(drs) + coeff * drs * exp(-drs * drs));
    a[0] += dx0 * ir3;
    a[1] += dx1 * ir3;
    a[2] += dx2 * ir3;
}

/* stable grouping of a list by target (counting sort) */
static int group_by_target(const o_list *l, int first_id, int nid, long **off_out, long **order_out)
{
    long *off = calloc((size_t)nid + 1, sizeof(long));
    long *order = malloc(sizeof(long) * (l->n ? l->n : 1));
    if (!off || !order) { free(off); free(order); return -1; }
    for (long i = 0; i < l->n; i++) off[l->t[i] - first_id + 1]++;
    for (int i = 0; i < nid; i++) off[i + 1] += off[i];
    long *fill = malloc(sizeof(long) * ((size_t)nid + 1));
    if (!fill) { free(off); free(order); return -1; }
    memcpy(fill, off, sizeof(long) * ((size_t)nid + 1));
    for (long i = 0; i < l->n; i++) order[fill[l->t[i] - first_id]++] = i;
    free(fill);
    *off_out = off;
    *order_out = order;
    return 0;
}

typedef struct {
    po_state *s;
    long *off, *order;      /* grouped P2P list */
    const o_list *l;
    int ext;                /* 0: local tasks, 1: image tasks */
    int next;
    pthread_mutex_t mu;
} p2p_job;

/* Per target leaf, in list order.  Local tasks sum each task separately and
   then add it (src/fmm.c:823-868); image tasks add pair by pair
   (src/remotes.c:26-56). */
static void p2p_target(p2p_job *J, int lf_index)
{
    po_state *s = J->s;
    const po_params *p = &s->p;
    double coeff = 2.0 / sqrt(M_PI);
    o_leaf *T = &s->leaf[lf_index];
    for (long k = J->off[lf_index]; k < J->off[lf_index + 1]; k++) {
        long e = J->order[k];
        const int received = J->ext && J->l->img[e] >= PO_IMG_RECEIVED;
        o_leaf *S = received ? NULL : LEAF(s, J->l->s[e]);
        if (!J->ext) {
            for (int q = 0; q < T->npart; q++) {
                int ip = T->ipart + q;
                if (s->part_on && !s->part_on[ip]) continue;
                double a[3] = {0, 0, 0};
                for (int jp = S->ipart; jp < S->ipart + S->npart; jp++) {
                    if (jp == ip) continue;
                    pair_force(s->pos + 3 * jp, s->pos + 3 * ip, p, coeff, a);
                }
                for (int d = 0; d < 3; d++) s->acc[3 * ip + d] += a[d];
            }
        } else {
            int img = J->l->img[e];
            if (img >= PO_IMG_RECEIVED) {
                /* bodies of a received leaf (src/remotes.c:26-56 on exrbody) */
                const o_rtree *rt = &s->rt[img - PO_IMG_RECEIVED];
                const o_rnode *R = &rt->node[J->l->s[e]];
                for (int ip = T->ipart; ip < T->ipart + T->npart; ip++) {
                    if (s->part_on && !s->part_on[ip]) continue;
                    for (int jp = R->son[0]; jp < R->son[1]; jp++)
                        pair_force(rt->body + 3 * (size_t)jp, s->pos + 3 * ip, p, coeff, s->acc + 3 * ip);
                }
                continue;
            }
            double sh[3];
            int c = 0;
            for (int mi = -1; mi <= 1; mi++)
                for (int mj = -1; mj <= 1; mj++)
                    for (int mk = -1; mk <= 1; mk++) {
                        if (mi == 0 && mj == 0 && mk == 0) continue;
                        if (++c == img) { sh[0] = mi * p->boxsize; sh[1] = mj * p->boxsize; sh[2] = mk * p->boxsize; }
                    }
            for (int ip = T->ipart; ip < T->ipart + T->npart; ip++) {
                if (s->part_on && !s->part_on[ip]) continue;
                for (int jp = S->ipart; jp < S->ipart + S->npart; jp++) {
                    double pj[3] = {s->pos[3 * jp] + sh[0], s->pos[3 * jp + 1] + sh[1], s->pos[3 * jp + 2] + sh[2]};
                    pair_force(pj, s->pos + 3 * ip, p, coeff, s->acc + 3 * ip);
                }
            }
        }
    }
}

static void *p2p_worker(void *arg)
{
    p2p_job *J = arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int i = J->next;
        J->next += 16;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->s->nleaf) break;
        int e = i + 16 < J->s->nleaf ? i + 16 : J->s->nleaf;
        for (; i < e; i++)
            if (!J->s->leaf_on || J->s->leaf_on[i]) p2p_target(J, i);
    }
    return 0;
}

static int run_p2p(po_state *s, const o_list *l, int ext)
{
    p2p_job J;
    memset(&J, 0, sizeof J);
    J.s = s; J.l = l; J.ext = ext;
    if (group_by_target(l, s->first_leaf, s->nleaf, &J.off, &J.order) != 0) return PO_ERR_NOMEM;
    pthread_mutex_init(&J.mu, 0);
    int nt = s->p.nthreads > 1 ? s->p.nthreads : 1;
    if (nt == 1) {
        p2p_worker(&J);
    } else {
        pthread_t *th = malloc(sizeof(pthread_t) * nt);
        for (int i = 0; i < nt; i++) pthread_create(&th[i], 0, p2p_worker, &J);
        for (int i = 0; i < nt; i++) pthread_join(th[i], 0);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    free(J.off);
    free(J.order);
    return PO_OK;
}

static void image_shift(const po_params *p, int img, double sh[3])
{
    int c = 0;
    for (int mi = -1; mi <= 1; mi++)
        for (int mj = -1; mj <= 1; mj++)
            for (int mk = -1; mk <= 1; mk++) {
                if (mi == 0 && mj == 0 && mk == 0) continue;
                if (++c == img) { sh[0] = mi * p->boxsize; sh[1] = mj * p->boxsize; sh[2] = mk * p->boxsize; }
            }
}

/* src/fmm.c:875-907 and src/remotes.c:598-628, in list order */
static void run_m2l(po_state *s, const o_list *l)
{
    for (long e = 0; e < l->n; e++) {
        int im = l->t[e], jm = l->s[e];
        if (s->leaf_on && !(IS_LEAF(s, im) ? s->leaf_on[im - s->first_leaf] : s->node_on[im - s->first_node]))
            continue;
        const double *ci = geom_center(s, im);
        double *L = IS_LEAF(s, im) ? LEAF(s, im)->L : NODE(s, im)->L;
        if (l->img[e] >= PO_IMG_RECEIVED) {
            /* a received node: its centre already carries the sender's shift */
            const o_rnode *R = &s->rt[l->img[e] - PO_IMG_RECEIVED].node[jm];
            po_m2l(ci[0] - R->center[0], ci[1] - R->center[1], ci[2] - R->center[2], R->M, L, s->p.rs);
            continue;
        }
        double sh[3] = {0, 0, 0};
        if (l->img[e]) image_shift(&s->p, l->img[e], sh);
        const double *cj = geom_center(s, jm);
        double cjs[3] = {cj[0] + sh[0], cj[1] + sh[1], cj[2] + sh[2]};
        const double *M = IS_LEAF(s, jm) ? LEAF(s, jm)->M : NODE(s, jm)->M;
        if (l->img[e])
            po_m2l(ci[0] - cjs[0], ci[1] - cjs[1], ci[2] - cjs[2], M, L, s->p.rs);
        else
            po_m2l(ci[0] - cj[0], ci[1] - cj[1], ci[2] - cj[2], M, L, s->p.rs);
    }
}

static double wall(void)
{
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

/* ------------------------------------------------------------------ */
/* walks on several threads, lists in the sequential order             */
/* ------------------------------------------------------------------ */
typedef struct {
    po_state *s;
    o_walker *sub;          /* one walker per deferred sub-walk */
    long nsub;
    long next;
    pthread_mutex_t mu;
} walk_job;

static void walk_run(o_walker *w, int im, int jm)
{
    if (w->image >= PO_IMG_RECEIVED) walk_received(w, &w->s->rt[w->image - PO_IMG_RECEIVED], im, jm, 0);
    else if (w->image) walk_image(w, im, jm, 0);
    else walk_local(w, im, jm, 0);
}

static void *walk_worker(void *arg)
{
    walk_job *J = arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        long i = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->nsub) break;
        o_walker *w = &J->sub[i];
        walk_run(w, w->items[0].a, w->items[0].b);
    }
    return 0;
}

static void walker_free(o_walker *w)
{
    for (int k = 0; k < 4; k++) { free(w->list[k].t); free(w->list[k].s); free(w->list[k].img); }
    free(w->items);
}

static int list_append(o_list *dst, const o_list *src)
{
    for (long i = 0; i < src->n; i++)
        if (list_push(dst, src->t[i], src->s[i], src->img[i]) != 0) return -1;
    return 0;
}

/* The local walk (image 0) and then the 26 image walks, each as the
   reference runs it (fmm_task, then fmm_ext's loop over images).  Each walk
   is first expanded sequentially down to a fixed recursion depth; the
   pairs met there are walked on the worker threads into lists of their
   own, which are then concatenated in the order the sequential traversal
   would have emitted them, so the lists are identical to a one-thread
   walk's. */
static int run_walks(po_state *s, int images)
{
    /* walks in order: the local tree, its 26 images (on the fly), then the
       received trees */
    const int nown = images ? NIMG : 1;
    int nimg = nown + s->nrt;
    o_walker *top = calloc((size_t)nimg, sizeof(o_walker));
    if (!top) return PO_ERR_NOMEM;
    long nsub = 0;
    int rc = PO_OK;
    for (int k = 0; k < nimg; k++) {
        const int img = k < nown ? k : PO_IMG_RECEIVED + (k - nown);
        top[k].s = s;
        top[k].image = img;
        if (img && img < PO_IMG_RECEIVED) image_shift(&s->p, img, top[k].shift);
        top[k].defer_depth = 12;
        walk_run(&top[k], s->first_node, img >= PO_IMG_RECEIVED ? 0 : s->first_node);
        if (top[k].err) rc = top[k].err;
        for (long i = 0; i < top[k].nitems; i++) nsub += top[k].items[i].kind == 4;
    }
    walk_job J;
    memset(&J, 0, sizeof J);
    J.s = s;
    J.sub = calloc((size_t)(nsub ? nsub : 1), sizeof(o_walker));
    if (!J.sub) rc = PO_ERR_NOMEM;
    if (rc == PO_OK) {
        long k = 0;
        for (int t = 0; t < nimg; t++)
            for (long i = 0; i < top[t].nitems; i++) {
                if (top[t].items[i].kind != 4) continue;
                o_walker *w = &J.sub[k++];
                w->s = s;
                w->image = top[t].image;
                memcpy(w->shift, top[t].shift, sizeof w->shift);
                if (push_item(w, 4, top[t].items[i].a, top[t].items[i].b) != 0) rc = PO_ERR_NOMEM;
            }
        J.nsub = nsub;
    }
    if (rc == PO_OK) {
        pthread_mutex_init(&J.mu, 0);
        int nt = s->p.nthreads > 1 ? s->p.nthreads : 1;
        if (nt == 1) {
            walk_worker(&J);
        } else {
            pthread_t *th = malloc(sizeof(pthread_t) * nt);
            for (int i = 0; i < nt; i++) pthread_create(&th[i], 0, walk_worker, &J);
            for (int i = 0; i < nt; i++) pthread_join(th[i], 0);
            free(th);
        }
        pthread_mutex_destroy(&J.mu);
        /* concatenate in traversal order */
        long k = 0;
        for (int t = 0; t < nimg && rc == PO_OK; t++) {
            s->walk_m2l_count += top[t].m2l;
            for (long i = 0; i < top[t].nitems && rc == PO_OK; i++) {
                o_item *it = &top[t].items[i];
                if (it->kind != 4) {
                    if (list_push(&s->list[it->kind], it->a, it->b, top[t].image) != 0) rc = PO_ERR_NOMEM;
                    continue;
                }
                o_walker *w = &J.sub[k++];
                if (w->err) { rc = w->err; break; }
                s->walk_m2l_count += w->m2l;
                for (int kind = 0; kind < 4; kind++)
                    if (list_append(&s->list[kind], &w->list[kind]) != 0) rc = PO_ERR_NOMEM;
            }
        }
    }
    for (long i = 0; i < nsub && J.sub; i++) walker_free(&J.sub[i]);
    free(J.sub);
    for (int t = 0; t < nimg; t++) walker_free(&top[t]);
    free(top);
    return rc;
}

/* marks the nodes whose subtree holds a marked leaf */
static int mark_nodes(po_state *s, int id)
{
    if (IS_LEAF(s, id)) return s->leaf_on[id - s->first_leaf];
    o_node *nd = NODE(s, id);
    int a = mark_nodes(s, nd->son[0]);
    int b = mark_nodes(s, nd->son[1]);
    s->node_on[id - s->first_node] = (unsigned char)(a || b);
    return a || b;
}

/* The force phases of the pass on the tree and lists at hand: local P2P
   and M2L (fmm_task), image P2P and M2L (fmm_ext), L2L and L2P.  With
   targets (input indices), only those particles, their leaves and the
   leaves' ancestors are formed, after their accelerations and local
   expansions are cleared, so the same tree can serve several samples. */
static int forces(po_state *s, int nt, const int *targets)
{
    int n = s->n;
    if (targets) {
        free(s->part_on); free(s->leaf_on); free(s->node_on);
        s->part_on = calloc((size_t)n, 1);
        s->leaf_on = calloc((size_t)s->nleaf, 1);
        s->node_on = calloc((size_t)s->nnode, 1);
        int *where = malloc(sizeof(int) * (size_t)n);
        if (!s->part_on || !s->leaf_on || !s->node_on || !where) { free(where); return PO_ERR_NOMEM; }
        for (int i = 0; i < n; i++) where[s->perm[i]] = i;
        for (int k = 0; k < nt; k++) {
            if (targets[k] < 0 || targets[k] >= n) { free(where); return PO_ERR_ARG; }
            int q = where[targets[k]];
            s->part_on[q] = 1;
            for (int d = 0; d < 3; d++) s->acc[3 * (size_t)q + d] = 0.0;
        }
        free(where);
        for (int i = 0; i < s->nleaf; i++) {
            o_leaf *lf = &s->leaf[i];
            for (int q = lf->ipart; q < lf->ipart + lf->npart; q++)
                if (s->part_on[q]) { s->leaf_on[i] = 1; break; }
            if (s->leaf_on[i]) memset(lf->L, 0, sizeof lf->L);
        }
        mark_nodes(s, s->first_node);
        for (int i = 0; i < s->nnode; i++)
            if (s->node_on[i]) memset(s->node[i].L, 0, sizeof s->node[i].L);
    }
    int rc = run_p2p(s, &s->list[PO_LIST_P2P], 0);
    if (rc) return rc;
    run_m2l(s, &s->list[PO_LIST_M2L]);
    if (s->acc_task) memcpy(s->acc_task, s->acc, sizeof(double) * 3 * (size_t)n);
    if (s->p.images) {
        rc = run_p2p(s, &s->list[PO_LIST_P2P_EXT], 1);
        if (rc) return rc;
        run_m2l(s, &s->list[PO_LIST_M2L_EXT]);
    }
    downward(s, s->first_node);
    for (int i = 0; i < s->nleaf; i++) {
        if (s->leaf_on && !s->leaf_on[i]) continue;
        o_leaf *lf = &s->leaf[i];
        po_l2p(lf->npart, s->pos + 3 * lf->ipart, lf->center, lf->L, s->acc + 3 * lf->ipart);
    }
    return PO_OK;
}

/* pairs of the ext P2P list (images and received trees): n_t n_s per task,
   as src/remotes.c:26-56 counts p2p_count_remote */
static long long ext_pairs(const po_state *s)
{
    long long b = 0;
    const o_list *l = &s->list[PO_LIST_P2P_EXT];
    for (long e = 0; e < l->n; e++) {
        long long ns;
        if (l->img[e] >= PO_IMG_RECEIVED) {
            const o_rnode *R = &s->rt[l->img[e] - PO_IMG_RECEIVED].node[l->s[e]];
            ns = R->son[1] - R->son[0];
        } else {
            ns = LEAF(s, l->s[e])->npart;
        }
        b += (long long)LEAF(s, l->t[e])->npart * ns;
    }
    return b;
}

/* the whole pass: src/fmm.c:329-360 (construct), 719-770 (prepare),
   909-984 (task), 987-1075 (ext) at one rank.  With targets, the tree,
   walks, counters and multipoles are complete, but forces are formed only
   for the listed particles (P2P into them, M2L into their leaves and
   ancestors, L2L down those paths, L2P on them), in the same operation
   order as the full pass, so their accelerations are identical to it. */
/* src/fmm.c:180-264 (tree) and 719-747 (P2M, M2M): t[0] tree build and
   geometry, t[1] multipoles; keep_task: keep a copy of the accelerations
   after the local task phase */
static int prepare_pass(po_state *s, const po_params *p, int n, const double *pos_in, int keep_task, double *t)
{
    init_tables();
    if (!s || !p || n < 1 || p->maxleaf < 1) return PO_ERR_ARG;
    if (n <= p->maxleaf) return PO_ERR_SMALL;
    free_run(s);
    for (int k = 0; k < 4; k++) s->list[k].n = 0;
    s->p = *p;
    s->n = n;
    s->err = 0;
    s->walk_m2l_count = 0;
    s->p2p_count_remote = 0;

    s->pos = malloc(sizeof(double) * 3 * (size_t)n);
    s->perm = malloc(sizeof(int) * (size_t)n);
    s->acc = calloc(3 * (size_t)n, sizeof(double));
    s->acc_task = keep_task ? calloc(3 * (size_t)n, sizeof(double)) : NULL;
    /* capacity rule of src/fmm.c:203-209 */
    int cap = (int)(2.0 * ((double)n) / ((double)p->maxleaf));
    if (cap > n) cap = n + 1;
    s->nleaf_cap = s->nnode_cap = cap;
    s->leaf = calloc((size_t)cap, sizeof(o_leaf));
    s->node = calloc((size_t)cap, sizeof(o_node));
    if (!s->pos || !s->perm || !s->acc || (keep_task && !s->acc_task) || !s->leaf || !s->node) return PO_ERR_NOMEM;
    for (int i = 0; i < cap; i++) s->node[i].son[0] = s->node[i].son[1] = -1;
    memcpy(s->pos, pos_in, sizeof(double) * 3 * (size_t)n);
    for (int i = 0; i < n; i++) s->perm[i] = i;

    double t0 = wall();
    s->first_leaf = n;
    s->first_node = n + cap;
    int last_leaf = s->first_leaf, last_node = s->first_node;
    build(s, s->domain_set ? s->axis0 : 0, 0, n, s->first_node, &last_leaf, &last_node);
    if (s->err) return s->err;
    s->nleaf = last_leaf - s->first_leaf;
    s->nnode = last_node - s->first_node + 1;
    double lo[3] = {0, 0, 0}, hi[3] = {p->boxsize, p->boxsize, p->boxsize};
    if (s->domain_set)
        for (int d = 0; d < 3; d++) { lo[d] = s->dom_lo[d]; hi[d] = s->dom_hi[d]; }
    geometry(s, s->domain_set ? s->axis0 : 0, s->first_node, lo, hi);
    double t1 = wall();
    for (int i = 0; i < s->nleaf; i++) {
        o_leaf *lf = &s->leaf[i];
        po_p2m(lf->npart, s->pos + 3 * lf->ipart, p->mass, lf->center, lf->M);
    }
    upward(s, s->first_node);
    double t2 = wall();
    t[0] = t1 - t0;
    t[1] = t2 - t1;
    return PO_OK;
}

static int run_pass(po_state *s, const po_params *p, int n, const double *pos_in, int nt, const int *targets,
                    double *times)
{
    if (nt < 0) return PO_ERR_ARG;
    /* a plain pass: the whole periodic box, nothing received */
    if (s) {
        s->domain_set = 0;
        for (int k = 0; k < s->nrt; k++) { free(s->rt[k].node); free(s->rt[k].body); }
        free(s->rt);
        s->rt = NULL;
        s->nrt = 0;
    }
    double tp[2];
    int rc = prepare_pass(s, p, n, pos_in, targets == NULL, tp);
    if (rc) return rc;
    double t2 = wall();
    rc = run_walks(s, p->images);
    if (rc) return rc;
    s->p2p_count_remote = ext_pairs(s);
    double t3 = wall();

    rc = forces(s, nt, targets);
    if (rc) return rc;
    double t4 = wall();
    if (times) {
        times[0] = tp[0];     /* tree build and geometry */
        times[1] = tp[1];     /* P2M, M2M */
        times[2] = t3 - t2;   /* local and image walks */
        times[3] = t4 - t3;   /* forces (all particles, or the listed ones) */
    }
    return PO_OK;
}

int po_run(po_state *s, const po_params *p, int n, const double *pos_in, double *seconds)
{
    double t[4];
    int rc = run_pass(s, p, n, pos_in, 0, NULL, t);
    if (rc == PO_OK && seconds) *seconds = t[0] + t[1] + t[2] + t[3];
    return rc;
}

static int gather_targets(po_state *s, int nt, const int *targets, double *acc_out)
{
    int n = s->n;
    int *where = malloc(sizeof(int) * (size_t)n);
    if (!where) return PO_ERR_NOMEM;
    for (int i = 0; i < n; i++) where[s->perm[i]] = i;
    for (int k = 0; k < nt; k++)
        for (int d = 0; d < 3; d++) acc_out[3 * k + d] = s->acc[3 * (size_t)where[targets[k]] + d];
    free(where);
    return PO_OK;
}

int po_run_sample(po_state *s, const po_params *p, int n, const double *pos_in, int nt, const int *targets,
                  double *acc_out, double *times)
{
    if (!targets || !acc_out) return PO_ERR_ARG;
    int rc = run_pass(s, p, n, pos_in, nt, targets, times);
    if (rc != PO_OK) return rc;
    return gather_targets(s, nt, targets, acc_out);
}

int po_forces_sample(po_state *s, int nt, const int *targets, double *acc_out, double *seconds)
{
    if (!s || !s->leaf || !targets || !acc_out || nt < 0) return PO_ERR_ARG;
    double t0 = wall();
    int rc = forces(s, nt, targets);
    if (rc != PO_OK) return rc;
    if (seconds) *seconds = wall() - t0;
    return gather_targets(s, nt, targets, acc_out);
}

/* pairs of the local and image P2P lists as the reference evaluates them:
   n_t n_s per task, minus the self pairs of a leaf with itself (local);
   n_t n_s per image task */
void po_pairs(const po_state *s, long long *pairs_local, long long *pairs_image)
{
    long long a = 0, b = 0;
    const o_list *l = &s->list[PO_LIST_P2P];
    for (long e = 0; e < l->n; e++) {
        long long nt = LEAF(s, l->t[e])->npart, ns = LEAF(s, l->s[e])->npart;
        a += l->t[e] == l->s[e] ? nt * (nt - 1) : nt * ns;
    }
    b = ext_pairs(s);
    *pairs_local = a;
    *pairs_image = b;
}

/* ------------------------------------------------------------------ */
/* several ranks, emulated in one process                              */
/* ------------------------------------------------------------------ */
/* Domain ids of src/initial.c:197-222: domains are the leaves P-1..2P-2 of
   a heap-ordered binary tree; rank r owns domain r + mostleft (wrapped). */
static int most_left(int P)
{
    if (P == 1) return 0;
    int m = 1;
    while (m < 2 * P - 1) m *= 2;
    return m / 2 - 1;
}

static int rank_of_domain(int P, int d) { return (d - most_left(P) + P) % P; }

static double domain_time(int P, int id)
{
    if (id >= P - 1) return 1.0;  /* every domain's time is 1 at the first step */
    return domain_time(P, 2 * id + 1) + domain_time(P, 2 * id + 2);
}

/* src/domains.c:400-425 (domain_volume_part): split planes dividing each
   node's box in the ratio of its children's times (equal per domain) */
static void domain_volume_part(int P, int id, double bl[3], double br[3], int dim, double *split)
{
    if (id >= P - 1) return;
    double tl = domain_time(P, 2 * id + 1), tr = domain_time(P, 2 * id + 2);
    double frac = bl[dim] + (br[dim] - bl[dim]) * tl / (tl + tr);
    split[id] = frac;
    double keep = br[dim];
    br[dim] = frac;
    domain_volume_part(P, 2 * id + 1, bl, br, (dim + 1) % 3, split);
    br[dim] = keep;
    keep = bl[dim];
    bl[dim] = frac;
    domain_volume_part(P, 2 * id + 2, bl, br, (dim + 1) % 3, split);
    bl[dim] = keep;
}

/* src/toptree.c:157-182 (center_toptree): each domain's box and the axis
   its local tree splits first (direct_local_start) */
static void domain_boxes(int P, int id, int dir, double lo[3], double hi[3], const double *split, double *box,
                         int *axis)
{
    if (id >= P - 1) {
        int r = rank_of_domain(P, id);
        for (int d = 0; d < 3; d++) { box[6 * r + d] = lo[d]; box[6 * r + 3 + d] = hi[d]; }
        axis[r] = dir;
        return;
    }
    double keep = hi[dir];
    hi[dir] = split[id];
    domain_boxes(P, 2 * id + 1, (dir + 1) % 3, lo, hi, split, box, axis);
    hi[dir] = keep;
    keep = lo[dir];
    lo[dir] = split[id];
    domain_boxes(P, 2 * id + 2, (dir + 1) % 3, lo, hi, split, box, axis);
    lo[dir] = keep;
}

int po_domains(int P, double boxsize, double *box, int *axis, double *split)
{
    if (P < 1 || !box || !axis) return PO_ERR_ARG;
    double *sp = calloc((size_t)(P > 1 ? P - 1 : 1), sizeof(double));
    if (!sp) return PO_ERR_NOMEM;
    double bl[3] = {0, 0, 0}, br[3] = {boxsize, boxsize, boxsize};
    domain_volume_part(P, 0, bl, br, 0, sp);
    double lo[3] = {0, 0, 0}, hi[3] = {boxsize, boxsize, boxsize};
    domain_boxes(P, 0, 0, lo, hi, sp, box, axis);
    if (split)
        for (int i = 0; i < P - 1; i++) split[i] = sp[i];
    free(sp);
    return PO_OK;
}

/* src/domains.c:165-298: the rank whose domain holds x (a coordinate above a
   split plane goes to the upper child) */
static int rank_of_position(int P, const double *split, const double x[3])
{
    int id = 0, D = 0;
    while (id < P - 1) {
        id = x[D] > split[id] ? 2 * id + 2 : 2 * id + 1;
        D = (D + 1) % 3;
    }
    return rank_of_domain(P, id);
}

/* the root's bounds from the top-tree node's box: centre -/+ half the width
   (src/toptree.c:150-159, src/fmm.c:189-197) */
static void set_domain(po_state *s, const double lo[3], const double hi[3], int axis)
{
    s->domain_set = 1;
    for (int d = 0; d < 3; d++) {
        double c = 0.5 * (hi[d] + lo[d]), w = hi[d] - lo[d];
        s->dom_lo[d] = c - 0.5 * w;
        s->dom_hi[d] = c + 0.5 * w;
    }
    s->axis0 = axis;
}

/* One force pass over P ranks as src/photoNs.c drives them
   (fmm_prepare, fmm_task, fmm_ext) with the ranks emulated in turn: each
   rank's tree covers its domain; fmm_remote(idx, shift) of
   src/remotes.c:684-751 becomes an export from rank r - idx of its tree
   shifted by `shift`, pruned against rank r's domain, walked by rank r:
   the other ranks' trees (shift 0), then for each image shift every
   rank's shifted tree, in fmm_ext's order.  With explicit_self the rank's
   own periodic images also go through an export, otherwise they use the
   single-rank image walk.  acc_out[3n] in input order; counters[16 P] per
   rank as po_counters; rank_out[n]: each particle's rank. */
int po_run_domains(int P, const po_params *p, int n, const double *pos_in, int explicit_self, double *acc_out,
                   long long *counters, int *rank_out)
{
    init_tables();
    if (P < 1 || !p || n < 1 || !pos_in || !acc_out) return PO_ERR_ARG;
    double *box = malloc(sizeof(double) * 6 * (size_t)P), *split = calloc((size_t)P, sizeof(double));
    int *axis = malloc(sizeof(int) * (size_t)P), *rank = malloc(sizeof(int) * (size_t)n);
    int *cnt = calloc((size_t)P, sizeof(int)), *fill = calloc((size_t)P, sizeof(int));
    int *order = malloc(sizeof(int) * (size_t)n);
    double *lpos = malloc(sizeof(double) * 3 * (size_t)n);
    po_state **st = calloc((size_t)P, sizeof(po_state *));
    int rc = (!box || !split || !axis || !rank || !cnt || !fill || !order || !lpos || !st) ? PO_ERR_NOMEM : PO_OK;
    if (!rc) rc = po_domains(P, p->boxsize, box, axis, split);
    if (!rc) {
        for (int i = 0; i < n; i++) { rank[i] = rank_of_position(P, split, pos_in + 3 * (size_t)i); cnt[rank[i]]++; }
        for (int r = 1; r < P; r++) fill[r] = fill[r - 1] + cnt[r - 1];
        for (int i = 0; i < n; i++) order[fill[rank[i]]++] = i;  /* each rank's particles in input order */
        for (int i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) lpos[3 * (size_t)i + d] = pos_in[3 * (size_t)order[i] + d];
        if (rank_out) memcpy(rank_out, rank, sizeof(int) * (size_t)n);
    }
    /* fmm_prepare on every rank */
    int first = 0;
    for (int r = 0; r < P && !rc; r++) {
        st[r] = po_create();
        if (!st[r]) { rc = PO_ERR_NOMEM; break; }
        set_domain(st[r], box + 6 * r, box + 6 * r + 3, axis[r]);
        if (cnt[r] <= p->maxleaf) { rc = PO_ERR_SMALL; break; }
        double t[2];
        rc = prepare_pass(st[r], p, cnt[r], lpos + 3 * (size_t)first, 0, t);
        first += cnt[r];
    }
    /* the trees each rank receives, in fmm_ext's order; the receiving
       domain as its root holds it (connect_local_toptree copies every
       rank's root geometry into the top tree, src/toptree.c:21-40) */
    for (int r = 0; r < P && !rc; r++) {
        int maxrt = (P - 1) + (NIMG - 1) * P;
        st[r]->rt = calloc((size_t)maxrt, sizeof(o_rtree));
        if (!st[r]->rt) { rc = PO_ERR_NOMEM; break; }
        double rcen[3], rwid[3];
        for (int d = 0; d < 3; d++) {
            rcen[d] = 0.5 * (st[r]->dom_hi[d] + st[r]->dom_lo[d]);
            rwid[d] = st[r]->dom_hi[d] - st[r]->dom_lo[d];
        }
        for (int pass = 0; pass < NIMG && !rc; pass++) {
            double sh[3] = {0, 0, 0};
            if (pass) image_shift(p, pass, sh);
            for (int idx = pass ? 0 : 1; idx < P && !rc; idx++) {
                if (pass && idx == 0 && !explicit_self) continue;
                po_state *q = st[(r - idx + P) % P];
                o_rtree *t = &st[r]->rt[st[r]->nrt];
                t->node = malloc(sizeof(o_rnode) * (size_t)(q->nleaf + q->nnode));
                t->body = malloc(sizeof(double) * 3 * (size_t)q->n);
                if (!t->node || !t->body) { rc = PO_ERR_NOMEM; break; }
                export_node(q, q->first_node, rcen, rwid, sh, t);
                st[r]->nrt++;
            }
        }
    }
    /* fmm_task and fmm_ext on every rank */
    first = 0;
    for (int r = 0; r < P && !rc; r++) {
        po_state *q = st[r];
        q->walk_m2l_count = 0;
        rc = run_walks(q, p->images && !explicit_self);
        if (rc) break;
        q->p2p_count_remote = ext_pairs(q);
        rc = forces(q, 0, NULL);
        if (rc) break;
        for (int i = 0; i < cnt[r]; i++)
            for (int d = 0; d < 3; d++)
                acc_out[3 * (size_t)order[first + q->perm[i]] + d] = q->acc[3 * (size_t)i + d];
        if (counters) po_counters(q, counters + 16 * (size_t)r);
        first += cnt[r];
    }
    for (int r = 0; r < P && st; r++) {
        if (!st[r]) continue;
        for (int k = 0; k < st[r]->nrt; k++) { free(st[r]->rt[k].node); free(st[r]->rt[k].body); }
        free(st[r]->rt);
        st[r]->rt = NULL;
        st[r]->nrt = 0;
        po_destroy(st[r]);
    }
    free(st); free(box); free(split); free(axis); free(rank); free(cnt); free(fill); free(order); free(lpos);
    return rc;
}

/* fmm_prepare for one rank's domain (its tree over the domain box from its
   first axis, multipoles); po_export then gives its exported trees.  lo,
   hi: the domain's top-tree box. */
int po_prepare_domain(po_state *s, const po_params *p, const double lo[3], const double hi[3], int axis, int n,
                      const double *pos_in)
{
    if (!s || !p || !lo || !hi || axis < 0 || axis > 2) return PO_ERR_ARG;
    set_domain(s, lo, hi, axis);
    double t[2];
    return prepare_pass(s, p, n, pos_in, 0, t);
}

/* A tree received from another rank (layout of po_export), kept for
   po_finish_domain; copied. */
int po_import(po_state *s, int nnode, const void *nodes, int nbody, const double *bodies)
{
    if (!s || !s->node || nnode < 0 || nbody < 0) return PO_ERR_ARG;
    if (nnode == 0) return PO_OK;
    o_rtree *rt = realloc(s->rt, sizeof(o_rtree) * (size_t)(s->nrt + 1));
    if (!rt) return PO_ERR_NOMEM;
    s->rt = rt;
    o_rtree *t = &s->rt[s->nrt];
    t->nnode = nnode;
    t->nbody = nbody;
    t->node = malloc(sizeof(o_rnode) * (size_t)nnode);
    t->body = malloc(sizeof(double) * 3 * (size_t)(nbody ? nbody : 1));
    if (!t->node || !t->body) { free(t->node); free(t->body); return PO_ERR_NOMEM; }
    memcpy(t->node, nodes, sizeof(o_rnode) * (size_t)nnode);
    if (nbody) memcpy(t->body, bodies, sizeof(double) * 3 * (size_t)nbody);
    s->nrt++;
    return PO_OK;
}

/* fmm_task and fmm_ext of a prepared domain over the trees received so far
   (own periodic images on the fly); acc_out[3n] in the prepared positions'
   order; the received trees are released */
int po_finish_domain(po_state *s, double *acc_out)
{
    if (!s || !s->node || !acc_out) return PO_ERR_ARG;
    s->walk_m2l_count = 0;
    int rc = run_walks(s, s->p.images);
    if (!rc) {
        s->p2p_count_remote = ext_pairs(s);
        rc = forces(s, 0, NULL);
    }
    if (!rc)
        for (int i = 0; i < s->n; i++)
            for (int d = 0; d < 3; d++) acc_out[3 * (size_t)s->perm[i] + d] = s->acc[3 * (size_t)i + d];
    for (int k = 0; k < s->nrt; k++) { free(s->rt[k].node); free(s->rt[k].body); }
    free(s->rt);
    s->rt = NULL;
    s->nrt = 0;
    return rc;
}

void po_counters(const po_state *s, long long *c)
{
    c[0] = s->list[PO_LIST_P2P].n;
    c[1] = s->list[PO_LIST_M2L].n;
    c[2] = s->walk_m2l_count;
    c[3] = s->p2p_count_remote;
    c[4] = s->nleaf_cap;
    c[5] = s->nnode_cap;
    c[6] = s->nleaf;
    c[7] = s->nnode;
    c[8] = s->first_leaf;
    c[9] = s->first_node;
    c[10] = 0;
    c[11] = s->list[PO_LIST_P2P].n;
    c[12] = s->list[PO_LIST_M2L].n;
    c[13] = s->list[PO_LIST_P2P_EXT].n;
    c[14] = s->list[PO_LIST_M2L_EXT].n;
    c[15] = s->p.images ? NIMG - 1 : 0;
}

void po_particles(const po_state *s, double *pos, double *acc_task, double *acc, int *perm)
{
    size_t b = sizeof(double) * 3 * (size_t)s->n;
    if (pos) memcpy(pos, s->pos, b);
    if (acc_task) memcpy(acc_task, s->acc_task, b);
    if (acc) memcpy(acc, s->acc, b);
    if (perm) memcpy(perm, s->perm, sizeof(int) * (size_t)s->n);
}

long po_list_size(const po_state *s, int kind) { return (kind >= 0 && kind < 4) ? s->list[kind].n : -1; }

void po_list_copy(const po_state *s, int kind, int *t, int *src, int *img)
{
    const o_list *l = &s->list[kind];
    memcpy(t, l->t, sizeof(int) * l->n);
    memcpy(src, l->s, sizeof(int) * l->n);
    memcpy(img, l->img, sizeof(int) * l->n);
}

void po_copy_leaves(const po_state *s, int *ip_np, double *geom, double *M, double *L)
{
    for (int i = 0; i < s->nleaf; i++) {
        const o_leaf *p = &s->leaf[i];
        ip_np[2 * i] = p->ipart; ip_np[2 * i + 1] = p->npart;
        for (int d = 0; d < 3; d++) { geom[6 * i + d] = p->center[d]; geom[6 * i + 3 + d] = p->width[d]; }
        memcpy(M + NM * i, p->M, sizeof p->M);
        memcpy(L + NM * i, p->L, sizeof p->L);
    }
}

void po_copy_nodes(const po_state *s, int *info, double *geom, double *M, double *L)
{
    for (int i = 0; i < s->nnode; i++) {
        const o_node *p = &s->node[i];
        info[3 * i] = p->npart; info[3 * i + 1] = p->son[0]; info[3 * i + 2] = p->son[1];
        geom[7 * i] = p->split;
        for (int d = 0; d < 3; d++) { geom[7 * i + 1 + d] = p->center[d]; geom[7 * i + 4 + d] = p->width[d]; }
        memcpy(M + NM * i, p->M, sizeof p->M);
        memcpy(L + NM * i, p->L, sizeof p->L);
    }
}

/* ------------------------------------------------------------------ */
/* FP64 direct sum (error oracle)                                      */
/* ------------------------------------------------------------------ */
typedef struct {
    const po_params *p;
    int n, nt;
    const double *pos;
    const int *targets;
    double rmax;
    double *acc;
    int ncell;
    double cell;
    const int *head, *next;
    int cursor;
    pthread_mutex_t mu;
} ds_job;

static inline double min_image(double d, double L)
{
    if (d > 0.5 * L) d -= L;
    else if (d < -0.5 * L) d += L;
    return d;
}

static void ds_one(ds_job *J, int t)
{
    const po_params *p = J->p;
    int i = J->targets[t];
    const double *pi = J->pos + 3 * i;
    double coeff = 2.0 / sqrt(M_PI), L = p->boxsize, r2max = J->rmax * J->rmax;
    double a[3] = {0, 0, 0};
    int ci[3];
    for (int d = 0; d < 3; d++) {
        ci[d] = (int)(pi[d] / J->cell);
        if (ci[d] >= J->ncell) ci[d] = J->ncell - 1;
        if (ci[d] < 0) ci[d] = 0;
    }
    int span = J->ncell >= 3 ? 1 : 0;
    int lo = J->ncell >= 3 ? -1 : 0, hi = J->ncell >= 3 ? 1 : 0;
    (void)span;
    if (J->ncell < 3) { lo = 0; hi = 0; }
    for (int ox = lo; ox <= hi; ox++)
        for (int oy = lo; oy <= hi; oy++)
            for (int oz = lo; oz <= hi; oz++) {
                int cx = (ci[0] + ox + J->ncell) % J->ncell, cy = (ci[1] + oy + J->ncell) % J->ncell,
                    cz = (ci[2] + oz + J->ncell) % J->ncell;
                int c = (cx * J->ncell + cy) * J->ncell + cz;
                if (J->ncell < 3) c = -1;
                int j = (c >= 0) ? J->head[c] : 0;
                for (; (c >= 0) ? (j >= 0) : (j < J->n); j = (c >= 0) ? J->next[j] : j + 1) {
                    if (j == i) continue;
                    const double *pj = J->pos + 3 * j;
                    double dx0 = min_image(pj[0] - pi[0], L), dx1 = min_image(pj[1] - pi[1], L),
                           dx2 = min_image(pj[2] - pi[2], L);
                    double r2 = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
                    if (r2 >= r2max) continue;
                    double dr = sqrt(r2);
                    double ir3 = (dr < p->eps) ? p->mass / (p->eps * p->eps * p->eps) : p->mass / (dr * dr * dr);
                    double drs = 0.5 * dr / p->rs;
                    ir3 *= (erfc(drs) + coeff * drs * exp(-drs * drs));
                    a[0] += dx0 * ir3; a[1] += dx1 * ir3; a[2] += dx2 * ir3;
                }
            }
    for (int d = 0; d < 3; d++) J->acc[3 * t + d] = a[d];
}

static void *ds_worker(void *arg)
{
    ds_job *J = arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int t = J->cursor;
        J->cursor += 8;
        pthread_mutex_unlock(&J->mu);
        if (t >= J->nt) break;
        int e = t + 8 < J->nt ? t + 8 : J->nt;
        for (; t < e; t++) ds_one(J, t);
    }
    return 0;
}

int po_direct_sum(const po_params *p, int n, const double *pos, int nt, const int *targets, double rmax,
                  double *acc_out)
{
    if (!p || n < 1 || nt < 0 || rmax <= 0) return PO_ERR_ARG;
    ds_job J;
    memset(&J, 0, sizeof J);
    J.p = p; J.n = n; J.nt = nt; J.pos = pos; J.targets = targets; J.rmax = rmax; J.acc = acc_out;
    int ncell = (int)(p->boxsize / rmax);
    if (ncell > 256) ncell = 256;
    if (ncell < 1) ncell = 1;
    J.ncell = ncell;
    J.cell = p->boxsize / ncell;
    int *head = NULL, *next = NULL;
    if (ncell >= 3) {
        head = malloc(sizeof(int) * (size_t)ncell * ncell * ncell);
        next = malloc(sizeof(int) * (size_t)n);
        if (!head || !next) { free(head); free(next); return PO_ERR_NOMEM; }
        for (long c = 0; c < (long)ncell * ncell * ncell; c++) head[c] = -1;
        for (int j = n - 1; j >= 0; j--) {
            int cc[3];
            for (int d = 0; d < 3; d++) {
                cc[d] = (int)(pos[3 * j + d] / J.cell);
                if (cc[d] >= ncell) cc[d] = ncell - 1;
                if (cc[d] < 0) cc[d] = 0;
            }
            int c = (cc[0] * ncell + cc[1]) * ncell + cc[2];
            next[j] = head[c];
            head[c] = j;
        }
    }
    J.head = head; J.next = next;
    pthread_mutex_init(&J.mu, 0);
    int nth = p->nthreads > 1 ? p->nthreads : 1;
    if (nth == 1) ds_worker(&J);
    else {
        pthread_t *th = malloc(sizeof(pthread_t) * nth);
        for (int i = 0; i < nth; i++) pthread_create(&th[i], 0, ds_worker, &J);
        for (int i = 0; i < nth; i++) pthread_join(th[i], 0);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    free(head);
    free(next);
    return PO_OK;
}

/* ------------------------------------------------------------------ */
/* time integration                                                     */
/* ------------------------------------------------------------------ */

/* Simpson's rule with 128 intervals in log a of z^zpow / h, h = 0.1 sqrt(Om z^3
   + OL), z = 1/a; weights 1, 4, 2, 4, ..., 4, 1 accumulated in index order
   (src/initial.c:639-683, whose kick uses zpow 1 and drift zpow 2). */
static double po_loga_simpson(double om, double ox, double la, double lb, int zpow)
{
    const int nb = 128;
    double dl = (lb - la) / nb;
    double z = 1.0 / exp(la);
    double h = 0.1 * sqrt(om * z * z * z + ox);
    double acc = zpow == 1 ? dl * z / h : dl * z * z / h;
    for (int k = 1; k < nb; k++) {
        z = 1.0 / (exp(la + dl * k));
        h = 0.1 * sqrt(om * z * z * z + ox);
        acc += zpow == 1 ? 2.0 * (1 + k % 2) * dl * z / h : 2.0 * (1 + k % 2) * dl * z * z / h;
    }
    z = 1.0 / exp(lb);
    h = 0.1 * sqrt(om * z * z * z + ox);
    acc += zpow == 1 ? dl * z / h : dl * z * z / h;
    return acc / 3.0;
}

double po_kick_loga(double omega_m, double omega_x, double loga_i, double loga_f)
{
    return po_loga_simpson(omega_m, omega_x, loga_i, loga_f, 1);
}

double po_drift_loga(double omega_m, double omega_x, double loga_i, double loga_f)
{
    return po_loga_simpson(omega_m, omega_x, loga_i, loga_f, 2);
}

/* src/photoNs.c:164-174: one velocity update per coordinate */
void po_kick(long long m, double *vel, const double *acc, double dkh)
{
    for (long long i = 0; i < m; i++) vel[i] += acc[i] * dkh;
}

/* src/photoNs.c:176-196: move, then bring each coordinate back into [0, L) */
void po_drift(long long m, double *pos, const double *vel, double dd, double L)
{
    for (long long i = 0; i < m; i++) {
        double x = pos[i] + vel[i] * dd;
        while (x < 0.0) x += L;
        while (x >= L) x -= L;
        pos[i] = x;
    }
}
