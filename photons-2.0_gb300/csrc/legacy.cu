// The reference's FMM entry points (inc/fmm.h, inc/operator.h,
// inc/remotes.h, inc/photoNs.h:325) with unchanged names and signatures.
//
// They read and write the reference's globals exactly as src/fmm.c,
// src/operator.c and src/remotes.c do, so the reference driver
// (src/photoNs.c:97-116, 229-254) can call them in place of the CPU FMM:
//   fmm_construct  top-tree geometry of the (single) domain
//   fmm_prepare    GPU tree build + P2M/M2M; part[] permuted into tree
//                  order and btree/leaf filled as build_localtree would
//   fmm_task       local walk, local P2P (added to part[].acc) and local M2L
//   fmm_ext        26 images (P2P and M2L), L2L and L2P, added to part[].acc
// Counters idxP2P, idxM2L, walk_m2l_count and p2p_count_remote advance as
// the reference's do.  Errors print and exit like the reference; the
// photons_gpu_* functions report them without exiting.
//
// The operator.h functions work on host data in FP64 (the reference's
// top-tree code, src/toptree.c:185-244, calls m2m/m2l on host TopNodes);
// the force pass itself never calls them.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "api_internal.cuh"
#include "ref_abi.h"

// ------------------------------------------------------------------
// the reference's globals (tentative definitions in its headers; defined
// here so the library also loads on its own)
// ------------------------------------------------------------------
extern "C" {
Body *part = nullptr;
Node *btree = nullptr;
Pack *leaf = nullptr;
TopNode *toptree = nullptr;
double open_angle = 0.3;
int first_node = 0, last_node = 0, first_leaf = 0, last_leaf = 0, MAXLEAF = 8;
int PROC_RANK = 0, PROC_SIZE = 1;
double BOXSIZE = 0.0;
int NPART = 0, NLEAF = 0, NNODE = 0;
long NPART_TOTAL = 0;
double MASSPART = 0.0, SoftenScale = 0.0, cutoffRadius = 0.0, splitRadius = 0.0;
int first_domain = 0, last_domain = 0, this_domain = 0, mostleft = 0, direct_local_start = 0;
double width_this_domain = 0.0;
int *ExtDomain = nullptr;
REF_INT64 idxP2P = 0, idxM2L = 0, walk_m2l_count = 0, p2p_count_remote = 0, m2l_count = 0;
double dtime_p2p = 0, dtime_m2l = 0, dtime_fmm = 0, dtime_task = 0, dtime_ext = 0, dtime_prep = 0,
       dtime_fmm_remote = 0;
double DTIME_THIS_DOMAIN = 0.0;
int NSIDE = 0;          // PM mesh side (inc/photoNs.h:58)
double dtime_pm = 0.0;  // inc/photoNs.h:107
}

static photons_ctx *g_ctx = nullptr;
static std::vector<double> g_stage;  // host staging for positions / accelerations
static Pack *g_leaf_base = nullptr;
static Node *g_node_base = nullptr;

static double wall()
{
    struct timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void fatal(const char *where)
{
    printf(" photons %s: %s\n", where, photons_gpu_error());
    fflush(stdout);
    exit(1);
}

static photons_ctx *ctx()
{
    if (!g_ctx) {
        g_ctx = photons_create(0);
        if (!g_ctx) fatal("context");
    }
    return g_ctx;
}

static photons_params legacy_params()
{
    photons_params p;
    memset(&p, 0, sizeof p);
    p.boxsize = BOXSIZE;
    p.theta = open_angle;
    p.rs = splitRadius;
    p.rcut = cutoffRadius;
    p.eps = SoftenScale;
    p.mass = MASSPART;
    p.maxleaf = MAXLEAF;
    p.precision = PHOTONS_FP64;
    const char *prec = getenv("PHOTONS_PRECISION");
    if (prec && (!strcmp(prec, "fp32") || !strcmp(prec, "split"))) p.precision = PHOTONS_FP32_SPLIT;
    return p;
}

// src/fmm.c:329-360 at one rank: the domain is the whole periodic box
extern "C" void fmm_construct(void)
{
    photons_gpu_clear_error();
    if (PROC_SIZE != 1) {
        ph_set_error(PH_ERR_UNSUPPORTED, "PROC_SIZE=%d: only the single-GPU, single-rank pass is provided", PROC_SIZE);
        fatal("fmm_construct");
    }
    if (!toptree) toptree = (TopNode *)calloc(1, sizeof(TopNode));
    first_domain = last_domain = this_domain = mostleft = 0;
    toptree[0].son[0] = toptree[0].son[1] = -1;
    // center_toptree(0, 0, {0,0,0}, {L,L,L}), src/toptree.c:150-182
    for (int d = 0; d < 3; d++) {
        toptree[0].width[d] = BOXSIZE - 0.0;
        toptree[0].center[d] = 0.5 * (BOXSIZE + 0.0);
    }
    direct_local_start = 0;
}

static void free_host_tree()
{
    free(g_leaf_base);
    free(g_node_base);
    g_leaf_base = nullptr;
    g_node_base = nullptr;
    leaf = nullptr;
    btree = nullptr;
}

// GPU build + host mirror of the tree in the reference's layout
static void build_and_mirror(bool multipoles)
{
    photons_ctx *c = ctx();
    photons_params p = legacy_params();
    if (!part || NPART < 1) { ph_set_error(PH_ERR_ARG, "no particles"); fatal("fmm_prepare"); }
    g_stage.resize((size_t)3 * NPART);
    for (int i = 0; i < NPART; i++)
        for (int d = 0; d < 3; d++) g_stage[3 * (size_t)i + d] = part[i].pos[d];
    if (ph_stage_build(c, &p, NPART, g_stage.data(), 0)) fatal("fmm_prepare");
    if (multipoles && ph_stage_multipoles(c)) fatal("fmm_prepare");
    // permute part[] into tree order (src/fmm.c:30-78 moves whole Body records)
    std::vector<int> perm(NPART);
    if (photons_get_perm(c, perm.data())) fatal("fmm_prepare");
    std::vector<Body> tmp(part, part + NPART);
    for (int i = 0; i < NPART; i++) part[i] = tmp[perm[i]];
    // host tree in the reference's index space (src/fmm.c:203-259)
    HostTree h;
    if (ph_download_tree(c, h, true)) fatal("fmm_prepare");
    NLEAF = NNODE = c->info.nleaf_cap;
    free_host_tree();
    g_leaf_base = (Pack *)calloc((size_t)NLEAF, sizeof(Pack));
    g_node_base = (Node *)calloc((size_t)NNODE, sizeof(Node));
    if (!g_leaf_base || !g_node_base) { ph_set_error(PH_ERR_NOMEM, "host tree"); fatal("fmm_prepare"); }
    first_leaf = NPART;
    last_leaf = NPART + h.nleaf;
    first_node = NPART + NLEAF;
    last_node = first_node + h.nnode - 1;
    for (int n = 0; n < NNODE; n++) g_node_base[n].son[0] = g_node_base[n].son[1] = -1;
    auto rid = [&](int u) { return u < h.nleaf ? first_leaf + u : first_node + (u - h.nleaf); };
    for (int u = 0; u < h.nleaf; u++) {
        Pack &q = g_leaf_base[u];
        q.npart = h.npart[u];
        q.ipart = h.ipart[u];
        q.center[0] = h.cx[u]; q.center[1] = h.cy[u]; q.center[2] = h.cz[u];
        q.width[0] = h.wx[u]; q.width[1] = h.wy[u]; q.width[2] = h.wz[u];
        for (int m = 0; m < REF_NMULTI; m++) q.M[m] = h.M[(size_t)u * PH_NMULTI + m];
    }
    for (int k = 0; k < h.nnode; k++) {
        int u = h.nleaf + k;
        Node &q = g_node_base[k];
        q.npart = h.npart[u];
        q.son[0] = rid(h.son0[u]);
        q.son[1] = rid(h.son1[u]);
        q.split = h.split[u];
        q.center[0] = h.cx[u]; q.center[1] = h.cy[u]; q.center[2] = h.cz[u];
        q.width[0] = h.wx[u]; q.width[1] = h.wy[u]; q.width[2] = h.wz[u];
        for (int m = 0; m < REF_NMULTI; m++) q.M[m] = h.M[(size_t)u * PH_NMULTI + m];
    }
    // the reference indexes btree/leaf with its global ids
    btree = g_node_base - first_node;
    leaf = g_leaf_base - first_leaf;
}

extern "C" void build_localtree(void)
{
    photons_gpu_clear_error();
    build_and_mirror(false);
}

// src/fmm.c:719-770
extern "C" void fmm_prepare(void)
{
    photons_gpu_clear_error();
    double t0 = wall();
    m2l_count = 0;
    build_and_mirror(true);
    // connect_local_toptree at one rank (src/toptree.c:11-50): the domain
    // node takes the root's box and multipoles
    if (toptree) {
        Node &r = btree[first_node];
        for (int d = 0; d < 3; d++) { toptree[0].width[d] = r.width[d]; toptree[0].center[d] = r.center[d]; }
        for (int m = 0; m < REF_NMULTI; m++) toptree[0].M[m] = r.M[m];
        width_this_domain = toptree[0].width[0];
        if (width_this_domain < toptree[0].width[1]) width_this_domain = toptree[0].width[1];
        if (width_this_domain < toptree[0].width[2]) width_this_domain = toptree[0].width[2];
    }
    free(ExtDomain);
    ExtDomain = (int *)calloc((size_t)PROC_SIZE, sizeof(int));
    idxM2L = 0;
    idxP2P = 0;
    dtime_prep = wall() - t0;
    dtime_fmm = dtime_prep;
}

// run one walk over the selected images, P2P into part[].acc, M2L into L
static void interact(unsigned mask, bool downward)
{
    photons_ctx *c = ctx();
    photons_params p = legacy_params();
    if (!c->have_tree) { ph_set_error(PH_ERR_STATE, "fmm_prepare has not run"); fatal("fmm_task"); }
    if (ph_stage_walk(c, mask)) fatal("walk");
    if (ph_stage_p2p(c, p.precision, 1)) fatal("p2p");
    unsigned long long nm2l = c->ws.c[ph::WC_M2L_LOCAL] + c->ws.c[ph::WC_M2L_IMAGE];
    if (nm2l && ph_stage_m2l(c, p.precision)) fatal("m2l");
    if (downward && ph_stage_downward(c, p.precision)) fatal("l2l/l2p");
    if (ph_stage_output(c, g_stage.data(), 0, 1)) fatal("download");
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) { ph_set_error(PH_ERR_CUDA, "stream"); fatal("sync"); }
    for (int i = 0; i < NPART; i++)
        for (int d = 0; d < 3; d++) part[i].acc[d] += g_stage[3 * (size_t)i + d];
    if (nm2l || downward) {
        // local expansions back into the host tree, as the reference keeps them
        HostTree h;
        if (ph_download_tree(c, h, true)) fatal("download");
        for (int u = 0; u < h.nleaf; u++)
            for (int m = 0; m < REF_NMULTI; m++) g_leaf_base[u].L[m] = h.L[(size_t)u * PH_NMULTI + m];
        for (int k = 0; k < h.nnode; k++)
            for (int m = 0; m < REF_NMULTI; m++) g_node_base[k].L[m] = h.L[(size_t)(h.nleaf + k) * PH_NMULTI + m];
    }
}

// src/fmm.c:909-984
extern "C" void fmm_task(void)
{
    photons_gpu_clear_error();
    double t0 = wall();
    interact(1u, false);
    photons_ctx *c = ctx();
    idxP2P += c->ws.c[ph::WC_P2P_LOCAL];
    idxM2L += c->ws.c[ph::WC_M2L_LOCAL];
    walk_m2l_count += c->ws.c[ph::WC_M2L_LOCAL];
    dtime_task = wall() - t0;
}

// src/fmm.c:987-1075 (PERIODIC_CONDITION build: 26 images at one rank)
extern "C" void fmm_ext(void)
{
    photons_gpu_clear_error();
    double t0 = wall();
    interact(((1u << PH_NIMG) - 1u) & ~1u, true);
    photons_ctx *c = ctx();
    walk_m2l_count += c->ws.c[ph::WC_M2L_IMAGE];
    p2p_count_remote += c->ws.c[ph::WC_PAIRS_IMAGE];
    DTIME_THIS_DOMAIN = (double)(idxP2P + idxM2L);
    dtime_ext = wall() - t0;
    dtime_fmm_remote = dtime_ext;
}

// src/remotes.c:684-751 at one rank: idx 0, shift one of the 26 image offsets
extern "C" void fmm_remote(int idx, double shift[3])
{
    photons_gpu_clear_error();
    if (idx != 0 || PROC_SIZE != 1) {
        ph_set_error(PH_ERR_UNSUPPORTED, "fmm_remote(%d): only the single-rank periodic self-exchange is provided", idx);
        fatal("fmm_remote");
    }
    int o[3];
    for (int d = 0; d < 3; d++) {
        double q = shift[d] / BOXSIZE;
        o[d] = (int)lround(q);
        if (o[d] < -1 || o[d] > 1 || fabs(q - o[d]) > 1e-12) {
            ph_set_error(PH_ERR_ARG, "shift is not a periodic image offset");
            fatal("fmm_remote");
        }
    }
    if (!o[0] && !o[1] && !o[2]) { ph_set_error(PH_ERR_ARG, "zero shift"); fatal("fmm_remote"); }
    int cell = (o[0] + 1) * 9 + (o[1] + 1) * 3 + (o[2] + 1);
    int img = cell < 13 ? cell + 1 : cell;
    interact(1u << img, false);
    photons_ctx *c = ctx();
    walk_m2l_count += c->ws.c[ph::WC_M2L_IMAGE];
    p2p_count_remote += c->ws.c[ph::WC_PAIRS_IMAGE];
}

// ------------------------------------------------------------------
// inc/kernels.h:4-8: one local P2P task, leaf inode's particles from leaf
// jnode's (reference leaf ids, after fmm_prepare), on the GPU in FP64 and
// added to part[].acc as src/fmm.c:823-868 adds a task.  The reference
// declares these three but never defines them; here
//   p2p_kernel           the pair force as src/fmm.c:834-852 writes it
//                        (sqrt, division, erfc, exp)
//   p2p_kernel_rinvsqrt  the same force with 1/r from the reciprocal
//                        square root and the split factor from piecewise
//                        polynomials (the FP64 pass's form)
//   p2p_kernel_inleaf    a leaf with itself (jnode must equal inode), self
//                        pairs skipped
// ------------------------------------------------------------------
static double *g_pair_dev = nullptr;  // [targets | sources | out], 3 doubles per particle each
static int g_pair_cap = 0;
static std::vector<double> g_pair_host;

static void leaf_pair(int inode, int jnode, int exact, const char *who)
{
    photons_gpu_clear_error();
    if (!leaf || !part) { ph_set_error(PH_ERR_STATE, "%s: fmm_prepare has not run", who); fatal(who); }
    if (inode < first_leaf || inode >= last_leaf || jnode < first_leaf || jnode >= last_leaf) {
        ph_set_error(PH_ERR_ARG, "%s(%d, %d): leaf ids must lie in [%d, %d)", who, inode, jnode, first_leaf, last_leaf);
        fatal(who);
    }
    photons_ctx *c = ctx();
    const Pack &T = leaf[inode], &S = leaf[jnode];
    const int cap = T.npart > S.npart ? T.npart : S.npart;
    if (cap > g_pair_cap) {
        cudaFree(g_pair_dev);
        g_pair_dev = nullptr;
        g_pair_cap = 0;
        if (cudaMalloc(&g_pair_dev, sizeof(double) * 9 * (size_t)cap) != cudaSuccess) {
            cudaGetLastError();
            ph_set_error(PH_ERR_NOMEM, "%s: device buffer", who);
            fatal(who);
        }
        g_pair_cap = cap;
    }
    g_pair_host.resize((size_t)3 * (T.npart + S.npart));
    for (int q = 0; q < T.npart; q++)
        for (int d = 0; d < 3; d++) g_pair_host[3 * (size_t)q + d] = part[T.ipart + q].pos[d];
    for (int q = 0; q < S.npart; q++)
        for (int d = 0; d < 3; d++) g_pair_host[3 * (size_t)(T.npart + q) + d] = part[S.ipart + q].pos[d];
    double *dt = g_pair_dev, *ds = g_pair_dev + 3 * (size_t)cap, *dout = g_pair_dev + 6 * (size_t)cap;
    cudaStream_t st = c->stream;
    cudaError_t e = cudaMemcpyAsync(dt, g_pair_host.data(), sizeof(double) * 3 * T.npart, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ds, g_pair_host.data() + 3 * (size_t)T.npart, sizeof(double) * 3 * S.npart,
                            cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { ph_set_cuda_error(e, "cudaMemcpyAsync", __FILE__, __LINE__); fatal(who); }
    if (ph::launch_leaf_pair_fp64(dt, T.npart, T.ipart, ds, S.npart, S.ipart, SoftenScale, MASSPART, splitRadius, exact,
                                  dout, st))
        fatal(who);
    e = cudaMemcpyAsync(g_pair_host.data(), dout, sizeof(double) * 3 * T.npart, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { ph_set_cuda_error(e, "leaf pair", __FILE__, __LINE__); fatal(who); }
    for (int q = 0; q < T.npart; q++)
        for (int d = 0; d < 3; d++) part[T.ipart + q].acc[d] += g_pair_host[3 * (size_t)q + d];
}

extern "C" void p2p_kernel(int inode, int jnode) { leaf_pair(inode, jnode, 1, "p2p_kernel"); }

extern "C" void p2p_kernel_rinvsqrt(int inode, int jnode) { leaf_pair(inode, jnode, 0, "p2p_kernel_rinvsqrt"); }

extern "C" void p2p_kernel_inleaf(int inode, int jnode)
{
    if (inode != jnode) {
        photons_gpu_clear_error();
        ph_set_error(PH_ERR_ARG, "p2p_kernel_inleaf(%d, %d): a leaf with itself takes equal ids", inode, jnode);
        fatal("p2p_kernel_inleaf");
    }
    leaf_pair(inode, inode, 1, "p2p_kernel_inleaf");
}

// src/fmm.c:1077-1087
extern "C" void fmm_deconstruct(void)
{
    free_host_tree();
    free(ExtDomain);
    ExtDomain = nullptr;
    free(toptree);
    toptree = nullptr;
}

// ------------------------------------------------------------------
// host operators (FP64), same expansions as the device operators
// ------------------------------------------------------------------
namespace {
struct HMI {
    int e[20][3], ord[20], idx[4][4][4];
    double invf[20];
    HMI()
    {
        int i = 0;
        for (int k = 0; k <= 3; k++)
            for (int a = k; a >= 0; a--)
                for (int b = k - a; b >= 0; b--) {
                    int c = k - a - b;
                    e[i][0] = a; e[i][1] = b; e[i][2] = c; ord[i] = k; idx[a][b][c] = i;
                    double f = 1;
                    for (int q = 2; q <= a; q++) f *= q;
                    for (int q = 2; q <= b; q++) f *= q;
                    for (int q = 2; q <= c; q++) f *= q;
                    invf[i] = 1.0 / f;
                    i++;
                }
    }
};
const HMI &mi()
{
    static HMI t;
    return t;
}
void mono(double dx, double dy, double dz, double *out)
{
    const HMI &t = mi();
    double px[4] = {1, dx, dx * dx, dx * dx * dx}, py[4] = {1, dy, dy * dy, dy * dy * dy},
           pz[4] = {1, dz, dz * dz, dz * dz * dz};
    for (int i = 0; i < 20; i++) out[i] = px[t.e[i][0]] * py[t.e[i][1]] * pz[t.e[i][2]] * t.invf[i];
}
}  // namespace

// src/operator.c:13-93
extern "C" void p2m(int iPart, int npart, double center[3], double M[])
{
    double m[20];
    for (int i = 0; i < 20; i++) M[i] = 0.0;
    for (int p = iPart; p < iPart + npart; p++) {
        mono(-(part[p].pos[0] - center[0]), -(part[p].pos[1] - center[1]), -(part[p].pos[2] - center[2]), m);
        for (int i = 0; i < 20; i++) M[i] += MASSPART * m[i];
    }
}

// src/operator.c:96-160
extern "C" void m2m(double dx, double dy, double dz, double M[], double tM[])
{
    const HMI &t = mi();
    double m[20], out[20];
    mono(dx, dy, dz, m);
    for (int a = 0; a < 20; a++) {
        double s = 0;
        for (int b = 0; b < 20; b++) {
            int g0 = t.e[a][0] - t.e[b][0], g1 = t.e[a][1] - t.e[b][1], g2 = t.e[a][2] - t.e[b][2];
            if (g0 < 0 || g1 < 0 || g2 < 0) continue;
            s += M[b] * m[t.idx[g0][g1][g2]];
        }
        out[a] = s;
    }
    for (int a = 0; a < 20; a++) tM[a] += out[a];
}

// src/operator.c:255-392 (LONGSHORT)
extern "C" void m2l(double dx, double dy, double dz, double M[], double toL[])
{
    const HMI &t = mi();
    walk_m2l_count++;
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    double a = 0.5 / splitRadius, a2 = a * a, u = a * r;
    double ce = 1.1283791670955126 * exp(-u * u), er = erfc(u);
    double ir = 1.0 / r, ir2 = ir * ir;
    double f[4] = {er * ir, -er * ir * ir2 - ce * a * ir2,
                   3.0 * er * ir * ir2 * ir2 + ce * (3.0 * a * ir2 * ir2 + 2.0 * a * a2 * ir2),
                   -15.0 * er * ir * ir2 * ir2 * ir2 -
                       ce * (15.0 * a * ir2 * ir2 * ir2 + 10.0 * a * a2 * ir2 * ir2 + 4.0 * a * a2 * a2 * ir2)};
    double x[3] = {dx, dy, dz}, D[20];
    for (int g = 0; g < 20; g++) {
        int e[3] = {t.e[g][0], t.e[g][1], t.e[g][2]}, k = t.ord[g];
        double v = f[k] * std::pow(x[0], e[0]) * std::pow(x[1], e[1]) * std::pow(x[2], e[2]);
        if (k >= 2)
            for (int d = 0; d < 3; d++) {
                if (e[d] < 2) continue;
                int ee[3] = {e[0], e[1], e[2]};
                ee[d] -= 2;
                v += f[k - 1] * (e[d] * (e[d] - 1) / 2) * std::pow(x[0], ee[0]) * std::pow(x[1], ee[1]) *
                     std::pow(x[2], ee[2]);
            }
        D[g] = v;
    }
    for (int b = 0; b < 20; b++) {
        double s = 0;
        for (int aa = 0; aa < 20; aa++) {
            if (t.ord[aa] + t.ord[b] > 3) continue;
            s += M[aa] * D[t.idx[t.e[aa][0] + t.e[b][0]][t.e[aa][1] + t.e[b][1]][t.e[aa][2] + t.e[b][2]]];
        }
        toL[b] += s;
    }
}

// src/operator.c:395-494
extern "C" void l2l(double dx, double dy, double dz, double L[], double toL[])
{
    const HMI &t = mi();
    double m[20];
    mono(dx, dy, dz, m);
    for (int b = 0; b < 20; b++) {
        double s = 0;
        for (int g = 0; g < 20; g++) {
            if (t.ord[b] + t.ord[g] > 3) continue;
            s += L[t.idx[t.e[b][0] + t.e[g][0]][t.e[b][1] + t.e[g][1]][t.e[b][2] + t.e[g][2]]] * m[g];
        }
        toL[b] += s;
    }
}

// src/operator.c:197-251
extern "C" void l2p(int ileaf)
{
    const HMI &t = mi();
    const Pack &q = leaf[ileaf];
    double m[20];
    for (int n = q.ipart; n < q.ipart + q.npart; n++) {
        mono(part[n].pos[0] - q.center[0], part[n].pos[1] - q.center[1], part[n].pos[2] - q.center[2], m);
        for (int i = 0; i < 3; i++) {
            double s = 0;
            for (int g = 0; g < 20; g++) {
                if (t.ord[g] > 2) continue;
                int e[3] = {t.e[g][0], t.e[g][1], t.e[g][2]};
                e[i]++;
                s += q.L[t.idx[e[0]][e[1]][e[2]]] * m[g];
            }
            part[n].acc[i] += s;
        }
    }
}

// src/operator.c:165-194
extern "C" void walk_m2m(int iNode)
{
    for (int n = 0; n < 2; n++) {
        int idx = btree[iNode].son[n];
        if (idx < first_node) {
            m2m(btree[iNode].center[0] - leaf[idx].center[0], btree[iNode].center[1] - leaf[idx].center[1],
                btree[iNode].center[2] - leaf[idx].center[2], leaf[idx].M, btree[iNode].M);
        } else {
            walk_m2m(idx);
            m2m(btree[iNode].center[0] - btree[idx].center[0], btree[iNode].center[1] - btree[idx].center[1],
                btree[iNode].center[2] - btree[idx].center[2], btree[idx].M, btree[iNode].M);
        }
    }
}

// src/operator.c:498-528
extern "C" void walk_l2l(int inode)
{
    if (inode < first_node) return;
    for (int n = 0; n < 2; n++) {
        int idx = btree[inode].son[n];
        if (idx >= first_node) {
            l2l(btree[idx].center[0] - btree[inode].center[0], btree[idx].center[1] - btree[inode].center[1],
                btree[idx].center[2] - btree[inode].center[2], btree[inode].L, btree[idx].L);
            walk_l2l(idx);
        } else if (idx >= first_leaf) {
            l2l(leaf[idx].center[0] - btree[inode].center[0], leaf[idx].center[1] - btree[inode].center[1],
                leaf[idx].center[2] - btree[inode].center[2], btree[inode].L, leaf[idx].L);
        } else {
            return;
        }
    }
}

// src/fmm.c:266-326 (LONGSHORT), FP64 without contraction
extern "C" int acceptance(double wi[3], double wj[3], double dist[3])
{
    volatile double w[3], gap[3];
    for (int d = 0; d < 3; d++) w[d] = (wi[d] + wj[d]) * 0.5;
    volatile double s0 = dist[0] * dist[0], s1 = dist[1] * dist[1], s2 = dist[2] * dist[2];
    double dd2 = s0 + s1 + s2;
    for (int d = 0; d < 3; d++) {
        double g = fabs(dist[d]) - w[d];
        gap[d] = g <= 0.0 ? 0.0 : g;
    }
    if (gap[0] + gap[1] + gap[2] < 0.0001) return 0;
    volatile double g0 = gap[0] * gap[0], g1 = gap[1] * gap[1], g2 = gap[2] * gap[2];
    double dm2 = g0 + g1 + g2;
    double c2 = cutoffRadius * cutoffRadius;
    if (dm2 >= c2) return -1;
    if (dd2 > c2) return 0;
    double wmax = w[0];
    if (w[1] > wmax) wmax = w[1];
    if (w[2] > wmax) wmax = w[2];
    wmax *= 2;
    volatile double lhs = wmax * wmax, th2 = open_angle * open_angle;
    volatile double rhs = th2 * dd2;
    return lhs < rhs ? 1 : 0;
}

// ------------------------------------------------------------------
// the reference's PM entry points (inc/partmesh.h:16-21), on the GPU
// ------------------------------------------------------------------
// The reference driver runs pm_thread on a second host thread while the
// FMM runs (src/photoNs.c:104, 237), so the PM keeps a context (stream,
// mesh buffers, FFT plans) of its own and shares nothing with the FMM's.
static photons_ctx *g_pm_ctx = nullptr;
static std::vector<double> g_pm_stage;

// src/partmesh.c:18-795 (the -DPMTHREAD build) and :800-1582: part[].acc_pm
// from part[].pos on an NSIDE^3 mesh with splitRadius, BOXSIZE and
// MASSPART, at one rank (photons_pm_force: CIC deposit, the convolution of
// src/conv.f90:128-247, 4-point gradient, CIC interpolation)
extern "C" void partmesh_thread(void)
{
    photons_gpu_clear_error();
    if (PROC_SIZE != 1) {
        ph_set_error(PH_ERR_UNSUPPORTED, "PROC_SIZE=%d: only the single-GPU, single-rank PM is provided", PROC_SIZE);
        fatal("partmesh");
    }
    const double t0 = wall();
    if (!part || NPART < 1) { ph_set_error(PH_ERR_ARG, "no particles"); fatal("partmesh"); }
    if (!g_pm_ctx) {
        g_pm_ctx = photons_create(0);
        if (!g_pm_ctx) fatal("partmesh");
    }
    photons_params p;
    memset(&p, 0, sizeof p);
    p.boxsize = BOXSIZE;
    p.rs = splitRadius;
    p.mass = MASSPART;
    p.precision = PHOTONS_FP64;
    const size_t n = (size_t)NPART;
    g_pm_stage.resize(6 * n);
    double *pos = g_pm_stage.data(), *acc = pos + 3 * n;
    for (size_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) pos[3 * i + d] = part[i].pos[d];
    if (photons_pm_force(g_pm_ctx, &p, NSIDE, NPART, pos, acc)) fatal("partmesh");
    for (size_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) part[i].acc_pm[d] = acc[3 * i + d];
    dtime_pm = wall() - t0;
}

// src/partmesh.c:800 (the build without PMTHREAD)
extern "C" void partmesh(void) { partmesh_thread(); }

// src/partmesh.c:11-16: the thread entry src/photoNs.c:104 starts
extern "C" void *pm_thread(void *arg)
{
    (void)arg;
    partmesh_thread();
    return nullptr;
}

// src/conv.f90:3-23, called as decomp_2d_init by src/initial.c:226, 468:
// the pencil of one rank is the whole mesh (0-based start and end)
extern "C" void get_local_size_(int *global_size, int *vproc, int *local_start, int *local_end, int *local_size)
{
    if (vproc && vproc[0] * vproc[1] != 1) {
        ph_set_error(PH_ERR_UNSUPPORTED, "vproc %d x %d: only one rank is provided", vproc[0], vproc[1]);
        fatal("get_local_size");
    }
    for (int d = 0; d < 3; d++) {
        local_start[d] = 0;
        local_end[d] = global_size[d] - 1;
        local_size[d] = global_size[d];
    }
}
