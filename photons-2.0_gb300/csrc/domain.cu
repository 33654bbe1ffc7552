// Several ranks, one GPU each: the reference's domain decomposition
// (src/domains.c, src/toptree.c:157-182) and its locally essential trees
// (src/remotes.c:60-169, 684-751).
//
// A rank's pass:  photons_domain_prepare builds the tree of the rank's
// particles over its domain box, starting from the domain's split axis, and
// its multipoles.  photons_let_export writes that tree shifted and pruned
// against another rank's domain, in the reference's RemoteNode/RemoteBody
// layout and depth-first preorder, with four level-synchronous kernels over
// the tree's depth lists (keep/prune top-down, subtree sizes bottom-up,
// preorder indices top-down, then a scatter).  The caller moves the
// messages between ranks.  photons_let_import keeps each received tree;
// photons_domain_finish appends them all to the unified tree (nodes after
// the local ones, bodies after the local particles), so the same walk, P2P
// and M2L kernels serve them: their entries carry the image tag
// PH_IMG_IMPORT (no shift: the sender applied it), a received node is a
// leaf iff it holds <= MAXLEAF particles, and a node sent without children
// is taken by M2L, as src/remotes.c:213-552 walks a received tree.
#include <cmath>
#include <cstring>
#include <vector>

#include "api_internal.cuh"

struct DomainScratch {
    int *work = nullptr;  // six arrays over the unified ids: keep, pruned, nn, nb, pre, bo
    int cap_work = 0;
    photons_remote_node *out_nodes = nullptr;
    photons_remote_body *out_bodies = nullptr;
    int cap_out_nodes = 0, cap_out_bodies = 0;
    photons_remote_node *in_nodes = nullptr;
    photons_remote_body *in_bodies = nullptr;
    int cap_in_nodes = 0, cap_in_bodies = 0;
    int *roots = nullptr;
    int cap_roots = 0;
};

namespace {

// ------------------------------------------------------------------
// domain tree (host): heap order, domains are the leaves P-1 .. 2P-2
// ------------------------------------------------------------------
int most_left(int P)
{
    if (P == 1) return 0;
    int m = 1;
    while (m < 2 * P - 1) m *= 2;
    return m / 2 - 1;
}
int domain_of_rank(int P, int r)
{
    int d = r + most_left(P);
    return d > 2 * P - 2 ? d - P : d;
}
int rank_of_domain(int P, int d) { return (d - most_left(P) + P) % P; }

// time of a domain-tree node: the sum over its domains (src/domains.c:5-19)
double node_time(int P, int id, const std::vector<double> &dom_time)
{
    if (id >= P - 1) return dom_time[id];
    return node_time(P, 2 * id + 1, dom_time) + node_time(P, 2 * id + 2, dom_time);
}

// src/domains.c:400-425: planes dividing each box in the ratio of the times
void volume_part(int P, int id, double bl[3], double br[3], int dim, const std::vector<double> &t, double *split)
{
    if (id >= P - 1) return;
    const double tl = node_time(P, 2 * id + 1, t), tr = node_time(P, 2 * id + 2, t);
    const double frac = bl[dim] + (br[dim] - bl[dim]) * tl / (tl + tr);
    split[id] = frac;
    double keep = br[dim];
    br[dim] = frac;
    volume_part(P, 2 * id + 1, bl, br, (dim + 1) % 3, t, split);
    br[dim] = keep;
    keep = bl[dim];
    bl[dim] = frac;
    volume_part(P, 2 * id + 2, bl, br, (dim + 1) % 3, t, split);
    bl[dim] = keep;
}

// src/toptree.c:157-182: each domain's box and first split axis
void domain_boxes(int P, int id, int dir, double lo[3], double hi[3], const double *split, photons_domain *out)
{
    if (id >= P - 1) {
        photons_domain &D = out[rank_of_domain(P, id)];
        for (int d = 0; d < 3; d++) { D.lo[d] = lo[d]; D.hi[d] = hi[d]; }
        D.axis = dir;
        return;
    }
    double keep = hi[dir];
    hi[dir] = split[id];
    domain_boxes(P, 2 * id + 1, (dir + 1) % 3, lo, hi, split, out);
    hi[dir] = keep;
    keep = lo[dir];
    lo[dir] = split[id];
    domain_boxes(P, 2 * id + 2, (dir + 1) % 3, lo, hi, split, out);
    lo[dir] = keep;
}

// src/domains.c:45-82: how many of `size` domains lie on each side
void fraction(int size, int *l, int *r)
{
    int left, right;
    if (size == 1) { left = 1; right = 0; }
    else if (size == 2) { left = 1; right = 1; }
    else if (size == 3) { left = 2; right = 1; }
    else {
        left = 1;
        right = 2;
        while (size - left >= right - size) { left *= 2; right *= 2; }
        left >>= 1;
        right = size - left;
        if (left < right) { left = right; right = size - left; }
    }
    *l = left;
    *r = right;
}

// src/domains.c:86-144: a split plane moves by the relaxed difference of
// the per-domain times of its two sides; children are placed within the
// old planes, then the plane moves
void split_node(int D, int nproc, int id, int P, const std::vector<double> &t, double *split, const double bl[3],
                const double br[3])
{
    if (id >= P - 1) return;
    int nleft, nright;
    fraction(nproc, &nleft, &nright);
    const double relax = 0.3;
    const double t1 = node_time(P, 2 * id + 1, t) / nleft, t2 = node_time(P, 2 * id + 2, t) / nright;
    const double w0l = split[id] - bl[D], w0r = br[D] - split[id];
    const double shift = 0.5 * relax * (t2 - t1) / (t1 * nleft / w0l + t2 * nright / w0r);
    const double new_split = split[id] + shift;
    double lo[3] = {bl[0], bl[1], bl[2]}, hi[3] = {br[0], br[1], br[2]};
    hi[D] = split[id];
    split_node((D + 1) % 3, nleft, 2 * id + 1, P, t, split, lo, hi);
    lo[D] = split[id];
    hi[D] = br[D];
    split_node((D + 1) % 3, nright, 2 * id + 2, P, t, split, lo, hi);
    split[id] = new_split;
}

// the receiving domain as its root node holds it: the root's bounds are
// the top-tree node's centre -/+ half its width (src/fmm.c:189-197), its
// centre and width those of the bounds (src/fmm.c:126-131)
void root_geometry(const photons_domain &D, double c[3], double w[3])
{
    for (int d = 0; d < 3; d++) {
        const double tc = 0.5 * (D.hi[d] + D.lo[d]), tw = D.hi[d] - D.lo[d];
        const double lo = tc - 0.5 * tw, hi = tc + 0.5 * tw;
        w[d] = hi - lo;
        c[d] = 0.5 * (hi + lo);
    }
}

// ------------------------------------------------------------------
// export kernels
// ------------------------------------------------------------------
struct ExportArgs {
    const int *depth_list, *depth_off, *parent, *son0, *son1, *npart, *ipart;
    const double *cx, *cy, *cz, *wx, *wy, *wz, *M, *px, *py, *pz;
    int nleaf;
    double rc[3], rw[3], sh[3];  // receiving domain (centre, width), shift
    double rcut, theta;
    int *keep, *pruned, *nn, *nb, *pre, *bo;
};

// prune rule of src/remotes.c:97-158, FP64 with the reference's rounding
__device__ bool export_pruned(const ExportArgs &A, int u)
{
    const double c[3] = {A.cx[u], A.cy[u], A.cz[u]}, w[3] = {A.wx[u], A.wy[u], A.wz[u]};
    double dr = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double g = __dsub_rn(__dsub_rn(A.rc[d], c[d]), A.sh[d]);
        if (g < 0.0) g = -g;
        g = __dsub_rn(g, __dmul_rn(__dadd_rn(A.rw[d], w[d]), 0.5));
        if (g > 0.0) dr = __dadd_rn(dr, __dmul_rn(g, g));
    }
    dr = __dsqrt_rn(dr);
    double wmax = w[0];
    if (wmax < w[1]) wmax = w[1];
    if (wmax < w[2]) wmax = w[2];
    if (dr >= A.rcut) return true;
    return wmax < __dmul_rn(__dmul_rn(0.95, A.theta), dr);
}

// top-down: a node is sent if its parent was sent with its children
__global__ void k_export_keep(ExportArgs A, int d)
{
    const int b = A.depth_off[d], e = A.depth_off[d + 1];
    for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
        const int u = A.depth_list[i];
        const int p = A.parent[u];
        const int keep = p < 0 ? 1 : (A.keep[p] && !A.pruned[p]);
        A.keep[u] = keep;
        A.pruned[u] = (keep && u >= A.nleaf) ? (int)export_pruned(A, u) : 0;
        if (p < 0) { A.pre[u] = 0; A.bo[u] = 0; }
    }
}

// bottom-up: sent nodes and bodies below each node
__global__ void k_export_count(ExportArgs A, int d)
{
    const int b = A.depth_off[d], e = A.depth_off[d + 1];
    for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
        const int u = A.depth_list[i];
        int nn = 0, nb = 0;
        if (A.keep[u]) {
            if (u < A.nleaf) { nn = 1; nb = A.npart[u]; }
            else if (A.pruned[u]) { nn = 1; }
            else {
                const int s0 = A.son0[u], s1 = A.son1[u];
                nn = 1 + A.nn[s0] + A.nn[s1];
                nb = A.nb[s0] + A.nb[s1];
            }
        }
        A.nn[u] = nn;
        A.nb[u] = nb;
    }
}

// top-down: preorder index and first body of each sent node's children
__global__ void k_export_index(ExportArgs A, int d)
{
    const int b = A.depth_off[d], e = A.depth_off[d + 1];
    for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
        const int u = A.depth_list[i];
        if (!A.keep[u] || u < A.nleaf || A.pruned[u]) continue;
        const int s0 = A.son0[u], s1 = A.son1[u];
        A.pre[s0] = A.pre[u] + 1;
        A.bo[s0] = A.bo[u];
        A.pre[s1] = A.pre[u] + 1 + A.nn[s0];
        A.bo[s1] = A.bo[u] + A.nb[s0];
    }
}

// one warp per sent node: the node record and, for a leaf, its bodies
__global__ void k_export_write(ExportArgs A, int nu, photons_remote_node *nodes, photons_remote_body *bodies)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int u = gw; u < nu; u += nw) {
        if (!A.keep[u]) continue;
        photons_remote_node &E = nodes[A.pre[u]];
        const bool leaf = u < A.nleaf;
        if (lane < PH_NMULTI) E.M[lane] = A.M[(size_t)u * PH_NMULTI + lane];
        if (lane == 0) {
            E.npart = A.npart[u];
            E.width[0] = A.wx[u]; E.width[1] = A.wy[u]; E.width[2] = A.wz[u];
            E.center[0] = __dadd_rn(A.cx[u], A.sh[0]);
            E.center[1] = __dadd_rn(A.cy[u], A.sh[1]);
            E.center[2] = __dadd_rn(A.cz[u], A.sh[2]);
            if (leaf) { E.son[0] = A.bo[u]; E.son[1] = A.bo[u] + A.npart[u]; }
            else if (A.pruned[u]) { E.son[0] = E.son[1] = -1; }
            else { E.son[0] = A.pre[A.son0[u]]; E.son[1] = A.pre[A.son1[u]]; }
        }
        if (leaf) {
            const int ip = A.ipart[u], np = A.npart[u], o = A.bo[u];
            for (int j = lane; j < np; j += 32) {
                photons_remote_body &B = bodies[o + j];
                B.pos[0] = __dadd_rn(A.px[ip + j], A.sh[0]);
                B.pos[1] = __dadd_rn(A.py[ip + j], A.sh[1]);
                B.pos[2] = __dadd_rn(A.pz[ip + j], A.sh[2]);
                B.replenish = 0.0;
            }
        }
    }
}

// ------------------------------------------------------------------
// import kernels: received trees into the unified arrays from id `base`
// and their bodies into the particle arrays from index `body0`
// ------------------------------------------------------------------
struct ImportArgs {
    const photons_remote_node *nodes;
    const photons_remote_body *bodies;
    int count, nbody, base, body0, maxleaf;
    int *ipart, *npart, *parent, *depth, *son0, *son1, *boxid;
    int2 *son2;
    double *cx, *cy, *cz, *wx, *wy, *wz, *wsum, *M;
    float *M32;
    float4 *chi, *clo, *w32, *pos4;
    double *px, *py, *pz;
};

__global__ void k_import_nodes(ImportArgs A)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < A.count; k += gridDim.x * blockDim.x) {
        const photons_remote_node &E = A.nodes[k];
        const int u = A.base + k;
        const bool leaf = E.npart <= A.maxleaf;
        A.npart[u] = E.npart;
        A.ipart[u] = leaf ? A.body0 + E.son[0] : 0;
        const int s0 = (!leaf && E.son[0] >= 0) ? A.base + E.son[0] : -1;
        const int s1 = (!leaf && E.son[1] >= 0) ? A.base + E.son[1] : -1;
        A.son0[u] = s0;
        A.son1[u] = s1;
        A.son2[u] = make_int2(s0, s1);
        A.parent[u] = -1;
        A.depth[u] = 0;
        A.boxid[u] = 0;
        const double c0 = E.center[0], c1 = E.center[1], c2 = E.center[2];
        const double w0 = E.width[0], w1 = E.width[1], w2 = E.width[2];
        A.cx[u] = c0; A.cy[u] = c1; A.cz[u] = c2;
        A.wx[u] = w0; A.wy[u] = w1; A.wz[u] = w2;
        const double ws = w0 + w1 + w2;
        A.wsum[u] = ws;
        // FP32 copies as the local tree's (centre hi + lo, widths)
        const float h0 = (float)c0, h1 = (float)c1, h2 = (float)c2;
        A.chi[u] = make_float4(h0, h1, h2, 0.f);
        A.clo[u] = make_float4((float)(c0 - h0), (float)(c1 - h1), (float)(c2 - h2), 0.f);
        A.w32[u] = make_float4((float)w0, (float)w1, (float)w2, (float)ws);
        for (int m = 0; m < PH_NMULTI; m++) {
            A.M[(size_t)u * PH_NMULTI + m] = E.M[m];
            A.M32[(size_t)u * PH_NMULTI + m] = (float)E.M[m];
        }
    }
}

// received bodies
__global__ void k_import_bodies(ImportArgs A)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < A.nbody; k += gridDim.x * blockDim.x) {
        const photons_remote_body &B = A.bodies[k];
        A.px[A.body0 + k] = B.pos[0];
        A.py[A.body0 + k] = B.pos[1];
        A.pz[A.body0 + k] = B.pos[2];
    }
}

// FP32 offsets of the received bodies from their leaf's centre
__global__ void k_import_offsets(ImportArgs A)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = gw; k < A.count; k += nw) {
        const photons_remote_node &E = A.nodes[k];
        if (E.npart > A.maxleaf) continue;
        const int ip = A.body0 + E.son[0];
        const double c0 = E.center[0], c1 = E.center[1], c2 = E.center[2];
        for (int j = lane; j < E.npart; j += 32)
            A.pos4[ip + j] = make_float4((float)(A.px[ip + j] - c0), (float)(A.py[ip + j] - c1),
                                         (float)(A.pz[ip + j] - c2), 0.f);
    }
}

template <typename T>
int grow(T *&p, int &cap, long long need)
{
    if (need <= cap) return 0;
    cudaFree(p);
    p = nullptr;
    cap = 0;
    const long long want = need + need / 4 + 64;
    if (want > 0x7fffffffLL) return ph_set_error(PH_ERR_CAPACITY, "domain buffers: %lld elements", want);
    cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        return ph_set_error(PH_ERR_NOMEM, "domain buffers: %lld elements", want);
    }
    cap = (int)want;
    return 0;
}

DomainScratch &scratch(photons_ctx *c)
{
    if (!c->dsc) c->dsc = new DomainScratch();
    return *c->dsc;
}

int check_domain(const photons_domain *d, double L)
{
    if (!d) return ph_set_error(PH_ERR_ARG, "null domain");
    for (int k = 0; k < 3; k++)
        if (!(d->lo[k] < d->hi[k]) || d->lo[k] < 0.0 || d->hi[k] > L)
            return ph_set_error(PH_ERR_ARG, "domain box outside [0, boxsize] or empty");
    if (d->axis < 0 || d->axis > 2) return ph_set_error(PH_ERR_ARG, "domain axis %d", d->axis);
    return 0;
}

// the tree and multipoles of the prepared positions
int prepare(photons_ctx *c)
{
    c->dom_set = true;
    photons_params p = c->dom_params;
    const int dio = p.flags & PHOTONS_F_DEVICE_IO;
    PH_TRY(ph_stage_build(c, &p, c->dom_n, c->dom_pos, dio));
    PH_TRY(ph_stage_multipoles(c));  // the exported trees carry them
    PH_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return 0;
}

}  // namespace

void ph_domain_release(photons_ctx *c)
{
    if (!c->dsc) return;
    DomainScratch &s = *c->dsc;
    cudaFree(s.work);
    cudaFree(s.out_nodes); cudaFree(s.out_bodies); cudaFree(s.in_nodes); cudaFree(s.in_bodies);
    cudaFree(s.roots);
    delete c->dsc;
    c->dsc = nullptr;
}

// ------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------
extern "C" int photons_domain_split(int nrank, double boxsize, photons_domain *domains, double *split)
{
    photons_gpu_clear_error();
    if (nrank < 1 || !(boxsize > 0) || !domains) return ph_set_error(PH_ERR_ARG, "bad domain split arguments");
    std::vector<double> t(2 * nrank - 1, 1.0), sp(nrank > 1 ? nrank - 1 : 1, 0.0);
    double bl[3] = {0, 0, 0}, br[3] = {boxsize, boxsize, boxsize};
    volume_part(nrank, 0, bl, br, 0, t, sp.data());
    double lo[3] = {0, 0, 0}, hi[3] = {boxsize, boxsize, boxsize};
    domain_boxes(nrank, 0, 0, lo, hi, sp.data(), domains);
    if (split)
        for (int i = 0; i < nrank - 1; i++) split[i] = sp[i];
    return 0;
}

extern "C" int photons_domain_assign(int nrank, const double *split, int n, const double *pos, int *rank)
{
    photons_gpu_clear_error();
    if (nrank < 1 || n < 0 || (nrank > 1 && !split) || (n > 0 && (!pos || !rank)))
        return ph_set_error(PH_ERR_ARG, "bad domain assignment arguments");
    for (int i = 0; i < n; i++) {
        int id = 0, D = 0;
        while (id < nrank - 1) {
            id = pos[3 * (size_t)i + D] > split[id] ? 2 * id + 2 : 2 * id + 1;
            D = (D + 1) % 3;
        }
        rank[i] = rank_of_domain(nrank, id);
    }
    return 0;
}

extern "C" int photons_domain_rebalance(int nrank, double boxsize, double *split, const double *rank_time,
                                        photons_domain *domains)
{
    photons_gpu_clear_error();
    if (nrank < 1 || !(boxsize > 0) || (nrank > 1 && !split) || !rank_time)
        return ph_set_error(PH_ERR_ARG, "bad rebalance arguments");
    for (int r = 0; r < nrank; r++)
        if (!(rank_time[r] > 0)) return ph_set_error(PH_ERR_ARG, "rank %d time must be positive", r);
    // src/domains.c:22-40: each rank's time on its domain node
    std::vector<double> t(2 * nrank - 1, 0.0);
    for (int r = 0; r < nrank; r++) t[domain_of_rank(nrank, r)] = rank_time[r];
    const double bl[3] = {0, 0, 0}, br[3] = {boxsize, boxsize, boxsize};
    split_node(0, nrank, 0, nrank, t, split, bl, br);
    if (domains) {
        double lo[3] = {0, 0, 0}, hi[3] = {boxsize, boxsize, boxsize};
        domain_boxes(nrank, 0, 0, lo, hi, split, domains);
    }
    return 0;
}

extern "C" int photons_domain_prepare(photons_ctx *c, const photons_params *p, const photons_domain *dom, int n,
                                      const double *pos)
{
    photons_gpu_clear_error();
    if (!c || !p || !pos) return ph_set_error(PH_ERR_ARG, "null argument");
    PH_TRY(ph_validate(p, n));
    PH_TRY(check_domain(dom, p->boxsize));
    cudaSetDevice(c->device);
    c->dom = *dom;
    c->dom_params = *p;
    c->dom_n = n;
    c->dom_pos = pos;
    c->imp_nodes.clear();
    c->imp_bodies.clear();
    c->imp_first.clear();
    c->walk_imp = ph::WalkImports();
    c->have_key = false;  // the captured pass does not hold the domain set-up
    int rc = prepare(c);
    if (rc) c->dom_set = false;
    return rc;
}

extern "C" int photons_let_export(photons_ctx *c, const photons_domain *receiver, const double shift[3],
                                  photons_remote_node *nodes, int node_cap, photons_remote_body *bodies, int body_cap,
                                  int *nnode, int *nbody)
{
    photons_gpu_clear_error();
    if (!c || !receiver || !shift || !nnode || !nbody) return ph_set_error(PH_ERR_ARG, "null argument");
    if (!c->dom_set || !c->have_tree || !c->have_multipoles)
        return ph_set_error(PH_ERR_STATE, "photons_domain_prepare has not run");
    PH_TRY(check_domain(receiver, c->pp.boxsize));
    cudaSetDevice(c->device);
    DomainScratch &S = scratch(c);
    const int nl = c->info.nleaf, nu = c->info.nleaf + c->info.nnode;
    PH_TRY(grow(S.work, S.cap_work, 6LL * nu));
    PH_TRY(grow(S.out_nodes, S.cap_out_nodes, nu));
    PH_TRY(grow(S.out_bodies, S.cap_out_bodies, c->n));
    ExportArgs A;
    memset(&A, 0, sizeof A);
    A.depth_list = c->t.depth_list; A.depth_off = c->t.depth_off; A.parent = c->t.parent;
    A.son0 = c->t.son0; A.son1 = c->t.son1; A.npart = c->t.npart; A.ipart = c->t.ipart;
    A.cx = c->t.cx; A.cy = c->t.cy; A.cz = c->t.cz; A.wx = c->t.wx; A.wy = c->t.wy; A.wz = c->t.wz;
    A.M = c->M; A.px = c->b.x; A.py = c->b.y; A.pz = c->b.z;
    A.nleaf = nl;
    root_geometry(*receiver, A.rc, A.rw);
    for (int d = 0; d < 3; d++) A.sh[d] = shift[d];
    A.rcut = c->pp.rcut;
    A.theta = c->pp.theta;
    A.keep = S.work; A.pruned = S.work + nu; A.nn = S.work + 2 * (size_t)nu; A.nb = S.work + 3 * (size_t)nu;
    A.pre = S.work + 4 * (size_t)nu; A.bo = S.work + 5 * (size_t)nu;
    cudaStream_t st = c->stream;
    const int nd = c->info.depth + 1, blocks = ph::device_sm_count() * 4;
    for (int d = 0; d < nd; d++) ph::note_launch(), k_export_keep<<<blocks, 256, 0, st>>>(A, d);
    for (int d = nd - 1; d >= 0; d--) ph::note_launch(), k_export_count<<<blocks, 256, 0, st>>>(A, d);
    for (int d = 0; d < nd; d++) ph::note_launch(), k_export_index<<<blocks, 256, 0, st>>>(A, d);
    ph::note_launch(), k_export_write<<<blocks, 256, 0, st>>>(A, nu, S.out_nodes, S.out_bodies);
    PH_CUDA_CHECK(cudaGetLastError());
    // the root is the only node at depth 0; its counts are the totals
    int root = 0, tot[2] = {0, 0};
    PH_CUDA_CHECK(cudaMemcpyAsync(&root, c->t.depth_list, sizeof(int), cudaMemcpyDeviceToHost, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    if (root < 0 || root >= nu) return ph_set_error(PH_ERR_STATE, "no root at depth 0");
    PH_CUDA_CHECK(cudaMemcpyAsync(&tot[0], A.nn + root, sizeof(int), cudaMemcpyDeviceToHost, st));
    PH_CUDA_CHECK(cudaMemcpyAsync(&tot[1], A.nb + root, sizeof(int), cudaMemcpyDeviceToHost, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    *nnode = tot[0];
    *nbody = tot[1];
    if (!nodes && !bodies) return 0;
    if (!nodes || !bodies || tot[0] > node_cap || tot[1] > body_cap)
        return ph_set_error(PH_ERR_CAPACITY, "export needs %d nodes and %d bodies", tot[0], tot[1]);
    PH_CUDA_CHECK(cudaMemcpyAsync(nodes, S.out_nodes, sizeof(photons_remote_node) * (size_t)tot[0],
                                  cudaMemcpyDeviceToHost, st));
    if (tot[1])
        PH_CUDA_CHECK(cudaMemcpyAsync(bodies, S.out_bodies, sizeof(photons_remote_body) * (size_t)tot[1],
                                      cudaMemcpyDeviceToHost, st));
    PH_CUDA_CHECK(cudaStreamSynchronize(st));
    return 0;
}

extern "C" int photons_let_import(photons_ctx *c, const photons_remote_node *nodes, int nnode,
                                  const photons_remote_body *bodies, int nbody)
{
    photons_gpu_clear_error();
    if (!c || nnode < 0 || nbody < 0 || (nnode && !nodes) || (nbody && !bodies))
        return ph_set_error(PH_ERR_ARG, "bad import arguments");
    if (!c->dom_set) return ph_set_error(PH_ERR_STATE, "photons_domain_prepare has not run");
    if (nnode == 0) return 0;  // nothing was sent (src/remotes.c:721-722)
    // every index must lie in the message, children after their parent
    const int maxleaf = c->pp.maxleaf;
    for (int k = 0; k < nnode; k++) {
        const photons_remote_node &E = nodes[k];
        if (E.npart < 0) return ph_set_error(PH_ERR_ARG, "received node %d: negative count", k);
        if (E.npart <= maxleaf) {
            if (E.son[0] < 0 || E.son[1] < E.son[0] || E.son[1] > nbody || E.son[1] - E.son[0] != E.npart)
                return ph_set_error(PH_ERR_ARG, "received leaf %d: body range outside the message", k);
        } else if (E.son[0] >= 0 || E.son[1] >= 0) {
            if (E.son[0] <= k || E.son[1] <= k || E.son[0] >= nnode || E.son[1] >= nnode)
                return ph_set_error(PH_ERR_ARG, "received node %d: child outside the message", k);
        }
    }
    const int n0 = (int)c->imp_nodes.size(), b0 = (int)c->imp_bodies.size();
    c->imp_first.push_back(n0);
    for (int k = 0; k < nnode; k++) {
        photons_remote_node E = nodes[k];
        if (E.npart <= maxleaf) { E.son[0] += b0; E.son[1] += b0; }
        else {
            if (E.son[0] >= 0) E.son[0] += n0;
            if (E.son[1] >= 0) E.son[1] += n0;
        }
        c->imp_nodes.push_back(E);
    }
    c->imp_bodies.insert(c->imp_bodies.end(), bodies, bodies + nbody);
    return 0;
}

extern "C" int photons_domain_finish(photons_ctx *c, double *acc)
{
    photons_gpu_clear_error();
    if (!c || !acc) return ph_set_error(PH_ERR_ARG, "null argument");
    if (!c->dom_set || !c->have_tree) return ph_set_error(PH_ERR_STATE, "photons_domain_prepare has not run");
    cudaSetDevice(c->device);
    const photons_params p = c->dom_params;
    const int dio = p.flags & PHOTONS_F_DEVICE_IO;
    const int nimp = (int)c->imp_nodes.size(), nbody = (int)c->imp_bodies.size();
    int base = c->info.nleaf + c->info.nnode;
    // room for the received trees; if the arrays must grow, the tree is
    // built again (the same tree: the build is deterministic)
    if (base + nimp > c->cap_u || c->n + nbody > c->cap_n) {
        c->imp_reserve_u = nimp + nimp / 4 + 1024;
        c->imp_reserve_body = nbody + nbody / 4 + 1024;
        PH_TRY(prepare(c));
        base = c->info.nleaf + c->info.nnode;
        if (base + nimp > c->cap_u || c->n + nbody > c->cap_n)
            return ph_set_error(PH_ERR_CAPACITY, "received trees do not fit");
    }
    DomainScratch &S = scratch(c);
    cudaStream_t st = c->stream;
    const int nroot = (int)c->imp_first.size();
    if (nimp) {
        PH_TRY(grow(S.in_nodes, S.cap_in_nodes, nimp));
        PH_TRY(grow(S.in_bodies, S.cap_in_bodies, nbody > 0 ? nbody : 1));
        PH_TRY(grow(S.roots, S.cap_roots, nroot));
        std::vector<int> roots(nroot);
        for (int k = 0; k < nroot; k++) roots[k] = base + c->imp_first[k];
        PH_CUDA_CHECK(cudaMemcpyAsync(S.in_nodes, c->imp_nodes.data(), sizeof(photons_remote_node) * (size_t)nimp,
                                      cudaMemcpyHostToDevice, st));
        if (nbody)
            PH_CUDA_CHECK(cudaMemcpyAsync(S.in_bodies, c->imp_bodies.data(),
                                          sizeof(photons_remote_body) * (size_t)nbody, cudaMemcpyHostToDevice, st));
        PH_CUDA_CHECK(cudaMemcpyAsync(S.roots, roots.data(), sizeof(int) * nroot, cudaMemcpyHostToDevice, st));
        ImportArgs A;
        memset(&A, 0, sizeof A);
        A.nodes = S.in_nodes; A.bodies = S.in_bodies; A.count = nimp; A.nbody = nbody; A.base = base;
        A.body0 = c->n; A.maxleaf = p.maxleaf;
        A.ipart = c->t.ipart; A.npart = c->t.npart; A.parent = c->t.parent; A.depth = c->t.depth;
        A.son0 = c->t.son0; A.son1 = c->t.son1; A.boxid = c->t.boxid; A.son2 = c->t.son2;
        A.cx = c->t.cx; A.cy = c->t.cy; A.cz = c->t.cz; A.wx = c->t.wx; A.wy = c->t.wy; A.wz = c->t.wz;
        A.wsum = c->t.wsum; A.M = c->M; A.M32 = c->M32; A.chi = c->t.chi; A.clo = c->t.clo; A.w32 = c->t.w32;
        A.pos4 = c->pos4; A.px = c->b.x; A.py = c->b.y; A.pz = c->b.z;
        const int blocks = ph::device_sm_count() * 4;
        ph::note_launch(), k_import_nodes<<<blocks, 256, 0, st>>>(A);
        if (nbody) ph::note_launch(), k_import_bodies<<<blocks, 256, 0, st>>>(A);
        ph::note_launch(), k_import_offsets<<<blocks, 256, 0, st>>>(A);
        PH_CUDA_CHECK(cudaGetLastError());
        c->walk_imp.root = S.roots;
        c->walk_imp.nroot = nroot;
        c->walk_imp.base = base;
    }
    // src/fmm.c:909-1075: the local tree, its 26 images and the received trees
    const unsigned mask = (1u << PH_NIMG) - 1u;
    int rc = ph_stage_walk(c, mask);
    if (!rc) rc = ph_stage_p2p(c, p.precision, 1);
    const unsigned long long nm2l = c->ws.c[ph::WC_M2L_LOCAL] + c->ws.c[ph::WC_M2L_IMAGE];
    if (!rc && !(p.flags & PHOTONS_F_NO_FARFIELD) && nm2l) {
        rc = ph_stage_m2l(c, p.precision);
        if (!rc) rc = ph_stage_downward(c, p.precision);
    }
    if (!rc) rc = ph_stage_output(c, acc, dio, p.flags & PHOTONS_F_TREE_ORDER);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = ph_set_cuda_error(e, "domain pass", __FILE__, __LINE__);
    }
    c->walk_imp = ph::WalkImports();
    c->dom_set = false;
    c->imp_nodes.clear();
    c->imp_bodies.clear();
    c->imp_first.clear();
    c->mask = mask;
    c->precision = p.precision;
    c->last_flags = p.flags;
    return rc;
}
