// Context and stage functions shared by the photons_* ABI (api.cu) and the
// reference-named entry points (legacy.cu).
#pragma once

#include <vector>

#include "fmm_context.cuh"
#include "multipole.cuh"
#include "p2p.cuh"
#include <cufft.h>

#include "photons_fmm.h"

enum {
    PH_OK = 0,
    PH_ERR_ARG = 1,
    PH_ERR_CUDA = 2,
    PH_ERR_NOMEM = 3,
    PH_ERR_CAPACITY = 4,
    PH_ERR_SMALL = 5,
    PH_ERR_STATE = 6,
    PH_ERR_DEPTH = 7,
    PH_ERR_UNSUPPORTED = 8
};

enum {
    EV_START = 0, EV_UPLOADED, EV_TREE, EV_WALK, EV_P2P_BEGIN, EV_P2P, EV_FAR, EV_GATHERED, EV_END, EV_COUNT
};

// Everything a captured pass bakes in; a pass with a different key is
// captured anew.  Zero-filled before use so it compares with memcmp.
struct PassKey {
    int n, nbox, levels, top, maxleaf, precision, flags, dio, variant, nwarps, stage_extra;
    unsigned mask;
    double boxsize, theta, rs, rcut, eps, mass;
    const void *pos, *acc;
    cudaStream_t stream;
    unsigned long long epoch;
};

// What a pass leaves for the host, written by one kernel into pinned host
// memory the device addresses (read after the stream has finished), and the
// kick-drift-kick factors the host puts there for the next step
struct PassReport {
    int cnt[ph::BC_NCOUNTERS];
    unsigned long long wc[ph::WC_N];
    long long mu_need;
    int mu_over;
    int ndepth_off;
    int depth_off[PH_MAX_DEPTH_CAP + 2];
    double kdk_f[2];
};

struct photons_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    cudaEvent_t ev[EV_COUNT] = {};
    ph::BuildBufs b;
    ph::TreeBufs t;
    ph::WalkBufs w;
    float4 *pos4 = nullptr;
    double *ax = nullptr, *ay = nullptr, *az = nullptr;
    double *M = nullptr, *L = nullptr;
    float *M32 = nullptr;  // multipoles rounded to FP32 for the split M2L
    double *io = nullptr;  // 3*cap_n staging for host transfers and gathers
    int *work_counter = nullptr;
    int *far_gate = nullptr;  // [2] far-field switches of the captured pass
    // mutual P2P (p2p.cu): per-leaf pairing data, per-entry slots, reaction buffer
    int *mu_sorted = nullptr, *mu_nrecv = nullptr, *mu_slot = nullptr, *mu_over = nullptr;
    long long *mu_size = nullptr, *mu_rbase = nullptr, *mu_total = nullptr, *mu_scan = nullptr;
    int *mu_nev = nullptr;
    int *mu_pq = nullptr;
    int2 *mu_ev = nullptr;
    float *mu_buf = nullptr;
    long long mu_buf_cap = 0, mu_slot_cap = 0, hint_mubuf = 0;
    bool mu_off = false;  // the reaction slots did not fit: every pair one way
    int pass_flags = 0;   // PHOTONS_F_* of the pass being prepared
    int mu_cap_leaves = 0;
    // PM mesh (pm.cu): density / potential, half spectrum, gradient grids, FFT plans
    int pm_n = 0, pm_cap_io = 0;
    double *pm_rho = nullptr, *pm_grad = nullptr, *pm_io = nullptr;
    double *pm_green = nullptr;                        // Green's function of the half spectrum
    double pm_green_pref = 0.0, pm_green_ismth2 = 0.0;  // the constants it was computed for
    cufftDoubleComplex *pm_rk = nullptr;
    cufftHandle pm_plan_r2c = 0, pm_plan_c2r = 0;
    int cap_n = 0, cap_u = 0;
    // last pass
    PassParams pp{};
    ph::TreeInfo info;
    ph::WalkStats ws{};
    int n = 0;
    unsigned mask = 0;
    int last_flags = 0, precision = 0;
    bool have_tree = false, have_lists = false, have_multipoles = false;
    long long hint_p2p = 0, hint_pd = 0, hint_m2l = 0;
    int hint_levels = 0;  // node levels to launch (0: estimate from N)
    int hint_top = 0;     // levels of wide nodes to launch (0: estimate from N)
    std::vector<BoxParams> h_boxes;  // this pass's box table (host copy)
    int cap_box = 0;
    int ndepth = 0;       // depths the walk and far field launch
    unsigned long long epoch = 0;  // bumped by every device (re)allocation
    // a rank's domain pass (domain.cu): the domain its tree covers, the
    // trees received from other ranks (host copies until the pass ends),
    // and the capacity reserved in the unified and particle arrays for them
    bool dom_set = false;
    photons_domain dom{};
    std::vector<photons_remote_node> imp_nodes;
    std::vector<photons_remote_body> imp_bodies;
    std::vector<int> imp_first;            // first node of each received tree in imp_nodes
    int imp_reserve_u = 0, imp_reserve_body = 0;
    ph::WalkImports walk_imp;               // what the next walk adds to the root's list
    struct DomainScratch *dsc = nullptr;    // export/import device buffers
    photons_params dom_params{};            // the prepared pass (for a rebuild with more room)
    int dom_n = 0;
    const double *dom_pos = nullptr;
    // the captured pass
    bool capturing = false, have_key = false;
    cudaGraphExec_t gexec = nullptr;
    unsigned long long graph_kernels = 0;  // kernel nodes of gexec
    PassKey key{};
    // the captured kick-drift-kick step: the pass's key, velocity array and
    // box side; device factors (dkh, dd) and the flag that stops the second kick
    cudaGraphExec_t kexec = nullptr;
    unsigned long long kdk_kernels = 0;
    bool have_kkey = false;
    PassKey kkey{};
    const double *kkey_vel = nullptr;
    double kkey_box = 0.0;
    double *kdk_f = nullptr;
    int *kdk_skip = nullptr;
    // pinned host memory the device addresses: the pass report, and the box
    // table staged for upload (hbox_cap entries); ev_hlink is recorded after
    // the last kernel that read the staged inputs
    PassReport *rep = nullptr, *rep_dev = nullptr;
    BoxParams *hbox = nullptr, *hbox_dev = nullptr;
    int hbox_cap = 0;
    cudaEvent_t ev_hlink = nullptr;
};

// return a nonzero status code from the enclosing function
#define PH_TRY(x)               \
    do {                        \
        int rc__ = (x);         \
        if (rc__) return rc__;  \
    } while (0)

struct HostTree {
    int nleaf = 0, nnode = 0;
    std::vector<int> ipart, npart, son0, son1, parent;
    std::vector<double> cx, cy, cz, wx, wy, wz, split, M, L;
};

int ph_validate(const photons_params *p, int n);
// kick and drift with the factor in device memory (integrate.cu)
int ph_enqueue_kick_dev(int n, double *vel, const double *acc, const double *dkh, const int *skip, cudaStream_t st);
int ph_enqueue_drift_dev(int n, double *pos, const double *vel, const double *dd, double L, cudaStream_t st);
// One kick-drift-kick step as one captured graph (api.cu).  *done:
// KDK_DONE the step ran whole; KDK_NOT_RUN nothing ran (no graph yet for
// this pass: the caller runs the step one launch at a time); KDK_PASS_AGAIN
// the kick and drift ran but the pass did not fit (its flags stopped the
// second kick): the caller runs the pass and the second kick.
enum { KDK_NOT_RUN = 0, KDK_DONE = 1, KDK_PASS_AGAIN = 2 };
int ph_kdk_graph_step(photons_ctx *c, const photons_params *q, int n, double *pos, double *vel, double *acc,
                      double dkh, double dd, int *done);
void ph_domain_release(photons_ctx *c);
int ph_stage_build(photons_ctx *c, const photons_params *p, int n, const double *pos, int device_io);
int ph_stage_walk(photons_ctx *c, unsigned mask);
int ph_stage_p2p(photons_ctx *c, int precision, int zero);
int ph_stage_multipoles(photons_ctx *c);
int ph_stage_m2l(photons_ctx *c, int precision);
int ph_stage_downward(photons_ctx *c, int precision);
int ph_stage_output(photons_ctx *c, double *acc, int device_io, int tree_order);
int ph_download_tree(photons_ctx *c, HostTree &h, bool with_expansions);
int ph_pm_enqueue(photons_ctx *c, const photons_params *p, int nside, int n, const double *pos, double *acc_pm);
void ph_pm_release(photons_ctx *c);

namespace ph {
int launch_init_particles(BuildBufs &b, const double *pos, int n, cudaStream_t st);
}
