// Host side of the C ABI (include/phybs.h): mesh packing, device memory,
// the graph-captured pass loop and parity/debug entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/phybs.h"
#include "phybs_internal.cuh"

using namespace pbs;

namespace {

constexpr int CHUNK_PASSES = 16;  // passes per body of the step graph

template <typename T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        n = count;
        return cudaMalloc((void **)&p, std::max<size_t>(count, 1) * sizeof(T));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
    }
};

int round_up(int x, int a) { return (x + a - 1) / a * a; }

}  // namespace

struct pbs_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    int N = 0, T = 0, B = 0, Np = 0, Tp = 0, n_tblk = 0, n_nblk = 0;
    int material = PBS_MATERIAL_NEOHOOKEAN;
    float density = 1000.f, gravity = 9.8f;
    pbs_step_params params{};
    DevParams dparams{};
    std::vector<int> user2pad, h_pad2user, h_tet_user, h_node_state;
    std::vector<float> h_rest;  // user layout, for reset

    // device mesh
    DevBuf<int4> tets, tslot;
    DevBuf<float4> row0, row1, row2, info, rest4;
    DevBuf<int> inc_ptr, inc, tblk_inst, nblk_inst, pad2user, tet_user, node_state, bad, staging_ids;
    // pass layout (chunks of tets) and the host copies it is rebuilt from
    int n_chunks = 0, chunk_tets = CHUNK_TETS, chunk_nodes = CHUNK_NODES, chunk_threads = CHUNK_THREADS;
    int chunk_stage = 0;
    int node_npt = NODE_NPT_DEFAULT;
    std::vector<int4> h_tets_pad;
    std::vector<double> h_rest_pad;
    DevBuf<int4> chunk;
    DevBuf<int> chunk_inst, qperm, pptr;
    uint4 *qcor = nullptr;  // in qrows, after the three row arrays
    DevBuf<int4> lmeta;
    // the pass tets' rows and corner records, one allocation (4 x 16 B a tet):
    // the L2 access-policy window of the per-tet kernel covers it
    DevBuf<float4> qrows, part, parth;
    float4 *qrow0 = nullptr, *qrow1 = nullptr, *qrow2 = nullptr;
    // L2 residency of the pass rows: persisting set-aside taken, window bytes,
    // hit ratio, and whether the launches use it (pbs_set_l2_residency)
    bool l2_setaside = false, l2_use = true;
    size_t l2_window = 0;
    float l2_hit = 0.f;
    DevBuf<double2> cpart;
    DevBuf<double> rslot;
    // device state
    DevBuf<float4> uh, ul, dd, oh, ol, u0h, u0l, th, tl, v, vold, ext, diag, hist1, hist2, bh, bl, ub, ch, cl;
    // learned warm start
    DevBuf<float> ws_theta, ws_stats;  // NPARAM; feat mean 24, feat std 24, out std 3
    bool ws_enabled = false;
    int ws_base = 0;  // 0: corrections to the plain guess, 1: to the extrapolation u0 + 2 d1 - d2
    bool guess_pending = false;  // parity 1 holds a caller guess for the next step
    int sms = 148;
    DevBuf<float> tf, hd, staging, staging2;
    int last_fp64_svd = 0;  // tets of the last pbs_eval_tets whose stretch stress took the FP64 SVD
    // boundary surface for picking and drag forces: faces and rings in padded
    // node ids on the device, rings in caller ids on the host
    int n_faces = 0;
    std::vector<int> h_ring_ptr, h_ring;
    DevBuf<int4> faces_pad;
    DevBuf<int> ring_pad, pick_id;
    DevBuf<float> pick_d2;
    DevBuf<float4> drag_ext;
    // backward-Euler step: block-CSR pattern (built on first use), values,
    // block-Jacobi inverses, CG vectors and reductions
    bool bsr_ready = false;
    DevBuf<int> bsr_ptr, bsr_col;
    DevBuf<float> bsr_val, cg_dinv;
    DevBuf<float4> cg_b, cg_x, cg_r, cg_z, cg_p, cg_q;
    DevBuf<double> cg_part;
    DevBuf<CgState> cg_state;
    CgState *h_cg = nullptr;
    // 16 CG iterations captured as one graph, for the system and stop rule of
    // the key (rebuilt when they change)
    cudaGraphExec_t cg_exec = nullptr;
    const void *cg_key[3] = {nullptr, nullptr, nullptr};
    double cg_key_tol2 = -1.0;
    int cg_key_int[3] = {-1, -1, -1};
    DevBuf<double2> tpart;
    DevBuf<double> npart;
    DevBuf<float> npartf;
    DevBuf<InstCtl> ctl, ctl2;  // ctl2: the pass graph's second control-block copy
    DevBuf<unsigned int> tcount;
    DevBuf<int> active;  // [0] instances running, [1] a device wait gave up
    // strain-based PBD (levels built on first use) and projective dynamics
    // (its matrix built per (dt_matrix, stiffness)); dyn_* are their per-step
    // positions, start positions and right-hand-side base
    std::vector<int> h_inst_tets;  // per instance: first, end padded tet
    std::vector<int> h_inst_nodes;  // per instance: first, end padded node
    bool pbd_ready = false;
    int pbd_groups = 0;
    DevBuf<int> pbd_grp, pbd_lvl;
    DevBuf<int4> pbd_tet;
    DevBuf<float4> pbd_d0, pbd_d1, pbd_d2;
    DevBuf<float2> pbd_node;  // {1 / mass, gravity_y} of the PBD rest data
    // distributed-shared-memory variant: per-corner codes and per-group ranges
    int pbd_smem = 0;  // 0: positions stay in global memory
    DevBuf<int4> pbd_codes, pbd_gnode;
    bool pd_ready = false;
    float pd_dtm = 0.f, pd_k = 0.f;
    DevBuf<float> pd_val, pd_dinv;
    DevBuf<float4> dyn_px, dyn_x0, dyn_s;
    // host pinned
    int *h_active = nullptr;   // 2 slots: running counts of the host loop, or the bodies the loop ran
    InstCtl *h_ctl = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr, ev_chunk[2] = {nullptr, nullptr};
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    bool graph_loop = false;  // graph is the WHILE node over the pass body (else the body alone)
    // persistent frame kernel: its barrier words and per-CTA sums
    int engine = PBS_ENGINE_GRAPH;
    DevBuf<FrameSync> fsync;
    DevBuf<double2> fce, fcr;
    double last_ms = 0.0;
    pbs_stats stats{};

    DevMesh mesh() const {
        DevMesh m;
        m.Np = Np; m.Tp = Tp; m.n_inst = B; m.n_tblk = n_tblk; m.n_nblk = n_nblk;
        m.tets = tets.p; m.row0 = row0.p; m.row1 = row1.p; m.row2 = row2.p;
        m.inc_ptr = inc_ptr.p; m.inc = inc.p; m.tslot = tslot.p; m.info = info.p; m.rest = rest4.p;
        m.tblk_inst = tblk_inst.p; m.nblk_inst = nblk_inst.p;
        m.n_chunks = n_chunks; m.chunk = chunk.p; m.chunk_inst = chunk_inst.p;
        m.chunk_tets = chunk_tets; m.chunk_nodes = chunk_nodes; m.chunk_threads = chunk_threads;
        m.chunk_stage = chunk_stage;
        m.node_npt = node_npt;
        m.qrow0 = qrow0; m.qrow1 = qrow1; m.qrow2 = qrow2; m.qcor = qcor; m.lmeta = lmeta.p;
        m.l2_base = l2_use && l2_window ? (const void *)qrows.p : nullptr;
        m.l2_bytes = l2_window;
        m.l2_hit = l2_hit;
        m.pptr = pptr.p;
        m.stream_grid = stream_grid(m, material, dparams.incremental != 0, sms);
        return m;
    }
    DevState state() const {
        DevState s;
        s.uh = uh.p; s.ul = ul.p; s.dd = dd.p; s.oh = oh.p; s.ol = ol.p; s.u0h = u0h.p; s.u0l = u0l.p;
        s.th = th.p; s.tl = tl.p; s.v = v.p; s.vold = vold.p; s.ext = ext.p; s.diag = diag.p;
        s.hist1 = hist1.p; s.hist2 = hist2.p; s.bh = bh.p; s.bl = bl.p; s.ub = ub.p; s.ch = ch.p; s.cl = cl.p;
        s.tf = tf.p; s.hd = hd.p; s.tpart = tpart.p; s.npart = npart.p; s.npartf = npartf.p; s.ctl = ctl.p; s.active = active.p;
        s.ctl2 = ctl2.p; s.tcount = tcount.p;
        s.cpart = cpart.p; s.part = part.p; s.parth = parth.p; s.rslot = rslot.p;
        return s;
    }
    void release() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        DevBuf<int4> *i4[] = {&tets, &tslot};
        for (auto b : i4) b->release();
        DevBuf<float4> *f4[] = {&row0, &row1, &row2, &info, &rest4, &uh, &ul, &dd, &oh, &ol, &u0h, &u0l, &th, &tl,
                                &v, &vold, &ext, &diag, &hist1, &hist2, &bh, &bl, &ub, &ch, &cl};
        for (auto b : f4) b->release();
        DevBuf<int> *ii[] = {&inc_ptr, &inc, &tblk_inst, &nblk_inst, &pad2user, &tet_user, &node_state, &bad, &active,
                             &staging_ids};
        for (auto b : ii) b->release();
        ws_theta.release(); ws_stats.release();
        chunk.release(); lmeta.release(); cpart.release(); rslot.release();
        DevBuf<int> *ci[] = {&chunk_inst, &qperm, &pptr};
        for (auto b : ci) b->release();
        DevBuf<float4> *cf[] = {&qrows, &part, &parth};
        for (auto b : cf) b->release();
        tf.release(); hd.release(); staging.release(); staging2.release(); tpart.release(); npart.release(); npartf.release(); ctl.release(); ctl2.release(); tcount.release();
        fsync.release(); fce.release(); fcr.release();
        faces_pad.release(); ring_pad.release(); pick_id.release(); pick_d2.release(); drag_ext.release();
        bsr_ptr.release(); bsr_col.release(); bsr_val.release(); cg_dinv.release(); cg_part.release(); cg_state.release();
        pbd_grp.release(); pbd_lvl.release(); pbd_tet.release(); pbd_d0.release(); pbd_d1.release(); pbd_d2.release();
        pbd_node.release(); pbd_codes.release(); pbd_gnode.release();
        pd_val.release(); pd_dinv.release(); dyn_px.release(); dyn_x0.release(); dyn_s.release();
        pbd_ready = pd_ready = false;
        DevBuf<float4> *cv[] = {&cg_b, &cg_x, &cg_r, &cg_z, &cg_p, &cg_q};
        for (auto b : cv) b->release();
        if (h_cg) cudaFreeHost(h_cg);
        h_cg = nullptr;
        if (cg_exec) cudaGraphExecDestroy(cg_exec);
        cg_exec = nullptr;
        bsr_ready = false;
        if (h_active) cudaFreeHost(h_active);
        if (h_ctl) cudaFreeHost(h_ctl);
        h_active = nullptr; h_ctl = nullptr;
        cudaEvent_t evs[] = {ev_start, ev_end, ev_chunk[0], ev_chunk[1]};
        for (auto e : evs) if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

#define CK(x)                                                   \
    do {                                                        \
        cudaError_t e__ = (x);                                  \
        if (e__ != cudaSuccess) {                               \
            return e__ == cudaErrorMemoryAllocation ? PBS_E_OUT_OF_MEMORY : PBS_E_CUDA; \
        }                                                       \
    } while (0)

// (Re)builds the pass layout with the given chunk shape: host chunking of the
// padded mesh, the device arrays, the chunk-ordered copy of the per-tet rows
// (when they exist) and the instances' chunk ranges.  host_ctl: the control
// blocks still on the host (creation), else those on the device are updated.
static int set_pass_layout(pbs_handle *h, int threads, int ct, int cn, int stage, std::vector<InstCtl> *host_ctl) {
    std::vector<InstCtl> ctl;
    if (host_ctl) {
        ctl = *host_ctl;
    } else {
        ctl.resize(h->B);
        CK(cudaMemcpy(ctl.data(), h->ctl.p, sizeof(InstCtl) * h->B, cudaMemcpyDeviceToHost));
    }
    ChunkLayout cl;
    build_chunks(h->Np, h->h_tets_pad, h->h_rest_pad, ctl, ct, cn, cl);
    const int nc = (int)cl.chunk.size();
    const size_t L = cl.lmeta.size(), T = (size_t)h->T;
    h->chunk.release(); h->chunk_inst.release(); h->cpart.release(); h->qperm.release();
    h->lmeta.release(); h->pptr.release();
    h->part.release(); h->parth.release();
    CK(h->chunk.alloc(nc)); CK(h->chunk_inst.alloc(nc)); CK(h->cpart.alloc(nc));
    CK(h->qperm.alloc(T));
    CK(h->lmeta.alloc(L)); CK(h->pptr.alloc(h->Np + 1));
    CK(h->part.alloc(L)); CK(h->parth.alloc(L));
    cudaStream_t s = h->stream;
    CK(cudaMemcpyAsync(h->chunk.p, cl.chunk.data(), sizeof(int4) * nc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->chunk_inst.p, cl.chunk_inst.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->qperm.p, cl.qperm.data(), sizeof(int) * T, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->qcor, cl.qcor.data(), sizeof(uint4) * T, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->lmeta.p, cl.lmeta.data(), sizeof(int4) * L, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->pptr.p, cl.pptr.data(), sizeof(int) * (h->Np + 1), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(h->part.p, 0, sizeof(float4) * std::max<size_t>(L, 1), s));
    CK(cudaMemsetAsync(h->parth.p, 0, sizeof(float4) * std::max<size_t>(L, 1), s));
    h->n_chunks = nc;
    h->chunk_threads = threads;
    h->chunk_tets = ct;
    h->chunk_nodes = cn;
    h->chunk_stage = stage;
    if (host_ctl) {
        *host_ctl = ctl;
    } else {
        CK(cudaMemcpyAsync(h->ctl.p, ctl.data(), sizeof(InstCtl) * h->B, cudaMemcpyHostToDevice, s));
        CK(launch_pass_rows(s, h->T, h->qperm.p, h->row0.p, h->row1.p, h->row2.p, h->qrow0, h->qrow1,
                            h->qrow2));
    }
    CK(cudaStreamSynchronize(s));
    h->graph_valid = false;
    return PBS_OK;
}

static void to_dev_params(const pbs_step_params &p, DevParams &d) {
    d.h = p.h;
    d.h2inv = 1.0f / (p.h * p.h);
    d.max_iters = p.max_iters;
    d.tol = p.tol;
    d.control = p.control;
    d.alpha0 = p.alpha0; d.alpha_min = p.alpha_min; d.alpha_shrink = p.alpha_shrink;
    d.ls_every = p.line_search_every; d.hd_every = p.hessian_every;
    d.n_profile = p.n_profile;
    for (int i = 0; i < 4; ++i) { d.profile_k[i] = p.profile_k[i]; d.profile_rho[i] = p.profile_rho[i]; }
    d.damping = p.damping; d.warm_start = p.warm_start; d.body_scale = p.body_force_scale;
    d.clamp_cpu = p.energy_clamp == PBS_CLAMP_CPU ? 1 : 0;
    d.pass_cap = p.pass_cap > 0 ? p.pass_cap : p.max_iters + 16;
    d.energy_slack = p.energy_slack;
    d.alpha_grow = p.alpha_grow;
    d.incremental = 0;  // set from the material and incremental_stress by the handle
}

extern "C" {

void pbs_default_params(pbs_step_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->h = 0.03f;
    p->max_iters = 96;
    p->tol = 0.0f;
    p->control = PBS_CONTROL_REFERENCE;
    p->alpha0 = 0.1f; p->alpha_min = 0.01f; p->alpha_shrink = 0.7f;
    p->line_search_every = 8;
    p->hessian_every = 32;
    p->n_profile = 3;
    p->profile_k[0] = 1; p->profile_k[1] = 7; p->profile_k[2] = 10;
    p->profile_rho[0] = 0.96f; p->profile_rho[1] = 0.991f; p->profile_rho[2] = 0.999f;
    p->damping = 0.99f;
    p->warm_start = 0.2f;
    p->body_force_scale = 2.0f;
    p->energy_clamp = PBS_CLAMP_CPU;
    p->pass_cap = 0;
    p->energy_slack = 0.0f;
    p->alpha_grow = 1.0f;
    p->incremental_stress = 1;
}

const char *pbs_error_string(int code) {
    switch (code) {
        case PBS_OK: return "ok";
        case PBS_E_INVALID_ARG: return "invalid argument";
        case PBS_E_CUDA: return "CUDA error";
        case PBS_E_NONFINITE: return "non-finite energy or residual";
        case PBS_E_ITER_CAP: return "pass cap reached";
        case PBS_E_BAD_MESH: return "bad mesh (index out of range, or non-positive rest volume)";
        case PBS_E_NO_DEVICE: return "no compute capability 10.3 CUDA device";
        case PBS_E_OUT_OF_MEMORY: return "out of device memory";
        case PBS_E_CAPACITY: return "size beyond the fixed maximum";
        case PBS_E_DEVICE_TIMEOUT: return "a kernel's bounded wait (its own copies, a grid barrier) ran out";
        default: return "unknown error";
    }
}

void pbs_lame(float young, float poisson, int reference_formula, float *mu, float *lambda) {
    float m = 0.5f * young / (1.0f + poisson);
    float l = m * 2.0f / (1.0f - 2.0f * poisson);
    if (!reference_formula) l *= poisson;
    if (mu) *mu = m;
    if (lambda) *lambda = l;
}

static int validate_params(const pbs_step_params *p) {
    if (!p) return PBS_E_INVALID_ARG;
    if (!(p->h > 0.f) || p->max_iters < 0 || p->line_search_every <= 0 || p->hessian_every <= 0 ||
        p->n_profile < 0 || p->n_profile > 4 || !(p->alpha0 > 0.f) || !(p->alpha_shrink > 0.f) ||
        p->alpha_shrink >= 1.f || (p->control != PBS_CONTROL_REFERENCE && p->control != PBS_CONTROL_RESTART) ||
        p->tol < 0.f || p->pass_cap < 0 || !(p->energy_slack >= 0.f) ||
        (p->incremental_stress != 0 && p->incremental_stress != 1) || !(p->alpha_grow >= 1.0f) ||
        !std::isfinite(p->alpha_grow))
        return PBS_E_INVALID_ARG;
    return PBS_OK;
}

// L2 residency of the pass rows (the per-tet kernels' 64 B a tet, read every
// pass): without it they stream from HBM on every pass although the step's
// working set is near L2's size.  Takes the persisting-L2 set-aside of this
// process's context (at most the rows' size, at most what the device allows)
// and sizes the window and its hit ratio to it; the limit belongs to the
// context, and pbs_destroy gives it back.  Devices without persisting L2 run
// without a window.
static void setup_l2_residency(pbs_handle *h, const cudaDeviceProp &prop) {
    const size_t bytes = h->qrows.n * sizeof(float4);
    if (prop.persistingL2CacheMaxSize <= 0 || prop.accessPolicyMaxWindowSize <= 0 || bytes == 0) return;
    const size_t aside = std::min<size_t>((size_t)prop.persistingL2CacheMaxSize, bytes);
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, aside) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    h->l2_setaside = true;
    h->l2_window = std::min<size_t>(bytes, (size_t)prop.accessPolicyMaxWindowSize);
    h->l2_hit = (float)std::min(1.0, (double)aside / (double)h->l2_window);
}

int pbs_create(const pbs_mesh_desc *d, pbs_handle **out) {
    if (!d || !out || d->n_nodes <= 0 || d->n_tets <= 0 || !d->rest || !d->tets || d->n_instances < 1 ||
        !(d->density > 0.f))
        return PBS_E_INVALID_ARG;
    if (d->n_instances > 1 && (!d->instance_node_ptr || !d->instance_tet_ptr)) return PBS_E_INVALID_ARG;
    *out = nullptr;
    int dev = 0, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PBS_E_NO_DEVICE;
    if (cudaGetDevice(&dev) != cudaSuccess) return PBS_E_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return PBS_E_NO_DEVICE;
    if (prop.major != 10 || prop.minor != 3) return PBS_E_NO_DEVICE;

    const int N = d->n_nodes, T = d->n_tets, B = d->n_instances;
    std::vector<int> nptr(B + 1), tptr(B + 1);
    if (B == 1) { nptr = {0, N}; tptr = {0, T}; }
    else {
        std::memcpy(nptr.data(), d->instance_node_ptr, sizeof(int) * (B + 1));
        std::memcpy(tptr.data(), d->instance_tet_ptr, sizeof(int) * (B + 1));
    }
    if (nptr[0] != 0 || tptr[0] != 0 || nptr[B] != N || tptr[B] != T) return PBS_E_INVALID_ARG;
    for (int b = 0; b < B; ++b)
        if (nptr[b + 1] < nptr[b] || tptr[b + 1] < tptr[b]) return PBS_E_INVALID_ARG;

    pbs_handle *h = new (std::nothrow) pbs_handle();
    if (!h) return PBS_E_OUT_OF_MEMORY;
    h->device = dev;
    h->sms = prop.multiProcessorCount;
    h->N = N; h->T = T; h->B = B;
    h->density = d->density; h->gravity = d->gravity;
    pbs_default_params(&h->params);
    to_dev_params(h->params, h->dparams);

    // ---- packing: each instance starts on a PAD boundary
    std::vector<InstCtl> ctl(B);
    int pn = 0, pt = 0;
    h->user2pad.assign(N, -1);
    std::vector<int> node_off(B), tet_off(B);
    for (int b = 0; b < B; ++b) {
        node_off[b] = pn; tet_off[b] = pt;
        int nn = nptr[b + 1] - nptr[b], nt = tptr[b + 1] - tptr[b];
        std::memset(&ctl[b], 0, sizeof(InstCtl));
        ctl[b].node_begin = pn; ctl[b].node_end = pn + nn;
        ctl[b].tet_begin = pt; ctl[b].tet_end = pt + nt;
        ctl[b].nblk_begin = pn / BLOCK; ctl[b].tblk_begin = pt / BLOCK;
        pn += round_up(std::max(nn, 1), PAD);
        pt += round_up(std::max(nt, 1), PAD);
        ctl[b].nblk_end = pn / BLOCK; ctl[b].tblk_end = pt / BLOCK;
        ctl[b].rho = 0.f; ctl[b].omega = 1.f; ctl[b].alpha = h->params.alpha0;
        for (int i = nptr[b]; i < nptr[b + 1]; ++i) h->user2pad[i] = node_off[b] + (i - nptr[b]);
        h->h_inst_tets.push_back(ctl[b].tet_begin);
        h->h_inst_tets.push_back(ctl[b].tet_end);
        h->h_inst_nodes.push_back(ctl[b].node_begin);
        h->h_inst_nodes.push_back(ctl[b].node_end);
    }
    const int Np = pn, Tp = pt;
    for (int b = 0; b < B; ++b) {  // mean edge length: cbrt(6 * mean |vol|)
        double vs = 0.0;
        for (int t = tptr[b]; t < tptr[b + 1]; ++t) {
            const int *q = d->tets + 4 * (size_t)t;
            double e[3][3];
            for (int c = 0; c < 3; ++c)
                for (int k = 0; k < 3; ++k) {
                    int a = q[c + 1], o = q[0];
                    if (a < 0 || a >= N || o < 0 || o >= N) { delete h; return PBS_E_BAD_MESH; }
                    e[c][k] = (double)d->rest[3 * (size_t)a + k] - d->rest[3 * (size_t)o + k];
                }
            vs += std::fabs(e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                            e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0])) / 6.0;
        }
        const int nt = tptr[b + 1] - tptr[b];
        ctl[b].ell = nt > 0 ? (float)std::cbrt(6.0 * vs / nt) : 1.0f;
    }
    h->Np = Np; h->Tp = Tp; h->n_tblk = Tp / BLOCK; h->n_nblk = Np / BLOCK;
    h->h_pad2user.assign(Np, -1);
    for (int i = 0; i < N; ++i) h->h_pad2user[h->user2pad[i]] = i;
    h->h_tet_user.assign(Tp, -1);
    std::vector<int4> tets_pad(Tp, make_int4(-1, -1, -1, -1));
    std::vector<int> tblk(h->n_tblk), nblk(h->n_nblk);
    for (int b = 0; b < B; ++b) {
        for (int j = ctl[b].tblk_begin; j < ctl[b].tblk_end; ++j) tblk[j] = b;
        for (int j = ctl[b].nblk_begin; j < ctl[b].nblk_end; ++j) nblk[j] = b;
        for (int t = tptr[b]; t < tptr[b + 1]; ++t) {
            int tp = tet_off[b] + (t - tptr[b]);
            h->h_tet_user[tp] = t;
            int id[4];
            for (int c = 0; c < 4; ++c) {
                int u = d->tets[4 * (size_t)t + c];
                if (u < nptr[b] || u >= nptr[b + 1]) { delete h; return PBS_E_BAD_MESH; }
                id[c] = h->user2pad[u];
            }
            tets_pad[tp] = make_int4(id[0], id[1], id[2], id[3]);
        }
    }
    // ---- canonical node -> (tet, corner) gather (ascending tet, then corner)
    std::vector<int> iptr(Np + 1, 0), ient(4 * (size_t)T);
    for (int tp = 0; tp < Tp; ++tp) {
        if (tets_pad[tp].x < 0) continue;
        const int *q = &tets_pad[tp].x;
        for (int c = 0; c < 4; ++c) iptr[q[c] + 1]++;
    }
    for (int i = 0; i < Np; ++i) iptr[i + 1] += iptr[i];
    {
        std::vector<int> fill(iptr.begin(), iptr.end() - 1);
        for (int tp = 0; tp < Tp; ++tp) {
            if (tets_pad[tp].x < 0) continue;
            const int *q = &tets_pad[tp].x;
            for (int c = 0; c < 4; ++c) ient[fill[q[c]]++] = 4 * tp + c;
        }
    }
    std::vector<int4> tslot(Tp, make_int4(-1, -1, -1, -1));
    for (size_t j = 0; j < ient.size(); ++j) (&tslot[ient[j] >> 2].x)[ient[j] & 3] = (int)j;
    h->h_node_state.assign(Np, 2);
    for (int i = 0; i < N; ++i) h->h_node_state[h->user2pad[i]] = (d->pin_mask && d->pin_mask[i] > 0) ? 1 : 0;
    std::vector<double> rest_pad(3 * (size_t)Np, 0.0);
    std::vector<float4> rest4(Np, make_float4(0.f, 0.f, 0.f, 0.f));
    const float *p0 = d->positions ? d->positions : d->rest;
    for (int i = 0; i < N; ++i) {
        int ip = h->user2pad[i];
        for (int k = 0; k < 3; ++k) {
            float r = d->rest[3 * (size_t)i + k];
            if (!std::isfinite(r) || !std::isfinite(p0[3 * (size_t)i + k])) { delete h; return PBS_E_INVALID_ARG; }
            rest_pad[3 * (size_t)ip + k] = r;
        }
        rest4[ip] = make_float4(d->rest[3 * (size_t)i], d->rest[3 * (size_t)i + 1], d->rest[3 * (size_t)i + 2], 0.f);
    }
    h->h_rest.assign(d->rest, d->rest + 3 * (size_t)N);
    h->h_tets_pad = tets_pad;
    h->h_rest_pad = rest_pad;

    auto fail = [&](int code) { h->release(); delete h; return code; };
#define CKC(x) do { cudaError_t e__ = (x); if (e__ != cudaSuccess) return fail(e__ == cudaErrorMemoryAllocation ? PBS_E_OUT_OF_MEMORY : PBS_E_CUDA); } while (0)
    CKC(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CKC(cudaEventCreate(&h->ev_start));
    CKC(cudaEventCreate(&h->ev_end));
    CKC(cudaEventCreateWithFlags(&h->ev_chunk[0], cudaEventDisableTiming));
    CKC(cudaEventCreateWithFlags(&h->ev_chunk[1], cudaEventDisableTiming));
    CKC(cudaMallocHost((void **)&h->h_active, 2 * sizeof(int)));
    CKC(cudaMallocHost((void **)&h->h_ctl, B * sizeof(InstCtl)));
    std::memset(h->h_ctl, 0, B * sizeof(InstCtl));
    CKC(h->tets.alloc(Tp)); CKC(h->tslot.alloc(Tp)); CKC(h->row0.alloc(Tp)); CKC(h->row1.alloc(Tp)); CKC(h->row2.alloc(Tp));
    CKC(h->info.alloc(Np)); CKC(h->inc_ptr.alloc(Np + 1)); CKC(h->inc.alloc(4 * (size_t)T));
    CKC(h->tblk_inst.alloc(h->n_tblk)); CKC(h->nblk_inst.alloc(h->n_nblk));
    CKC(h->pad2user.alloc(Np)); CKC(h->tet_user.alloc(Tp)); CKC(h->node_state.alloc(Np)); CKC(h->bad.alloc(1));
    CKC(h->uh.alloc(2 * (size_t)Np)); CKC(h->ul.alloc(2 * (size_t)Np)); CKC(h->dd.alloc(2 * (size_t)Np));
    CKC(h->oh.alloc(Np)); CKC(h->ol.alloc(Np)); CKC(h->u0h.alloc(Np)); CKC(h->u0l.alloc(Np));
    CKC(h->th.alloc(Np)); CKC(h->tl.alloc(Np)); CKC(h->v.alloc(Np)); CKC(h->vold.alloc(Np));
    CKC(h->ext.alloc(Np)); CKC(h->diag.alloc(Np)); CKC(h->rest4.alloc(Np));
    CKC(h->hist1.alloc(Np)); CKC(h->hist2.alloc(Np)); CKC(h->bh.alloc(Np)); CKC(h->bl.alloc(Np));
    CKC(h->ch.alloc(Np)); CKC(h->cl.alloc(Np));
    CKC(h->ub.alloc(Np));
    // slot-ordered hot-loop buffers (3 * 4T) also serve the per-tet probes (12 * Tp)
    CKC(h->tf.alloc(std::max(12 * (size_t)Tp, 16 * (size_t)T))); CKC(h->hd.alloc(std::max(12 * (size_t)Tp, 16 * (size_t)T)));
    CKC(h->staging.alloc(3 * (size_t)N)); CKC(h->staging2.alloc(12 * (size_t)Tp)); CKC(h->staging_ids.alloc(N));
    CKC(h->tpart.alloc(h->n_tblk)); CKC(h->npart.alloc(h->n_nblk)); CKC(h->npartf.alloc(h->n_nblk));
    CKC(h->ctl.alloc(B)); CKC(h->ctl2.alloc(B)); CKC(h->tcount.alloc(B)); CKC(h->active.alloc(4));
    CKC(cudaMemsetAsync(h->ctl2.p, 0, sizeof(InstCtl) * B, h->stream));
    CKC(cudaMemsetAsync(h->tcount.p, 0, sizeof(unsigned int) * B, h->stream));
    CKC(cudaMemsetAsync(h->active.p, 0, 4 * sizeof(int), h->stream));
    CKC(h->qrows.alloc(4 * (size_t)T)); CKC(h->rslot.alloc(12 * (size_t)T));
    h->qrow0 = h->qrows.p;
    h->qrow1 = h->qrows.p + (size_t)T;
    h->qrow2 = h->qrows.p + 2 * (size_t)T;
    h->qcor = reinterpret_cast<uint4 *>(h->qrows.p + 3 * (size_t)T);
    setup_l2_residency(h, prop);
    CKC(prepare_chunk_kernels());
    cudaStream_t s = h->stream;
    {
        const int rc = set_pass_layout(h, CHUNK_THREADS, CHUNK_TETS, CHUNK_NODES, 0, &ctl);
        if (rc != PBS_OK) return fail(rc);
    }
    CKC(cudaMemcpyAsync(h->tets.p, tets_pad.data(), sizeof(int4) * Tp, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->tslot.p, tslot.data(), sizeof(int4) * Tp, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->inc_ptr.p, iptr.data(), sizeof(int) * (Np + 1), cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->inc.p, ient.data(), sizeof(int) * 4 * (size_t)T, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->tblk_inst.p, tblk.data(), sizeof(int) * h->n_tblk, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->nblk_inst.p, nblk.data(), sizeof(int) * h->n_nblk, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->pad2user.p, h->h_pad2user.data(), sizeof(int) * Np, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->tet_user.p, h->h_tet_user.data(), sizeof(int) * Tp, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->node_state.p, h->h_node_state.data(), sizeof(int) * Np, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->ctl.p, ctl.data(), sizeof(InstCtl) * B, cudaMemcpyHostToDevice, s));
    CKC(cudaMemcpyAsync(h->rest4.p, rest4.data(), sizeof(float4) * Np, cudaMemcpyHostToDevice, s));
    CKC(cudaMemsetAsync(h->v.p, 0, sizeof(float4) * Np, s));
    CKC(cudaMemsetAsync(h->vold.p, 0, sizeof(float4) * Np, s));
    CKC(cudaMemsetAsync(h->diag.p, 0, sizeof(float4) * Np, s));
    CKC(cudaMemsetAsync(h->ext.p, 0, sizeof(float4) * Np, s));
    CKC(cudaMemsetAsync(h->tf.p, 0, sizeof(float) * std::max(12 * (size_t)Tp, 16 * (size_t)T), s));
    CKC(cudaMemsetAsync(h->hd.p, 0, sizeof(float) * std::max(12 * (size_t)Tp, 16 * (size_t)T), s));
    {
        DevBuf<float4> *zero[] = {&h->uh, &h->ul, &h->dd};
        for (auto b : zero) CKC(cudaMemsetAsync(b->p, 0, sizeof(float4) * 2 * (size_t)Np, s));
        DevBuf<float4> *zero1[] = {&h->oh, &h->ol, &h->u0h, &h->u0l, &h->th, &h->tl, &h->hist1, &h->hist2, &h->bh,
                                   &h->bl, &h->ub};
        for (auto b : zero1) CKC(cudaMemsetAsync(b->p, 0, sizeof(float4) * (size_t)Np, s));
    }
    CKC(cudaMemsetAsync(h->bad.p, 0, sizeof(int), s));
    {
        // FP64 rest state on the device
        DevBuf<double> rest_d, tmass;
        CKC(rest_d.alloc(3 * (size_t)Np));
        if (tmass.alloc(Tp) != cudaSuccess) { rest_d.release(); return fail(PBS_E_OUT_OF_MEMORY); }
        cudaError_t e = cudaMemcpyAsync(rest_d.p, rest_pad.data(), sizeof(double) * 3 * (size_t)Np, cudaMemcpyHostToDevice, s);
        DevMesh m = h->mesh();
        if (e == cudaSuccess) e = launch_rest(s, m, rest_d.p, h->density, h->row0.p, h->row1.p, h->row2.p, tmass.p, h->bad.p);
        if (e == cudaSuccess) e = launch_mass(s, m, tmass.p, h->node_state.p, h->gravity, h->info.p);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        rest_d.release();
        tmass.release();
        CKC(e);
    }
    int bad = 0;
    CKC(cudaMemcpy(&bad, h->bad.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) return fail(PBS_E_BAD_MESH);
    if (d->positions) {
        CKC(cudaMemcpyAsync(h->staging.p, d->positions, sizeof(float) * 3 * (size_t)N, cudaMemcpyHostToDevice, s));
        CKC(launch_unpack_positions(s, h->mesh(), h->staging.p, h->pad2user.p, h->u0h.p, h->u0l.p));
        CKC(cudaStreamSynchronize(s));
    }
    // default material: TetMesh.cpp:185 (E = 5e5, nu = 0.45), the reference's Lame formula
    float mu, lam;
    pbs_lame(5e5f, 0.45f, 1, &mu, &lam);
    int rc = pbs_set_material(h, PBS_MATERIAL_NEOHOOKEAN, &mu, &lam, 1);
    if (rc != PBS_OK) return fail(rc);
    CKC(cudaStreamSynchronize(s));
    *out = h;
    return PBS_OK;
#undef CKC
}

void pbs_destroy(pbs_handle *h) {
    if (!h) return;
    DeviceScope scope(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->l2_setaside) {  // the persisting lines back to normal, the set-aside returned
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    }
    h->release();
    delete h;
}

int pbs_set_l2_residency(pbs_handle *h, int enable) {
    if (!h || (enable != 0 && enable != 1)) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    if (enable && !h->l2_setaside) return PBS_E_INVALID_ARG;  // the device offers no persisting L2
    if ((enable != 0) != h->l2_use) {
        h->l2_use = enable != 0;
        h->graph_valid = false;  // the captured launches carry the window
        if (!enable) cudaCtxResetPersistingL2Cache();
    }
    return PBS_OK;
}

int pbs_set_material(pbs_handle *h, int model, const float *mu, const float *lambda, int count) {
    if (!h || !mu || !lambda || (count != 1 && count != h->T)) return PBS_E_INVALID_ARG;
    if (model != PBS_MATERIAL_NEOHOOKEAN && model != PBS_MATERIAL_STRETCH) return PBS_E_INVALID_ARG;
    for (int i = 0; i < count; ++i)
        if (!std::isfinite(mu[i]) || !std::isfinite(lambda[i])) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    // stage mu and lambda through the (3N-float) staging buffer's neighbour
    DevBuf<float> buf;
    CK(buf.alloc(2 * (size_t)count));
    cudaError_t e = cudaMemcpyAsync(buf.p, mu, sizeof(float) * count, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf.p + count, lambda, sizeof(float) * count, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = launch_set_lame(h->stream, h->Tp, h->tets.p, buf.p, buf.p + count, count, h->row1.p, h->row2.p, h->tet_user.p);
    if (e == cudaSuccess)  // the pass kernel's copy of the rows, in chunk order
        e = launch_pass_rows(h->stream, h->T, h->qperm.p, h->row0.p, h->row1.p, h->row2.p, h->qrow0, h->qrow1,
                             h->qrow2);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    buf.release();
    CK(e);
    if (h->material != model) h->graph_valid = false;
    h->material = model;
    h->dparams.incremental = model == PBS_MATERIAL_NEOHOOKEAN && h->params.incremental_stress ? 1 : 0;
    return PBS_OK;
}

int pbs_set_params(pbs_handle *h, const pbs_step_params *p) {
    if (!h) return PBS_E_INVALID_ARG;
    int rc = validate_params(p);
    if (rc != PBS_OK) return rc;
    h->params = *p;
    to_dev_params(h->params, h->dparams);
    h->dparams.incremental = h->material == PBS_MATERIAL_NEOHOOKEAN && h->params.incremental_stress ? 1 : 0;
    h->graph_valid = false;
    return PBS_OK;
}

int pbs_get_params(pbs_handle *h, pbs_step_params *p) {
    if (!h || !p) return PBS_E_INVALID_ARG;
    *p = h->params;
    return PBS_OK;
}

// CHUNK_PASSES passes and the closing settle, captured from h->stream.
static cudaError_t capture_body(pbs_handle *h, const LoopCtl *loop) {
    DevMesh m = h->mesh();
    DevState st = h->state();
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < CHUNK_PASSES && e == cudaSuccess; ++i)
        e = launch_pass(h->stream, m, h->dparams, st, h->material, i & 1);
    // the last pass's decision, so that the next run, the host and the
    // epilogue see settled control blocks
    if (e == cudaSuccess) e = launch_settle(h->stream, m, h->dparams, st, CHUNK_PASSES & 1, true, loop);
    return e;
}

// Bodies of CHUNK_PASSES passes a step needs at most (its pass cap).
static int max_runs(const pbs_handle *h) { return (h->dparams.pass_cap + CHUNK_PASSES - 1) / CHUNK_PASSES; }

// The step graph as a WHILE node over the body: k_settle's last CTA ends the
// loop when no instance runs or max_runs bodies ran, so a step is one graph
// launch and neither the host nor an extra body waits on the outcome.
static cudaError_t build_loop_graph(pbs_handle *h, cudaGraphExec_t *out) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    LoopCtl lc{};
    lc.max_runs = max_runs(h);
    e = cudaGraphConditionalHandleCreate(&lc.cond, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {};
    if (e == cudaSuccess) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = lc.cond;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    }
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(h->stream, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t ec = capture_body(h, &lc);
        cudaGraph_t body = nullptr;
        e = cudaStreamEndCapture(h->stream, &body);
        if (ec != cudaSuccess) e = ec;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    return e;
}

static int ensure_graph(pbs_handle *h) {
    if (h->graph_valid) return PBS_OK;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    h->graph_loop = build_loop_graph(h, &h->graph) == cudaSuccess;
    if (!h->graph_loop) {
        // without conditional nodes: the body alone, launched by the host
        (void)cudaGetLastError();
        h->graph = nullptr;
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t e = capture_body(h, nullptr);
        const cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) { if (g) cudaGraphDestroy(g); return PBS_E_CUDA; }
        const cudaError_t e3 = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        CK(e3);
    }
    h->graph_valid = true;
    return PBS_OK;
}

// CTAs of the frame kernel for the handle's current layout; 0 when the frame
// engine does not apply to it.
static int frame_ctas(const pbs_handle *h) {
    return frame_grid(h->mesh(), h->material, h->material == PBS_MATERIAL_NEOHOOKEAN && h->dparams.incremental,
                      h->sms);
}

// Enqueues one frame-kernel launch of at most max_passes passes with params p
// (the barrier words zeroed first).  PBS_E_INVALID_ARG when the frame engine
// does not apply to the handle's layout.
static int launch_frame_step(pbs_handle *h, const DevParams &p, int max_passes) {
    const int G = frame_ctas(h);
    if (G <= 0) return PBS_E_INVALID_ARG;
    cudaStream_t s = h->stream;
    if (!h->fsync.p) CK(h->fsync.alloc(1));
    if (h->fce.n < (size_t)G) {
        h->fce.release();
        h->fcr.release();
        CK(h->fce.alloc(G));
        CK(h->fcr.alloc(G));
    }
    CK(cudaMemsetAsync(h->fsync.p, 0, sizeof(FrameSync), s));
    FrameAux fx;
    fx.sync = h->fsync.p;
    fx.ce = h->fce.p;
    fx.cr = h->fcr.p;
    fx.max_passes = max_passes;
    CK(launch_frame(s, h->mesh(), p, h->state(), h->material, fx, G));
    return PBS_OK;
}

int pbs_step(pbs_handle *h, const float *ext, int *iters_out) {
    if (!h) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    const bool frame = h->engine == PBS_ENGINE_FRAME;
    if (frame && frame_ctas(h) <= 0) return PBS_E_INVALID_ARG;
    int rc = frame ? PBS_OK : ensure_graph(h);
    if (rc != PBS_OK) return rc;
    cudaStream_t s = h->stream;
    DevMesh m = h->mesh();
    DevState st = h->state();
    CK(cudaEventRecord(h->ev_start, s));
    if (ext) CK(cudaMemcpyAsync(h->staging.p, ext, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(h->active.p, 0, 4 * sizeof(int), s));
    CK(launch_init_ctl(s, h->B, h->dparams, st));
    CK(launch_prologue(s, m, h->dparams, st, ext ? h->staging.p : nullptr, h->pad2user.p));
    CK(launch_guess_check(s, m, h->dparams, st));
    CK(launch_ref_force(s, m, h->dparams, st));
    if (h->ws_enabled || h->guess_pending) {
        CK(launch_ws_gref(s, m, h->dparams, st, h->material));
        if (h->guess_pending)
            CK(launch_ws_choose(s, m, h->dparams, st));
        else
            CK(launch_ws_predict(s, m, h->dparams, st, h->ws_theta.p, h->ws_stats.p, h->ws_stats.p + 24,
                                 h->ws_stats.p + 48, h->hd.p, h->sms, h->ws_base, h->material));
        h->guess_pending = false;
    }
    CK(launch_to_increment(s, m, h->dparams, st));
    // The graph's WHILE node runs bodies of CHUNK_PASSES passes until no
    // instance runs; without it the host launches the body and reads the
    // active-instance count of body j-1 while body j runs, so the device never
    // idles on the poll (body j may then find every instance done).  The frame
    // engine: one launch runs every pass of the step (its pass cap ends it at
    // the latest).
    const int max_chunks = frame || h->graph_loop ? 0 : max_runs(h);
    int launched = 0;
    if (frame) {
        rc = launch_frame_step(h, h->dparams, h->dparams.pass_cap);
        if (rc != PBS_OK) return rc;
    } else if (h->graph_loop) {
        CK(cudaGraphLaunch(h->graph, s));
        CK(cudaMemcpyAsync(h->h_active, h->active.p + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    for (int j = 0; j < max_chunks; ++j) {
        ++launched;
        CK(cudaGraphLaunch(h->graph, s));
        CK(cudaMemcpyAsync(h->h_active + (j & 1), h->active.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaEventRecord(h->ev_chunk[j & 1], s));
        if (j >= 1) {
            CK(cudaEventSynchronize(h->ev_chunk[(j - 1) & 1]));
            if (h->h_active[(j - 1) & 1] == 0) break;
        }
    }
    CK(launch_from_increment(s, m, h->dparams, st));
    CK(launch_epilogue(s, m, h->dparams, st, h->pad2user.p));
    CK(cudaMemcpyAsync(h->h_ctl, h->ctl.p, sizeof(InstCtl) * h->B, cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(h->ev_end, s));
    CK(cudaMemsetAsync(h->ext.p, 0, sizeof(float4) * h->Np, s));  // fvm.cpp:188 resetExternalForce
    CK(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev_start, h->ev_end);
    h->last_ms = ms;
    if (!frame && h->graph_loop) launched = h->h_active[0];
    pbs_stats S{};
    S.status = PBS_OK;
    for (int b = 0; b < h->B; ++b) {
        const InstCtl &c = h->h_ctl[b];
        S.passes = std::max(S.passes, c.passes);
        S.iterations = std::max(S.iterations, c.k);
        S.rejections += c.rejections;
        S.converged += c.converged;
        S.warm_start_used += c.ws_used;
        S.guess_fallbacks += c.guess_bad;
        if (c.status != PBS_OK && S.status == PBS_OK) S.status = c.status;
        if (c.status == PBS_E_NONFINITE) S.status = PBS_E_NONFINITE;
    }
    S.alpha = h->h_ctl[0].alpha;
    S.rho = h->h_ctl[0].rho;
    S.omega = h->h_ctl[0].omega;
    S.energy = h->h_ctl[0].energy;
    S.residual_ratio = residual_ratio(h->h_ctl[0]);
    S.device_ms = ms;
    S.graph_launches = launched;
    h->stats = S;
    if (iters_out) *iters_out = S.iterations;
    return S.status;
}

int pbs_read_positions(pbs_handle *h, float *out) {
    if (!h || !out) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    CK(launch_pack_positions(h->stream, h->mesh(), h->u0h.p, h->u0l.p, h->pad2user.p, h->staging.p));
    CK(cudaMemcpyAsync(out, h->staging.p, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return PBS_OK;
}

static int upload_user(pbs_handle *h, const float *src, float4 *dst) {
    for (size_t i = 0; i < 3 * (size_t)h->N; ++i)
        if (!std::isfinite(src[i])) return PBS_E_INVALID_ARG;
    CK(cudaMemcpyAsync(h->staging.p, src, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyHostToDevice, h->stream));
    CK(launch_unpack(h->stream, h->Np, h->staging.p, h->pad2user.p, dst));
    CK(cudaStreamSynchronize(h->stream));
    return PBS_OK;
}

static int download_user(pbs_handle *h, const float4 *src, float *dst) {
    CK(launch_pack(h->stream, h->Np, src, h->pad2user.p, h->staging.p));
    CK(cudaMemcpyAsync(dst, h->staging.p, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return PBS_OK;
}

static int upload_positions(pbs_handle *h, const float *positions, float4 *hi, float4 *lo) {
    for (size_t i = 0; i < 3 * (size_t)h->N; ++i)
        if (!std::isfinite(positions[i])) return PBS_E_INVALID_ARG;
    CK(cudaMemcpyAsync(h->staging.p, positions, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyHostToDevice, h->stream));
    CK(launch_unpack_positions(h->stream, h->mesh(), h->staging.p, h->pad2user.p, hi, lo));
    CK(cudaStreamSynchronize(h->stream));
    return PBS_OK;
}

int pbs_update_positions(pbs_handle *h, const float *positions) {
    if (!h || !positions) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    return upload_positions(h, positions, h->u0h.p, h->u0l.p);
}

int pbs_set_node_positions(pbs_handle *h, int count, const int *ids, const float *xyz) {
    if (!h || count < 0 || count > h->N || (count > 0 && (!ids || !xyz))) return PBS_E_INVALID_ARG;
    if (count == 0) return PBS_OK;
    PBS_DEVICE_SCOPE(h->device);
    std::vector<int> pad(count);
    for (int i = 0; i < count; ++i) {
        if (ids[i] < 0 || ids[i] >= h->N) return PBS_E_INVALID_ARG;
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(xyz[3 * (size_t)i + k])) return PBS_E_INVALID_ARG;
        pad[i] = h->user2pad[ids[i]];
    }
    CK(cudaMemcpyAsync(h->staging_ids.p, pad.data(), sizeof(int) * count, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->staging.p, xyz, sizeof(float) * 3 * (size_t)count, cudaMemcpyHostToDevice, h->stream));
    CK(launch_scatter_positions(h->stream, h->mesh(), count, h->staging_ids.p, h->staging.p, h->u0h.p, h->u0l.p));
    CK(cudaStreamSynchronize(h->stream));
    return PBS_OK;
}

int pbs_set_warm_start(pbs_handle *h, const float *theta, const float *feat_mean, const float *feat_std,
                       const float *out_std, int enabled) {
    if (!h) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    if (!enabled) {
        h->ws_enabled = false;
        return PBS_OK;
    }
    if (enabled != 1 && enabled != 2) return PBS_E_INVALID_ARG;
    const int np = pbs_mlp_param_count();
    if (!theta || !feat_mean || !feat_std || !out_std) return PBS_E_INVALID_ARG;
    for (int i = 0; i < np; ++i)
        if (!std::isfinite(theta[i])) return PBS_E_INVALID_ARG;
    for (int i = 0; i < 24; ++i)
        if (!std::isfinite(feat_mean[i]) || !(feat_std[i] > 0.f)) return PBS_E_INVALID_ARG;
    for (int i = 0; i < 3; ++i)
        if (!(out_std[i] > 0.f)) return PBS_E_INVALID_ARG;
    if (!h->ws_theta.p) CK(h->ws_theta.alloc(np));
    if (!h->ws_stats.p) CK(h->ws_stats.alloc(51));
    std::vector<float> st(51);
    std::memcpy(st.data(), feat_mean, 24 * sizeof(float));
    std::memcpy(st.data() + 24, feat_std, 24 * sizeof(float));
    std::memcpy(st.data() + 48, out_std, 3 * sizeof(float));
    CK(cudaMemcpy(h->ws_theta.p, theta, sizeof(float) * np, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->ws_stats.p, st.data(), sizeof(float) * 51, cudaMemcpyHostToDevice));
    h->ws_enabled = true;
    h->ws_base = enabled == 2 ? 1 : 0;
    return PBS_OK;
}

int pbs_warm_start_features(pbs_handle *h, const float *ext, float *features, float *x_init, float *scale) {
    if (!h || !features) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    cudaStream_t s = h->stream;
    DevMesh m = h->mesh();
    DevState st = h->state();
    if (ext) CK(cudaMemcpyAsync(h->staging.p, ext, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(h->active.p, 0, 4 * sizeof(int), s));
    CK(launch_init_ctl(s, h->B, h->dparams, st));
    CK(launch_prologue(s, m, h->dparams, st, ext ? h->staging.p : nullptr, h->pad2user.p));
    DevBuf<float> out;
    CK(out.alloc(25 * (size_t)h->N));
    float *sc = out.p + 24 * (size_t)h->N;
    cudaError_t e = launch_ws_features(s, m, h->dparams, st, h->hd.p, h->pad2user.p, out.p, sc);
    if (e == cudaSuccess) e = cudaMemcpyAsync(features, out.p, sizeof(float) * 24 * (size_t)h->N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && scale) e = cudaMemcpyAsync(scale, sc, sizeof(float) * h->N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && x_init) e = launch_pack_positions(s, m, h->uh.p, h->ul.p, h->pad2user.p, h->staging.p);
    if (e == cudaSuccess && x_init)
        e = cudaMemcpyAsync(x_init, h->staging.p, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    out.release();
    CK(e);
    return PBS_OK;
}

int pbs_set_guess(pbs_handle *h, const float *positions) {
    if (!h || !positions) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    int rc = upload_positions(h, positions, h->uh.p + h->Np, h->ul.p + h->Np);
    if (rc != PBS_OK) return rc;
    h->guess_pending = true;
    return PBS_OK;
}

int pbs_get_stream(pbs_handle *h, void **stream) {
    if (!h || !stream) return PBS_E_INVALID_ARG;
    *stream = (void *)h->stream;
    return PBS_OK;
}

}  // extern "C"

// Times `passes` passes from the current state (CUDA events around each
// kernel on the handle's stream); the state the next step starts from (u0,
// velocities) is untouched.  Fails when an instance stopped before the last
// pass, leaving its counters in h->stats.
static int time_passes(pbs_handle *h, int passes, double *tet_ms, double *node_ms) {
    cudaStream_t s = h->stream;
    DevParams p = h->dparams;
    // a line-search rejection adds a pass and, under the reference control,
    // shortens the iteration budget (iterations -= k - 8): neither may end the
    // timed passes early
    p.max_iters = 4 * passes + 64;
    p.tol = 0.f;
    p.pass_cap = 4 * passes + 64;
    DevMesh m = h->mesh();
    DevState st = h->state();
    std::vector<cudaEvent_t> ev(2 * passes + 1, nullptr);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    cudaError_t e = cudaMemsetAsync(h->active.p, 0, 4 * sizeof(int), s);
    if (e == cudaSuccess) e = launch_init_ctl(s, h->B, p, st);
    if (e == cudaSuccess) e = launch_prologue(s, m, p, st, nullptr, h->pad2user.p);
    if (e == cudaSuccess) e = launch_guess_check(s, m, p, st);
    if (e == cudaSuccess) e = launch_ref_force(s, m, p, st);
    if (e == cudaSuccess) e = launch_to_increment(s, m, p, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], s);
    for (int i = 0; i < passes && e == cudaSuccess; ++i) {
        e = launch_tet_only(s, m, p, st, h->material, i & 1);
        if (e == cudaSuccess) e = cudaEventRecord(ev[2 * i + 1], s);
        if (e == cudaSuccess) e = launch_node_only(s, m, p, st, i & 1);
        if (e == cudaSuccess) e = cudaEventRecord(ev[2 * i + 2], s);
    }
    if (e == cudaSuccess) e = launch_settle(s, m, p, st, passes & 1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    double tt = 0.0, tn = 0.0;
    for (int i = 0; i < passes && e == cudaSuccess; ++i) {
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, ev[2 * i], ev[2 * i + 1]);
        cudaEventElapsedTime(&b, ev[2 * i + 1], ev[2 * i + 2]);
        tt += a;
        tn += b;
    }
    for (auto &x : ev) cudaEventDestroy(x);
    CK(e);
    // every pass must have done real work: an instance that finished early
    // (non-finite state, line-search stop) would leave no-op launches behind
    std::vector<InstCtl> c(h->B);
    CK(cudaMemcpy(c.data(), h->ctl.p, sizeof(InstCtl) * h->B, cudaMemcpyDeviceToHost));
    for (const InstCtl &x : c) {
        if (x.tet_end == x.tet_begin) continue;
        if (x.status != PBS_OK || x.passes < passes) {  // pbs_get_stats then describes the stopped instance
            pbs_stats S{};
            S.passes = x.passes; S.iterations = x.k; S.rejections = x.rejections; S.converged = x.converged;
            S.status = x.status; S.alpha = x.alpha; S.rho = x.rho; S.omega = x.omega; S.energy = x.energy;
            S.residual_ratio = residual_ratio(x);
            h->stats = S;
            return x.status != PBS_OK ? x.status : PBS_E_ITER_CAP;
        }
    }
    *tet_ms = tt / passes;
    *node_ms = tn / passes;
    return PBS_OK;
}

// The frame engine's counterpart of time_passes: one launch of exactly
// `passes` passes from the step's start state, timed with CUDA events.
static int time_frame(pbs_handle *h, int passes, double *pass_ms) {
    cudaStream_t s = h->stream;
    DevParams p = h->dparams;
    p.max_iters = 4 * passes + 64;
    p.tol = 0.f;
    p.pass_cap = 4 * passes + 64;
    DevMesh m = h->mesh();
    DevState st = h->state();
    cudaEvent_t ev[2] = {nullptr, nullptr};
    for (auto &e : ev) CK(cudaEventCreate(&e));
    cudaError_t e = cudaMemsetAsync(h->active.p, 0, 4 * sizeof(int), s);
    if (e == cudaSuccess) e = launch_init_ctl(s, h->B, p, st);
    if (e == cudaSuccess) e = launch_prologue(s, m, p, st, nullptr, h->pad2user.p);
    if (e == cudaSuccess) e = launch_guess_check(s, m, p, st);
    if (e == cudaSuccess) e = launch_ref_force(s, m, p, st);
    if (e == cudaSuccess) e = launch_to_increment(s, m, p, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], s);
    int rc = PBS_OK;
    if (e == cudaSuccess) rc = launch_frame_step(h, p, passes);
    if (e == cudaSuccess && rc == PBS_OK) e = cudaEventRecord(ev[1], s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    float ms = 0.f;
    if (e == cudaSuccess && rc == PBS_OK) cudaEventElapsedTime(&ms, ev[0], ev[1]);
    for (auto &x : ev) cudaEventDestroy(x);
    CK(e);
    if (rc != PBS_OK) return rc;
    InstCtl c;
    CK(cudaMemcpy(&c, h->ctl.p, sizeof(InstCtl), cudaMemcpyDeviceToHost));
    if (c.status != PBS_OK || c.passes < passes) {
        pbs_stats S{};
        S.passes = c.passes; S.iterations = c.k; S.rejections = c.rejections; S.converged = c.converged;
        S.status = c.status; S.alpha = c.alpha; S.rho = c.rho; S.omega = c.omega; S.energy = c.energy;
        S.residual_ratio = residual_ratio(c);
        h->stats = S;
        return c.status != PBS_OK ? c.status : PBS_E_ITER_CAP;
    }
    *pass_ms = ms / passes;
    return PBS_OK;
}

extern "C" {

int pbs_set_pass_engine(pbs_handle *h, int engine) {
    if (!h || (engine != PBS_ENGINE_GRAPH && engine != PBS_ENGINE_FRAME)) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    if (engine == PBS_ENGINE_FRAME && frame_ctas(h) <= 0) return PBS_E_INVALID_ARG;
    h->engine = engine;
    return PBS_OK;
}

int pbs_get_pass_engine(pbs_handle *h, int *engine) {
    if (!h || !engine) return PBS_E_INVALID_ARG;
    *engine = h->engine;
    return PBS_OK;
}

int pbs_profile_frame(pbs_handle *h, int passes, double *pass_ms) {
    if (!h || passes <= 0 || !pass_ms) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    return time_frame(h, passes, pass_ms);
}

int pbs_profile_kernels(pbs_handle *h, int passes, double *tet_ms, double *node_ms) {
    if (!h || passes <= 0 || !tet_ms || !node_ms) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    return time_passes(h, passes, tet_ms, node_ms);
}

int pbs_set_chunk_shape(pbs_handle *h, int threads, int chunk_tets, int chunk_nodes, int staged, int node_npt) {
    if (!h || (threads != 128 && threads != 256 && threads != 512) || chunk_tets < 1 || chunk_nodes < 4 ||
        (node_npt != 1 && node_npt != 2) ||
        4 * (size_t)chunk_tets > 65536 || chunk_nodes > 65536 || staged < 0 || staged > 2 ||
        (staged && threads == 512) ||
        chunk_smem(chunk_tets, chunk_nodes, true, staged) > (size_t)CHUNK_MAX_SMEM)
        return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    h->node_npt = node_npt;
    return set_pass_layout(h, threads, chunk_tets, chunk_nodes, staged, nullptr);
}

int pbs_autotune(pbs_handle *h, int passes, pbs_tune_result *out) {
    if (!h || passes <= 0) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    // chunk shapes: CTA threads, tets per chunk, nodes a chunk may touch,
    // staging (neo-Hookean only: 1 = rows staged in shared memory, 2 = the
    // persistent double-buffered kernel)
    static const int shapes[][4] = {{256, 1024, 448, 0}, {256, 768, 352, 0}, {256, 512, 256, 0},
                                    {128, 512, 256, 0},  {128, 256, 160, 0}, {512, 1024, 448, 0},
                                    {512, 2048, 832, 0}, {256, 640, 320, 0}, {256, 512, 256, 1},
                                    {256, 384, 208, 1},  {128, 256, 160, 1}, {128, 384, 208, 1},
                                    {256, 256, 160, 2},  {128, 256, 160, 2}, {256, 512, 256, 2},
                                    {128, 128, 96, 2},   {128, 384, 208, 0}, {256, 384, 208, 0},
                                    {128, 192, 128, 0},  {256, 256, 160, 0}};
    const int n = (int)(sizeof(shapes) / sizeof(shapes[0]));
    const bool can_stage = h->material == PBS_MATERIAL_NEOHOOKEAN;
    const int t0 = h->chunk_threads, c0 = h->chunk_tets, n0 = h->chunk_nodes, s0 = h->chunk_stage;
    double best = 1e300, first = -1.0;
    int bi = -1, tried = 0;
    for (int i = 0; i < n; ++i) {
        if (shapes[i][3] && !can_stage) continue;
        int rc = set_pass_layout(h, shapes[i][0], shapes[i][1], shapes[i][2], shapes[i][3], nullptr);
        if (rc != PBS_OK) return rc;
        double a = 0.0, b = 0.0;
        rc = time_passes(h, passes, &a, &b);  // warm-up run, then the timed one
        if (rc == PBS_OK) rc = time_passes(h, passes, &a, &b);
        if (rc != PBS_OK) {
            // the state cannot be timed: restore the shape the handle had
            const int rc2 = set_pass_layout(h, t0, c0, n0, s0, nullptr);
            return rc2 != PBS_OK ? rc2 : rc;
        }
        const double t = a + b;
        ++tried;
        if (i == 0) first = t;
        if (t < best) {
            best = t;
            bi = i;
        }
    }
    int rc = set_pass_layout(h, shapes[bi][0], shapes[bi][1], shapes[bi][2], shapes[bi][3], nullptr);
    if (rc != PBS_OK) return rc;
    // the node kernel: 1 or 2 nodes per thread (independent of the chunk shape)
    double node_ms[2] = {0.0, 0.0};
    const int npt0 = h->node_npt;
    for (int npt = 1; npt <= 2; ++npt) {
        h->node_npt = npt;
        double a = 0.0, b = 0.0;
        rc = time_passes(h, passes, &a, &b);
        if (rc == PBS_OK) rc = time_passes(h, passes, &a, &b);
        if (rc != PBS_OK) {
            h->node_npt = npt0;
            return rc;
        }
        node_ms[npt - 1] = b;
    }
    h->node_npt = node_ms[1] < node_ms[0] ? 2 : 1;
    h->graph_valid = false;
    if (out) {
        out->node_npt = h->node_npt;
        out->chunk_threads = shapes[bi][0];
        out->chunk_tets = shapes[bi][1];
        out->chunk_nodes = shapes[bi][2];
        out->chunk_staged = shapes[bi][3];
        out->n_tried = tried;
        out->pass_ms = best;
        out->default_pass_ms = first;
    }
    return PBS_OK;
}

int pbs_read_velocities(pbs_handle *h, float *v, float *v_old) {
    if (!h || (!v && !v_old)) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    int rc = PBS_OK;
    if (v) rc = download_user(h, h->v.p, v);
    if (rc == PBS_OK && v_old) rc = download_user(h, h->vold.p, v_old);
    return rc;
}

int pbs_write_velocities(pbs_handle *h, const float *v, const float *v_old) {
    if (!h || (!v && !v_old)) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    int rc = PBS_OK;
    if (v) rc = upload_user(h, v, h->v.p);
    if (rc == PBS_OK && v_old) rc = upload_user(h, v_old, h->vold.p);
    return rc;
}

int pbs_reset(pbs_handle *h) {
    if (!h) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    CK(cudaMemsetAsync(h->u0h.p, 0, sizeof(float4) * h->Np, h->stream));
    CK(cudaMemsetAsync(h->u0l.p, 0, sizeof(float4) * h->Np, h->stream));
    CK(cudaMemsetAsync(h->v.p, 0, sizeof(float4) * h->Np, h->stream));
    CK(cudaMemsetAsync(h->vold.p, 0, sizeof(float4) * h->Np, h->stream));
    // the warm start's displacement history starts over with the motion
    CK(cudaMemsetAsync(h->hist1.p, 0, sizeof(float4) * h->Np, h->stream));
    CK(cudaMemsetAsync(h->hist2.p, 0, sizeof(float4) * h->Np, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return PBS_OK;
}

int pbs_get_stats(pbs_handle *h, pbs_stats *s) {
    if (!h || !s) return PBS_E_INVALID_ARG;
    *s = h->stats;
    return PBS_OK;
}

int pbs_get_instance_stats(pbs_handle *h, int instance, pbs_stats *s) {
    if (!h || !s || instance < 0 || instance >= h->B) return PBS_E_INVALID_ARG;
    const InstCtl &c = h->h_ctl[instance];  // copied back at the end of every pbs_step
    pbs_stats S{};
    S.passes = c.passes; S.iterations = c.k; S.rejections = c.rejections; S.converged = c.converged;
    S.status = c.status; S.alpha = c.alpha; S.rho = c.rho; S.omega = c.omega; S.energy = c.energy;
    S.residual_ratio = residual_ratio(c); S.device_ms = h->stats.device_ms; S.graph_launches = h->stats.graph_launches;
    S.warm_start_used = c.ws_used;
    S.guess_fallbacks = c.guess_bad;
    *s = S;
    return PBS_OK;
}

int pbs_get_sizes(pbs_handle *h, int *n_nodes, int *n_tets, int *n_instances) {
    if (!h) return PBS_E_INVALID_ARG;
    if (n_nodes) *n_nodes = h->N;
    if (n_tets) *n_tets = h->T;
    if (n_instances) *n_instances = h->B;
    return PBS_OK;
}

int pbs_set_surface(pbs_handle *h, const int *faces, int n_faces) {
    if (!h || n_faces < 0 || (n_faces > 0 && !faces)) return PBS_E_INVALID_ARG;
    for (size_t i = 0; i < 3 * (size_t)n_faces; ++i)
        if (faces[i] < 0 || faces[i] >= h->N) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    h->faces_pad.release(); h->ring_pad.release(); h->pick_id.release(); h->pick_d2.release();
    h->n_faces = 0;
    h->h_ring_ptr.assign(1, 0);
    h->h_ring.clear();
    if (n_faces == 0) return PBS_OK;
    // TetMesh::computeBoundfaceRingIndices (TetMesh.cpp:229-277): each node's
    // neighbours through surface edges; a face's ring = its three nodes, then
    // the union of their neighbours without them, ascending
    std::vector<std::vector<int>> nbr(h->N);
    for (int f = 0; f < n_faces; ++f) {
        const int *q = faces + 3 * (size_t)f;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                if (a != b) nbr[q[a]].push_back(q[b]);
    }
    for (auto &v : nbr) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    std::vector<int4> fpad(n_faces);
    std::vector<int> tmp;
    for (int f = 0; f < n_faces; ++f) {
        const int *q = faces + 3 * (size_t)f;
        fpad[f] = make_int4(h->user2pad[q[0]], h->user2pad[q[1]], h->user2pad[q[2]], 0);
        tmp.clear();
        for (int a = 0; a < 3; ++a) tmp.insert(tmp.end(), nbr[q[a]].begin(), nbr[q[a]].end());
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        h->h_ring.insert(h->h_ring.end(), q, q + 3);
        for (int v : tmp)
            if (v != q[0] && v != q[1] && v != q[2]) h->h_ring.push_back(v);
        h->h_ring_ptr.push_back((int)h->h_ring.size());
    }
    std::vector<int> rpad(h->h_ring.size());
    for (size_t j = 0; j < rpad.size(); ++j) rpad[j] = h->user2pad[h->h_ring[j]];
    const int nb = pick_blocks(n_faces, h->sms);
    CK(h->faces_pad.alloc(n_faces)); CK(h->ring_pad.alloc(rpad.size()));
    CK(h->pick_id.alloc(nb + 1)); CK(h->pick_d2.alloc(nb));
    if (!h->drag_ext.p) CK(h->drag_ext.alloc(h->Np));
    CK(cudaMemcpyAsync(h->faces_pad.p, fpad.data(), sizeof(int4) * n_faces, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->ring_pad.p, rpad.data(), sizeof(int) * rpad.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->n_faces = n_faces;
    return PBS_OK;
}

int pbs_get_face_ring(pbs_handle *h, int face, int *ring, int capacity, int *size) {
    if (!h || !size || face < 0 || face >= h->n_faces || (ring && capacity < 0)) return PBS_E_INVALID_ARG;
    const int b = h->h_ring_ptr[face], e = h->h_ring_ptr[face + 1];
    *size = e - b;
    if (ring)
        for (int j = 0; j < std::min(e - b, capacity); ++j) ring[j] = h->h_ring[b + j];
    return PBS_OK;
}

static bool finite3(const float *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

int pbs_pick_face(pbs_handle *h, const float *orig, const float *dir, int *face) {
    if (!h || !orig || !dir || !face || h->n_faces == 0 || !finite3(orig) || !finite3(dir)) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    const int nb = pick_blocks(h->n_faces, h->sms);
    CK(launch_pick_face(h->stream, h->mesh(), h->state(), h->n_faces, h->faces_pad.p,
                        make_float3(orig[0], orig[1], orig[2]), make_float3(dir[0], dir[1], dir[2]), nb, h->pick_d2.p,
                        h->pick_id.p, h->pick_id.p + nb));
    int out = -1;
    CK(cudaMemcpyAsync(&out, h->pick_id.p + nb, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *face = out;
    return PBS_OK;
}

int pbs_drag_face_ring(pbs_handle *h, int face, const float *drag, float *ext) {
    if (!h || !drag || !ext || face < 0 || face >= h->n_faces || !finite3(drag)) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    const int b = h->h_ring_ptr[face], len = h->h_ring_ptr[face + 1] - b;
    CK(launch_drag_ring(h->stream, h->mesh(), h->state(), h->faces_pad.p, h->ring_pad.p, b, len,
                        make_float3(drag[0], drag[1], drag[2]), h->drag_ext.p));
    return download_user(h, h->drag_ext.p, ext);
}

// Block-CSR pattern of the padded mesh: per padded node, itself and every node
// sharing a tet with it, ascending; plus the CG buffers.
static int ensure_bsr(pbs_handle *h) {
    if (h->bsr_ready) return PBS_OK;
    std::vector<std::vector<int>> nb(h->Np);
    for (const int4 &q : h->h_tets_pad) {
        if (q.x < 0) continue;
        const int n[4] = {q.x, q.y, q.z, q.w};
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) nb[n[a]].push_back(n[b]);
    }
    std::vector<int> ptr(h->Np + 1, 0), col;
    for (int i = 0; i < h->Np; ++i) {
        auto &v = nb[i];
        v.push_back(i);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        col.insert(col.end(), v.begin(), v.end());
        ptr[i + 1] = (int)col.size();
        std::vector<int>().swap(v);
    }
    const size_t nnzb = col.size(), np = (size_t)h->Np;
    const int g = cg_blocks(h->Np);
    CK(h->bsr_ptr.alloc(np + 1)); CK(h->bsr_col.alloc(nnzb)); CK(h->bsr_val.alloc(9 * nnzb));
    CK(h->cg_dinv.alloc(9 * np)); CK(h->cg_part.alloc(3 * (size_t)g)); CK(h->cg_state.alloc(1));
    DevBuf<float4> *cv[] = {&h->cg_b, &h->cg_x, &h->cg_r, &h->cg_z, &h->cg_p, &h->cg_q};
    for (auto b : cv) CK(b->alloc(np));
    if (!h->h_cg) CK(cudaMallocHost(&h->h_cg, sizeof(CgState)));
    CK(cudaMemcpyAsync(h->bsr_ptr.p, ptr.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->bsr_col.p, col.data(), sizeof(int) * nnzb, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->bsr_ready = true;
    return PBS_OK;
}

// Launches 16 CG iterations on A x = b (state in cg_state) as one graph; the
// kernels of a finished solve return at once, so a group may overrun the cap.
static int cg_group(pbs_handle *h, const BsrView &A, const float *dinv9, float4 *x, double tol2, int max_iters,
                    int pnorm) {
    const void *key[3] = {A.val, dinv9, x};
    const int ki[3] = {max_iters, pnorm, A.scalar};
    bool same = h->cg_exec && h->cg_key_tol2 == tol2;
    for (int k = 0; k < 3; ++k) same = same && key[k] == h->cg_key[k] && ki[k] == h->cg_key_int[k];
    if (!same) {
        if (h->cg_exec) cudaGraphExecDestroy(h->cg_exec);
        h->cg_exec = nullptr;
        cudaStream_t s = h->stream;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 16 && e == cudaSuccess; ++k)
            e = launch_cg_iteration(s, h->Np, A, dinv9, x, h->cg_r.p, h->cg_z.p, h->cg_p.p, h->cg_q.p, h->cg_part.p,
                                    h->cg_state.p, tol2, max_iters, pnorm);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(s, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&h->cg_exec, g, 0);
        if (g) cudaGraphDestroy(g);
        CK(e);
        for (int k = 0; k < 3; ++k) { h->cg_key[k] = key[k]; h->cg_key_int[k] = ki[k]; }
        h->cg_key_tol2 = tol2;
    }
    CK(cudaGraphLaunch(h->cg_exec, h->stream));
    return PBS_OK;
}

int pbs_backward_euler_step(pbs_handle *h, float dt, float alpha, float beta, const float *ext, float tol,
                            int max_iters, int *iters_out, double *residual_out) {
    if (!h || !(dt > 0.f) || !(alpha >= 0.f) || !(beta >= 0.f) || !(tol > 0.f) || max_iters <= 0)
        return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    int rc = ensure_bsr(h);
    if (rc != PBS_OK) return rc;
    if (ext) {
        rc = upload_user(h, ext, h->ext.p);
        if (rc != PBS_OK) return rc;
    }
    cudaStream_t s = h->stream;
    const DevMesh m = h->mesh();
    const DevState st = h->state();
    BsrView A;
    A.ptr = h->bsr_ptr.p;
    A.col = h->bsr_col.p;
    A.val = h->bsr_val.p;
    const double tol2 = (double)tol * (double)tol;
    CK(launch_be_assemble(s, m, st, h->material, A, dt, alpha, beta, ext ? h->ext.p : nullptr, h->cg_b.p, h->cg_x.p,
                          h->cg_dinv.p));
    CK(launch_cg_init(s, h->Np, A, h->cg_dinv.p, h->cg_b.p, h->cg_x.p, h->cg_r.p, h->cg_z.p, h->cg_p.p,
                      h->cg_part.p, h->cg_state.p, tol2));
    // iterations in groups of 16; every kernel of a finished solve returns at
    // once, and the host reads the state once per group
    for (int it = 0; it < max_iters; it += 16) {
        rc = cg_group(h, A, h->cg_dinv.p, h->cg_x.p, tol2, max_iters, 0);
        if (rc != PBS_OK) return rc;
        CK(cudaMemcpyAsync(h->h_cg, h->cg_state.p, sizeof(CgState), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (h->h_cg->done) break;
    }
    const CgState c = *h->h_cg;
    if (iters_out) *iters_out = c.iters;
    if (residual_out) *residual_out = c.bb > 0.0 ? std::sqrt(c.rr / c.bb) : 0.0;
    if (c.status == PBS_E_NONFINITE) return PBS_E_NONFINITE;  // the state is left as it was
    CK(launch_be_finish(s, m, st, h->cg_x.p, dt));
    CK(cudaStreamSynchronize(s));
    h->guess_pending = false;
    return c.done ? c.status : PBS_E_ITER_CAP;
}

// ---- strain-based PBD and projective dynamics

// Levels of the caller's tet order per instance (a tet one level above the
// last earlier tet touching any of its nodes), the level-ordered tets, and
// the step's rest data formed as the reference forms it (launch_pbd_rest).
static int ensure_pbd(pbs_handle *h) {
    if (h->pbd_ready) return PBS_OK;
    const int B = h->B, Tp = h->Tp;
    std::vector<int> level(Tp, -1), last(h->Np, -1), grp(B + 1, 0), nlev(B, 0);
    for (int b = 0; b < B; ++b) {
        int top = -1;
        for (int tp = h->h_inst_tets[2 * b]; tp < h->h_inst_tets[2 * b + 1]; ++tp) {
            const int4 q = h->h_tets_pad[tp];
            if (q.x < 0) continue;
            const int l = 1 + std::max(std::max(last[q.x], last[q.y]), std::max(last[q.z], last[q.w]));
            level[tp] = l;
            last[q.x] = last[q.y] = last[q.z] = last[q.w] = l;
            top = std::max(top, l);
        }
        nlev[b] = top + 1;
        grp[b + 1] = grp[b] + nlev[b];
    }
    const int L = grp[B];
    std::vector<int> lvl(L + 1, 0);
    for (int b = 0; b < B; ++b)
        for (int tp = h->h_inst_tets[2 * b]; tp < h->h_inst_tets[2 * b + 1]; ++tp)
            if (level[tp] >= 0) lvl[grp[b] + level[tp] + 1]++;
    for (int l = 0; l < L; ++l) lvl[l + 1] += lvl[l];
    const int n = lvl[L];
    std::vector<int> fill(lvl.begin(), lvl.end() - 1), order(std::max(n, 1));
    for (int b = 0; b < B; ++b)
        for (int tp = h->h_inst_tets[2 * b]; tp < h->h_inst_tets[2 * b + 1]; ++tp)
            if (level[tp] >= 0) order[fill[grp[b] + level[tp]]++] = tp;
    std::vector<int4> tet(std::max(n, 1));
    for (int j = 0; j < n; ++j) tet[j] = h->h_tets_pad[order[j]];
    const size_t nn = (size_t)std::max(n, 1);
    CK(h->pbd_grp.alloc(B + 1)); CK(h->pbd_lvl.alloc(L + 1)); CK(h->pbd_tet.alloc(nn));
    CK(h->pbd_d0.alloc(nn)); CK(h->pbd_d1.alloc(nn)); CK(h->pbd_d2.alloc(nn)); CK(h->pbd_node.alloc(h->Np));
    CK(cudaMemcpy(h->pbd_grp.p, grp.data(), sizeof(int) * (B + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->pbd_lvl.p, lvl.data(), sizeof(int) * (L + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->pbd_tet.p, tet.data(), sizeof(int4) * n, cudaMemcpyHostToDevice));
    DevBuf<int> ord;  // level order -> padded tet, needed only here
    CK(ord.alloc(nn));
    cudaError_t e = cudaMemcpy(ord.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = launch_pbd_rest(h->stream, h->mesh(), ord.p, n, h->density, h->gravity, h->pbd_d0.p, h->pbd_d1.p,
                            h->pbd_d2.p, h->staging2.p, h->pbd_node.p);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    ord.release();
    CK(e);
    h->pbd_groups = B;
    // positions in the cluster's distributed shared memory when every
    // instance's nodes fit 16 slices (a few instances; batches of many small
    // instances keep the global-memory sweep)
    h->pbd_smem = 0;
    if (B <= 4) {
        int slice = 0;
        for (int b = 0; b < B; ++b)
            slice = std::max(slice, (h->h_inst_nodes[2 * b + 1] - h->h_inst_nodes[2 * b] + 15) / 16);
        const int smem = std::max(slice, 1) * (int)sizeof(float4);
        if (slice <= 0xffff && pbd_dsmem_fits(smem)) {
            std::vector<int4> gn(B), codes(std::max(n, 1));
            for (int b = 0; b < B; ++b) {
                const int nb = h->h_inst_nodes[2 * b], cnt = h->h_inst_nodes[2 * b + 1] - nb;
                gn[b] = make_int4(nb, std::max((cnt + 15) / 16, 1), cnt, 0);
            }
            for (int b = 0; b < B; ++b)
                for (int j = lvl[grp[b]]; j < lvl[grp[b + 1]]; ++j) {
                    const int *q = &tet[j].x;
                    int c[4];
                    for (int k = 0; k < 4; ++k) {
                        const int loc = q[k] - gn[b].x;
                        c[k] = ((loc / gn[b].y) << 16) | (loc % gn[b].y);
                    }
                    codes[j] = make_int4(c[0], c[1], c[2], c[3]);
                }
            CK(h->pbd_codes.alloc(codes.size())); CK(h->pbd_gnode.alloc(B));
            CK(cudaMemcpy(h->pbd_codes.p, codes.data(), sizeof(int4) * codes.size(), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(h->pbd_gnode.p, gn.data(), sizeof(int4) * B, cudaMemcpyHostToDevice));
            h->pbd_smem = smem;
        }
    }
    h->pbd_ready = true;
    return PBS_OK;
}

static int ensure_dyn_buffers(pbs_handle *h) {
    if (h->dyn_px.p) return PBS_OK;
    CK(h->dyn_px.alloc(h->Np)); CK(h->dyn_x0.alloc(h->Np)); CK(h->dyn_s.alloc(h->Np));
    return PBS_OK;
}

static bool finite_n(const float *v, int n) {
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

int pbs_pbd_step(pbs_handle *h, float dt, int iterations, const float *stretch, const float *shear,
                 const float *ext) {
    if (!h || !(dt > 0.f) || !std::isfinite(dt) || iterations < 0 || (stretch && !finite_n(stretch, 3)) ||
        (shear && !finite_n(shear, 3)))
        return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    int rc = ensure_pbd(h);
    if (rc == PBS_OK) rc = ensure_dyn_buffers(h);
    if (rc == PBS_OK && ext) rc = upload_user(h, ext, h->ext.p);
    if (rc != PBS_OK) return rc;
    const float st_def[3] = {1.f, 1.f, 1.f}, sh_def[3] = {0.8f, 0.8f, 0.8f};
    cudaStream_t s = h->stream;
    const DevMesh m = h->mesh();
    const DevState st = h->state();
    CK(launch_pbd_begin(s, m, st, h->pbd_node.p, ext ? h->ext.p : nullptr, dt, h->dyn_px.p, h->dyn_x0.p));
    if (iterations > 0) {
        PbdView v;
        v.grp = h->pbd_grp.p; v.lvl = h->pbd_lvl.p; v.tet = h->pbd_tet.p;
        v.d0 = h->pbd_d0.p; v.d1 = h->pbd_d1.p; v.d2 = h->pbd_d2.p; v.px = h->dyn_px.p;
        if (h->pbd_smem > 0)
            CK(launch_pbd_sweeps_dsmem(s, v, h->pbd_codes.p, h->pbd_gnode.p, h->pbd_groups, h->pbd_smem, iterations,
                                       stretch ? stretch : st_def, shear ? shear : sh_def));
        else
            CK(launch_pbd_sweeps(s, v, h->pbd_groups, iterations, stretch ? stretch : st_def, shear ? shear : sh_def));
    }
    CK(launch_dyn_end(s, m, st, h->dyn_px.p, h->dyn_x0.p, dt, 0));
    CK(cudaStreamSynchronize(s));
    h->guess_pending = false;
    return PBS_OK;
}

int pbs_pd_step(pbs_handle *h, float dt, float dt_matrix, float stiffness, int iterations, const float *ext,
                float tol, int max_cg, int *cg_iters_out) {
    if (!h || !(dt > 0.f) || !std::isfinite(dt) || !(dt_matrix >= 0.f) || !std::isfinite(dt_matrix) ||
        !(stiffness > 0.f) || !std::isfinite(stiffness) || iterations < 0 || !(tol > 0.f) || max_cg <= 0)
        return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    const float dtm = dt_matrix > 0.f ? dt_matrix : dt;
    int rc = ensure_bsr(h);
    if (rc == PBS_OK) rc = ensure_dyn_buffers(h);
    if (rc == PBS_OK && ext) rc = upload_user(h, ext, h->ext.p);
    if (rc != PBS_OK) return rc;
    cudaStream_t s = h->stream;
    const DevMesh m = h->mesh();
    const DevState st = h->state();
    BsrView A;
    A.ptr = h->bsr_ptr.p;
    A.col = h->bsr_col.p;
    A.scalar = 1;
    if (!h->pd_val.p) {
        int nnzb = 0;
        CK(cudaMemcpy(&nnzb, h->bsr_ptr.p + h->Np, sizeof(int), cudaMemcpyDeviceToHost));
        CK(h->pd_val.alloc((size_t)nnzb));
        CK(h->pd_dinv.alloc(9 * (size_t)h->Np));
    }
    A.val = h->pd_val.p;
    if (!h->pd_ready || h->pd_dtm != dtm || h->pd_k != stiffness) {
        CK(launch_pd_assemble(s, m, A, dtm, stiffness, h->pd_dinv.p));
        h->pd_ready = true;
        h->pd_dtm = dtm;
        h->pd_k = stiffness;
    }
    CK(launch_pd_begin(s, m, st, ext ? h->ext.p : nullptr, dt, h->dyn_s.p, h->dyn_px.p, h->dyn_x0.p));
    const double tol2 = (double)tol * (double)tol;
    int total = 0, status = PBS_OK;
    for (int it = 0; it < iterations; ++it) {
        CK(launch_pd_residual(s, m, h->dyn_px.p, stiffness, dt, dtm, reinterpret_cast<float4 *>(h->tf.p),
                              h->dyn_s.p, h->dyn_x0.p, h->cg_b.p, h->cg_x.p));
        CK(launch_cg_init(s, h->Np, A, h->pd_dinv.p, h->cg_b.p, h->cg_x.p, h->cg_r.p, h->cg_z.p, h->cg_p.p,
                          h->cg_part.p, h->cg_state.p, tol2, 1));
        for (int k0 = 0; k0 < max_cg; k0 += 16) {
            rc = cg_group(h, A, h->pd_dinv.p, h->cg_x.p, tol2, max_cg, 1);
            if (rc != PBS_OK) return rc;
            CK(cudaMemcpyAsync(h->h_cg, h->cg_state.p, sizeof(CgState), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (h->h_cg->done) break;
        }
        const CgState c = *h->h_cg;
        total += c.iters;
        if (c.status == PBS_E_NONFINITE) {
            if (cg_iters_out) *cg_iters_out = total;
            return PBS_E_NONFINITE;  // the state is left as it was
        }
        if (!c.done || c.status == PBS_E_ITER_CAP) status = PBS_E_ITER_CAP;
        CK(launch_pd_apply(s, h->Np, h->dyn_px.p, h->cg_x.p));
    }
    CK(launch_dyn_end(s, m, st, h->dyn_px.p, h->dyn_x0.p, dt, 1));
    CK(cudaStreamSynchronize(s));
    h->guess_pending = false;
    if (cg_iters_out) *cg_iters_out = total;
    return status;
}

int pbs_get_incidence(pbs_handle *h, int *row_ptr, int *entries) {
    if (!h || !row_ptr || !entries) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    std::vector<int> iptr(h->Np + 1), ient(4 * (size_t)h->T);
    CK(cudaMemcpy(iptr.data(), h->inc_ptr.p, sizeof(int) * (h->Np + 1), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ient.data(), h->inc.p, sizeof(int) * 4 * (size_t)h->T, cudaMemcpyDeviceToHost));
    // translate padded ids back to the caller's numbering
    row_ptr[0] = 0;
    size_t w = 0;
    for (int u = 0; u < h->N; ++u) {
        int ip = h->user2pad[u];
        for (int j = iptr[ip]; j < iptr[ip + 1]; ++j) {
            int tp = ient[j] >> 2, c = ient[j] & 3;
            entries[w++] = 4 * h->h_tet_user[tp] + c;
        }
        row_ptr[u + 1] = (int)w;
    }
    return PBS_OK;
}

int pbs_get_rest_data(pbs_handle *h, float *dm_inv9, float *signed_vol, float *mass, float *grav_y) {
    if (!h) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    std::vector<float4> r0(h->Tp), r1(h->Tp), r2(h->Tp), inf(h->Np);
    CK(cudaMemcpy(r0.data(), h->row0.p, sizeof(float4) * h->Tp, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r1.data(), h->row1.p, sizeof(float4) * h->Tp, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r2.data(), h->row2.p, sizeof(float4) * h->Tp, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(inf.data(), h->info.p, sizeof(float4) * h->Np, cudaMemcpyDeviceToHost));
    for (int tp = 0; tp < h->Tp; ++tp) {
        int t = h->h_tet_user[tp];
        if (t < 0) continue;
        if (dm_inv9) {
            float *o = dm_inv9 + 9 * (size_t)t;
            o[0] = r0[tp].x; o[1] = r0[tp].y; o[2] = r0[tp].z;
            o[3] = r1[tp].x; o[4] = r1[tp].y; o[5] = r1[tp].z;
            o[6] = r2[tp].x; o[7] = r2[tp].y; o[8] = r2[tp].z;
        }
        if (signed_vol) signed_vol[t] = r0[tp].w;
    }
    for (int u = 0; u < h->N; ++u) {
        int ip = h->user2pad[u];
        if (mass) mass[u] = inf[ip].x;
        if (grav_y) grav_y[u] = inf[ip].y;
    }
    return PBS_OK;
}

// The saved-state buffers are rewritten at iteration 0 of every step, so
// between steps they serve as scratch for evaluating given positions.
// The displacement pair (hi, lo) the probes evaluate: the uploaded positions,
// or the current state.
static int eval_common(pbs_handle *h, const float *positions, const float4 **xsrc, const float4 **xlo = nullptr) {
    if (positions) {
        int rc = upload_positions(h, positions, h->oh.p, h->ol.p);
        if (rc != PBS_OK) return rc;
        *xsrc = h->oh.p;
        if (xlo) *xlo = h->ol.p;
    } else {
        *xsrc = h->u0h.p;
        if (xlo) *xlo = h->u0l.p;
    }
    return PBS_OK;
}

int pbs_eval_tets(pbs_handle *h, const float *positions, float *corner_forces, float *energy, float *hess_diag) {
    if (!h) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    const float4 *x, *xl;
    int rc = eval_common(h, positions, &x, &xl);
    if (rc != PBS_OK) return rc;
    // per-tet outputs land in tf / hd / staging2 (padded order), then are
    // compacted into the caller's tet order on the host
    struct Counter {  // freed on every return path
        DevBuf<unsigned int> b;
        ~Counter() { b.release(); }
    } n64_buf;
    DevBuf<unsigned int> &n64 = n64_buf.b;
    CK(n64.alloc(1));
    CK(cudaMemsetAsync(n64.p, 0, sizeof(unsigned int), h->stream));
    CK(launch_eval_tets(h->stream, h->mesh(), x, h->material, h->dparams.clamp_cpu, h->tf.p, h->staging2.p, h->hd.p,
                        n64.p, xl));
    std::vector<float> tf(12 * (size_t)h->Tp), hd(12 * (size_t)h->Tp), en(h->Tp);
    unsigned int n64_host = 0;
    CK(cudaMemcpyAsync(tf.data(), h->tf.p, sizeof(float) * tf.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(hd.data(), h->hd.p, sizeof(float) * hd.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(en.data(), h->staging2.p, sizeof(float) * en.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(&n64_host, n64.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->last_fp64_svd = (int)n64_host;
    for (int tp = 0; tp < h->Tp; ++tp) {
        int t = h->h_tet_user[tp];
        if (t < 0) continue;
        if (corner_forces) std::memcpy(corner_forces + 12 * (size_t)t, &tf[12 * (size_t)tp], 12 * sizeof(float));
        if (hess_diag) std::memcpy(hess_diag + 12 * (size_t)t, &hd[12 * (size_t)tp], 12 * sizeof(float));
        if (energy) energy[t] = en[tp];
    }
    return PBS_OK;
}

int pbs_eval_fp64_svd_count(pbs_handle *h, int *count) {
    if (!h || !count) return PBS_E_INVALID_ARG;
    *count = h->last_fp64_svd;
    return PBS_OK;
}

int pbs_eval_base_force(pbs_handle *h, const float *positions, double *forces) {
    if (!h || !positions || !forces) return PBS_E_INVALID_ARG;
    if (h->material != PBS_MATERIAL_NEOHOOKEAN) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    const float4 *x;
    int rc = eval_common(h, positions, &x);
    if (rc != PBS_OK) return rc;
    struct Scratch {  // freed on every return path
        DevBuf<float4> b;
        ~Scratch() { b.release(); }
    } sb;
    CK(sb.b.alloc(4 * (size_t)h->Np));
    // the step's base-force kernels on the displacement's hi words, with the
    // body forces off and the sums landing in the scratch pair
    DevParams p = h->dparams;
    p.incremental = 1;
    p.body_scale = 0.f;
    DevState st = h->state();
    st.ub = const_cast<float4 *>(x);
    st.bh = sb.b.p;
    st.bl = sb.b.p + h->Np;
    st.ch = sb.b.p + 2 * (size_t)h->Np;  // the gather's gradient constant: scratch too
    st.cl = sb.b.p + 3 * (size_t)h->Np;
    CK(launch_ref_force(h->stream, h->mesh(), p, st));
    std::vector<float4> b(2 * (size_t)h->Np);
    CK(cudaMemcpyAsync(b.data(), sb.b.p, sizeof(float4) * b.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < h->Np; ++i) {
        const int u = h->h_pad2user[i];
        if (u < 0) continue;
        const float4 hi = b[i], lo = b[h->Np + i];
        forces[3 * (size_t)u] = (double)hi.x + (double)lo.x;
        forces[3 * (size_t)u + 1] = (double)hi.y + (double)lo.y;
        forces[3 * (size_t)u + 2] = (double)hi.z + (double)lo.z;
    }
    return PBS_OK;
}

int pbs_eval_nodes(pbs_handle *h, const float *positions, float *forces, float *hess_diag) {
    if (!h) return PBS_E_INVALID_ARG;
    PBS_DEVICE_SCOPE(h->device);
    const float4 *x, *xl;
    int rc = eval_common(h, positions, &x, &xl);
    if (rc != PBS_OK) return rc;
    DevBuf<float> out;
    CK(out.alloc(6 * (size_t)h->N));
    cudaError_t e = launch_eval_tets(h->stream, h->mesh(), x, h->material, h->dparams.clamp_cpu, h->tf.p, nullptr,
                                     h->hd.p, nullptr, xl);
    if (e == cudaSuccess) e = launch_gather(h->stream, h->mesh(), h->tf.p, h->hd.p, h->pad2user.p, out.p, out.p + 3 * (size_t)h->N);
    if (e == cudaSuccess && forces) e = cudaMemcpyAsync(forces, out.p, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && hess_diag) e = cudaMemcpyAsync(hess_diag, out.p + 3 * (size_t)h->N, sizeof(float) * 3 * (size_t)h->N, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    out.release();
    CK(e);
    return PBS_OK;
}

// IsotropicMaterial::allocateGlobalStiffnessMatrix (IsotropicMaterial.cpp:554-644):
// rows 3n+d hold the sorted columns 3m+e of every node m sharing a tet with n.
int pbs_stiffness_pattern(int n_nodes, int n_tets, const int *tets, int *nnz, int *row_ptr, int *col, int *diag_idx,
                          int *kid48) {
    if (n_nodes <= 0 || n_tets < 0 || !tets || !nnz) return PBS_E_INVALID_ARG;
    std::vector<int64_t> pairs;
    pairs.reserve(16 * (size_t)n_tets);
    for (int t = 0; t < n_tets; ++t)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) {
                int na = tets[4 * (size_t)t + a], nb = tets[4 * (size_t)t + b];
                if (na < 0 || na >= n_nodes || nb < 0 || nb >= n_nodes) return PBS_E_BAD_MESH;
                pairs.push_back(((int64_t)na << 32) | (uint32_t)nb);
            }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    std::vector<int> nptr(n_nodes + 1, 0);
    for (int64_t pr : pairs) nptr[(pr >> 32) + 1]++;
    for (int i = 0; i < n_nodes; ++i) nptr[i + 1] += nptr[i];
    const int64_t total = 9 * (int64_t)pairs.size();
    if (total > INT32_MAX) return PBS_E_CAPACITY;
    *nnz = (int)total;
    if (!col) return PBS_OK;
    if (!row_ptr) return PBS_E_INVALID_ARG;
    row_ptr[0] = 0;
    for (int n = 0; n < n_nodes; ++n) {
        int deg = nptr[n + 1] - nptr[n];
        for (int d = 0; d < 3; ++d) {
            int r = 3 * n + d;
            int start = 9 * nptr[n] + d * 3 * deg;
            row_ptr[r + 1] = start + 3 * deg;
            for (int j = 0; j < deg; ++j) {
                int m = (int)(pairs[nptr[n] + j] & 0xffffffff);
                for (int e = 0; e < 3; ++e) col[start + 3 * j + e] = 3 * m + e;
            }
        }
    }
    auto slot = [&](int r, int c) {
        const int *b = col + row_ptr[r], *e = col + row_ptr[r + 1];
        return (int)(std::lower_bound(b, e, c) - col);
    };
    if (diag_idx)
        for (int r = 0; r < 3 * n_nodes; ++r) diag_idx[r] = slot(r, r);
    if (kid48)
        for (int t = 0; t < n_tets; ++t)
            for (int fi = 0; fi < 4; ++fi)
                for (int fj = 0; fj < 3; ++fj) {
                    int gki = 3 * tets[4 * (size_t)t + fi] + fj;
                    for (int ni = 0; ni < 4; ++ni) kid48[48 * (size_t)t + (fi * 3 + fj) * 4 + ni] = slot(gki, 3 * tets[4 * (size_t)t + ni]);
                }
    return PBS_OK;
}

}  // extern "C"

void pbs::handle_view(const pbs_handle *h, HandleView *v) {
    v->device = h->device;
    v->stream = h->stream;
    v->material = h->material;
    v->mesh = h->mesh();
    v->pad2user = h->pad2user.p;
}
