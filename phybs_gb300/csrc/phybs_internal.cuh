// Internal device layout of a descent-step handle.
//
// HBM layout (Np / Tp = node / tet counts padded so that every instance starts
// on a PAD boundary and every 256-wide block belongs to one instance):
//   tets        int4[Tp]           padded node ids of the 4 corners
//   row0..2     float4[Tp] each    rows of Dm^-1; .w = {det Dm/6, mu, lambda}
//   uh, ul      float4[2][Np]      displacement u = x - X as an FP32 (hi, lo)
//                                  pair, ping-ponged between passes (with
//                                  incremental stress, during the passes: the
//                                  increment u - ub as such a pair)
//   dd          float4[2][Np]      last step d = u_k - u_{k-1} (Chebyshev history)
//   oh, ol      float4[Np]         displacement saved at the last accepted
//                                  line-search check (the reference's x_old)
//   u0h, u0l    float4[Np]         displacement at the start of the step
//   th, tl      float4[Np]         inertial target x~ - X (hi, lo)
//   bh, bl      float4[Np]         per-step force constant b (hi, lo)
//   ch, cl      float4[Np]         per-step gradient constant c = (M / h^2) x~ + b (hi, lo);
//                                  incremental stress: (M / h^2)(x~ - base) + b
//   v, vold     float4[Np]         velocities of this and the previous step
//   ext, diag   float4[Np]         external force; Jacobi diagonal + M/h^2
//   info        float4[Np]         {effective mass (pins 1e8), gravity_y,
//                                   state 0 free / 1 pinned / 2 padding, lumped mass}
//   rest        float4[Np]         rest positions X
//   inc_ptr     int[Np+1], inc int[4T]   node -> 4*tet+corner gather, canonical order
//   tslot       int4[Tp]           for each tet corner, its slot in the gather
//                                  (its position in inc): the per-tet kernel writes
//                                  corner forces straight into node-major order
//   tf, hd      float4[4T]         corner forces / Jacobi-diagonal terms by slot;
//                                  node i owns slots inc_ptr[i] .. inc_ptr[i+1]-1
//   tpart       double2[n_tblk]    per tet-block {sum e, sum e^2} of the energy
// Pass layout (the per-tet kernel of a descent pass works on chunks: runs of
// at most CHUNK_TETS tets of one instance, in Morton order of their centroids,
// touching at most CHUNK_NODES nodes):
//   chunk       int4[n_chunks]     {first pass tet, tet count, first local entry, local count}
//   qrow0..2    float4[T] each     row0..2 of the pass tets, in pass (chunk) order
//   qcor        uint4[T]           corner ids of a pass tet, two 16-bit fields a word:
//                                  {loc0 | loc1 << 16, loc2 | loc3 << 16, slot0 | slot1 << 16,
//                                  slot2 | slot3 << 16}; loc = local node of the tet's chunk,
//                                  slot = its shared-memory slot (a local node's slots are
//                                  contiguous, in (tet, corner) order)
//   lmeta       int4[L]            per local node {padded node id (ascending per chunk), first
//                                  slot, end slot, where the chunk's partial for the node goes}
//   pptr        int[Np+1]          node i's partials: part[pptr[i] .. pptr[i+1]-1], by chunk
//   part, parth float4[L]          per (node, chunk) partial force / Jacobi-diagonal sums
//   cpart       double2[n_chunks]  per chunk {sum e, sum e^2}
//   rslot       double[3][4T]      per-step FP64 corner forces at the base, by gather slot
//   npart       double[n_nblk]     per node-block |g|^2 (warm-start reference)
//   npartf      float[n_nblk]      per node-block |g|^2 of a pass (FP32 block sums)
//   ctl         InstCtl[n_inst]    per-instance descent state
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace pbs {

constexpr int PAD = 256;    // instance alignment (tets and nodes)
constexpr int BLOCK = 256;  // threads per block of the step kernels (nodes per node block)
// nodes per thread of the node kernel (BLOCK / npt threads per CTA): 1 or 2,
// picked by pbs_autotune
constexpr int NODE_NPT_DEFAULT = 1;
// Default chunk shape of the per-tet pass kernel (pbs_autotune may pick
// another): at most CHUNK_TETS tets touching at most CHUNK_NODES nodes, one
// CTA of CHUNK_THREADS threads per chunk.
constexpr int CHUNK_TETS = 1024;
constexpr int CHUNK_NODES = 448;
constexpr int CHUNK_THREADS = 256;
constexpr int CHUNK_MAX_SMEM = 200 * 1024;
// Dynamic shared memory of the per-tet pass kernel for a chunk shape and a
// staging mode: 0 = node words (u hi, u lo, and the force base with
// incremental stress, 16 B each) and one float4 per corner slot (written and
// read with one 128-bit access each); 1 = also the chunk's per-tet rows and
// corner records (64 B per tet) and local-node records (16 B per node); 2 =
// the persistent kernel, two buffers of rows, records and node words plus one
// set of slots.
__host__ __device__ constexpr size_t chunk_smem(int tets, int nodes, bool inc, int stage = 0) {
    return stage == 2 ? 2 * ((inc ? 4 : 3) * sizeof(float4) * (size_t)nodes + 64 * (size_t)tets) +
                            sizeof(float4) * 4 * (size_t)tets
                      : (inc ? 3 : 2) * sizeof(float4) * (size_t)nodes + sizeof(float4) * 4 * (size_t)tets +
                            (stage ? 64 * (size_t)tets + sizeof(int4) * (size_t)nodes : 0);
}

// Step parameters as the kernels see them (a by-value kernel argument).
struct DevParams {
    float h, h2inv;
    int max_iters;
    float tol;
    int control;
    float alpha0, alpha_min, alpha_shrink;
    int ls_every, hd_every;
    int n_profile;
    int profile_k[4];
    float profile_rho[4];
    float damping, warm_start, body_scale;
    int clamp_cpu;
    int pass_cap;
    float energy_slack;  // reject only if E > E_old + slack * 2^-24 * sqrt(sum e^2)
    float alpha_grow;    // RESTART: alpha <- min(alpha * alpha_grow, alpha0) on an accepted check
    int incremental;     // neo-Hookean: passes evaluate P(F) - P(F_base) against an FP64 force at the
                         // step's initial guess (the base)
};

// What the node kernel does in a pass (decided by the tet kernel's last block
// on line-search passes).
enum PassAction : int { ACT_STEP = 0, ACT_SAVE_STEP = 1, ACT_RESTORE = 2 };

// Per-instance descent state.
struct __align__(16) InstCtl {
    int k, iters, done, passes;
    int rejections, converged, status, par;
    int action, k_restart;  // k_restart: first iteration of the current rho schedule (RESTART control)
    unsigned int counter_t, counter_n;
    float alpha, rho, omega;
    int force_check;  // RESTART control: a non-finite residual makes the next pass a line-search pass
    int g0_fixed;     // g0 was set before iteration 0 (the plain guess's residual, warm start on)
    int ws_used;      // this step started from the learned guess
    float ell;        // mean edge length of the instance (feature scale)
    int guess_bad;    // RESTART control: the inertial guess inverts a tet; the step starts from u0
    double energy, energy_old, g0, r2;  // r2: |g|^2 of the last pass (ratio = sqrt(r2) / g0, on the host)
    // static ranges (padded indices)
    int node_begin, node_end, tet_begin, tet_end;
    int tblk_begin, tblk_end, nblk_begin, nblk_end;
    int cblk_begin, cblk_end;  // the instance's chunks
    // graph path: the pass decision of the last node update is not taken yet
    // (the next pass's first chunk or k_settle takes it); void_pass: this
    // pass's node update copies the state unchanged (a residual that turned
    // non-finite forces an energy check the pass's tet kernel did not make)
    int pending, void_pass;
    double g1;                             // |g| at the learned candidate (extrapolation base)
    double pad6;
};

// |g| / |g0| of an instance's last pass (-1 before the first pass).
inline double residual_ratio(const InstCtl &c) {
    if (c.r2 < 0.0 || c.g0 < 0.0) return -1.0;
    return c.g0 > 0.0 ? __builtin_sqrt(c.r2) / c.g0 : 0.0;
}

struct DevMesh {
    int Np, Tp, n_inst;
    int n_tblk, n_nblk;
    const int4 *tets;
    const float4 *row0, *row1, *row2;
    const int *inc_ptr, *inc;
    const int4 *tslot;
    const float4 *info, *rest;
    const int *tblk_inst, *nblk_inst;
    // pass layout
    int n_chunks, chunk_tets, chunk_nodes, chunk_threads, chunk_stage;
    int node_npt;
    const int4 *chunk;
    const int *chunk_inst;
    const float4 *qrow0, *qrow1, *qrow2;
    const uint4 *qcor;
    const int4 *lmeta;
    const int *pptr;
    int stream_grid;  // CTAs of the persistent chunk kernel (chunk_stage 2)
    // L2 access-policy window of the per-tet kernels' launches (host side):
    // the pass rows and records persist in L2 at hit ratio l2_hit; null = off
    const void *l2_base;
    size_t l2_bytes;
    float l2_hit;
};

struct DevState {
    float4 *uh, *ul, *dd;  // [2][Np] each; with incremental stress, during the passes (uh, ul) is
                           // the increment over ub (k_to_increment / k_from_increment)
    float4 *oh, *ol, *u0h, *u0l, *th, *tl;
    float4 *v, *vold, *ext, *diag;
    float4 *hist1, *hist2;  // displacement of the last step and of the one before
    float4 *ub;             // base displacement of the increments: the step's initial guess (hi word)
    float4 *bh, *bl;        // per node (hi, lo): elastic force at the base (incremental mode)
                            // plus body_force_scale * (external + gravity)
    float4 *ch, *cl;        // per node (hi, lo): c = (M / h^2) x~ + b, the step-constant part of
                            // the gradient g = (M / h^2) u - c - f (the node update reads these
                            // two words instead of x~ and b); with incremental stress the passes'
                            // u is the increment over the base and c = (M / h^2)(x~ - base) + b
    float *tf, *hd;
    double2 *tpart, *cpart;
    double *npart;
    float *npartf;
    float4 *part, *parth;
    double *rslot;  // 3 * 4T: FP64 corner forces at the base, by gather slot
    InstCtl *ctl;   // the control blocks between passes (and between steps)
    InstCtl *ctl2;  // the graph path's second copy: a pass reads one and writes the other
    unsigned int *tcount;  // per instance: the chunks of a line-search pass that finished
    int *active;  // [0] instances not yet done, [1] a device wait gave up (sticky for the step),
                  // [2] bodies of the step graph's loop run so far, [3] k_settle's ticket
};

// The control-block copy a pass with parity q reads (its tet kernel) or, with
// q ^ 1, the one its decisions go to and its node kernel reads.
__device__ __forceinline__ InstCtl *ctl_buf(const DevState &st, int q) { return q ? st.ctl2 : st.ctl; }

// Chebyshev omega for iteration k from the persistent (rho, omega), as
// DescentOptimize.cpp:156-175 / CUDAInterface.cu:967-986 compute it in FP32.
__device__ __host__ __forceinline__ void chebyshev_schedule(const DevParams &p, int k, float &rho, float &omega) {
    if (k == 0) { rho = 0.0f; omega = 1.0f; }
#ifdef __CUDA_ARCH__
    omega = __fdiv_rn(4.0f, __fsub_rn(4.0f, __fmul_rn(__fmul_rn(rho, rho), omega)));
#else
    omega = 4.0f / (4.0f - rho * rho * omega);
#endif
    // a fixed trip count (n_profile <= 4): constant indices keep the kernel
    // parameter's arrays out of local memory
    bool hit = false;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (hit || i >= p.n_profile) continue;
        if (k == p.profile_k[i] - 1) { rho = 0.0f; omega = 1.0f; }
        if (k == p.profile_k[i]) {
            rho = p.profile_rho[i];
#ifdef __CUDA_ARCH__
            omega = __fdiv_rn(2.0f, __fsub_rn(2.0f, __fmul_rn(rho, rho)));
#else
            omega = 2.0f / (2.0f - rho * rho);
#endif
            hit = true;
        }
    }
}

__device__ __forceinline__ float node_ell(const DevMesh &m, const DevState &st, int i) {
    return st.ctl[m.nblk_inst[i / BLOCK]].ell;
}
__device__ __forceinline__ int node_ctl_ws(const DevMesh &m, const DevState &st, int i) {
    return st.ctl[m.nblk_inst[i / BLOCK]].ws_used;
}

// Host: the pass layout of a packed mesh (chunks.cu).  tets: padded corner ids
// (-1 rows are padding); rest: padded rest positions (3 per node); ctl: the
// instances' node / tet ranges, whose cblk ranges are filled in.
struct ChunkLayout {
    std::vector<int4> chunk;
    std::vector<int> chunk_inst, qperm, pptr;
    std::vector<uint4> qcor;
    std::vector<int4> lmeta;
    int max_local = 0;
};
void build_chunks(int Np, const std::vector<int4> &tets, const std::vector<double> &rest, std::vector<InstCtl> &ctl,
                  int chunk_tets, int chunk_nodes, ChunkLayout &out);
cudaError_t launch_pass_rows(cudaStream_t s, int T, const int *qperm, const float4 *row0, const float4 *row1,
                             const float4 *row2, float4 *q0, float4 *q1, float4 *q2);
cudaError_t prepare_chunk_kernels();
// CTAs of the persistent chunk kernel (chunk_stage 2) for this mesh, material
// and stress mode on a device with `sms` SMs; 0 when it does not apply.
int stream_grid(const DevMesh &m, int material, bool inc, int sms);

// The persistent frame kernel (chunks.cu): one cooperative launch runs a
// step's passes of a one-instance handle, with grid barriers between its tet
// and node phases.  FrameSync: the barrier's words (zeroed before a launch);
// ce / cr: per-CTA {sum e, sum e^2} of a check pass and {|g|^2, 0} of a pass.
struct FrameSync {
    unsigned int count, gen;
    int err;  // a barrier wait ran out: the step ends with PBS_E_DEVICE_TIMEOUT
    int pad;
};
struct FrameAux {
    FrameSync *sync;
    double2 *ce, *cr;
    int max_passes;
};
// Co-resident CTAs of the frame kernel for this mesh and shape (at most one
// per chunk); 0 when the kernel does not apply (several instances, a staged
// chunk shape, a thread count without an instantiation).
int frame_grid(const DevMesh &m, int material, bool inc, int sms);
cudaError_t launch_frame(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material,
                         const FrameAux &fx, int grid);

// Launchers (kernels.cu, warmstart.cu)
cudaError_t launch_ref_force(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st);
// Incremental stress: the parity-0 state to its increment over the base
// before the passes, each instance's final state back after them (no-ops
// without incremental stress; kernels.cu)
cudaError_t launch_to_increment(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st);
cudaError_t launch_from_increment(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st);
cudaError_t launch_ws_gref(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material);
cudaError_t launch_ws_predict(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, const float *theta,
                              const float *feat_mean, const float *feat_std, const float *out_std, float *tetF,
                              int sms, int base, int material);
cudaError_t launch_ws_choose(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st);
cudaError_t launch_ws_features(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, float *tetF,
                               const int *pad2user, float *out, float *scale_out);
cudaError_t launch_rest(cudaStream_t s, const DevMesh &m, const double *rest_pad, float density, float4 *row0,
                        float4 *row1, float4 *row2, double *tmass, int *bad);
cudaError_t launch_mass(cudaStream_t s, const DevMesh &m, const double *tmass, const int *state, float gravity,
                        float4 *info);
cudaError_t launch_set_lame(cudaStream_t s, int Tp, const int4 *tets, const float *mu, const float *lambda, int count,
                            float4 *row1, float4 *row2, const int *tet_user);
// Resets the control blocks (both copies), the running count and the
// line-search counters for a step.
cudaError_t launch_init_ctl(cudaStream_t s, int n_inst, const DevParams &p, const DevState &st);
cudaError_t launch_prologue(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, const float *ext_user,
                            const int *pad2user);
// par: the pass's parity, the state buffer (0 or 1) it reads.  A step starts
// at parity 0 and every pass of a running instance flips it, so pass i of a
// step (and of the 16-pass step graph) has parity i & 1.
cudaError_t launch_pass(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material, int par);
// pdl: launch with programmatic stream serialization (the step graph's passes)
cudaError_t launch_tet_only(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material, int par,
                            bool pdl = false);
cudaError_t launch_node_only(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int par,
                             bool pdl = false);
// Takes the pending pass decisions after a run of passes whose next parity is
// par (the copy they are in), leaving them in st.ctl.  A run of passes must
// end with it before anything else reads the control blocks.
// With loop (the body of the step graph's WHILE node): the last CTA to settle
// counts the body run in active[2] and sets the node's condition, so the
// loop goes on while an instance runs and fewer than max_runs bodies ran.
struct LoopCtl {
    cudaGraphConditionalHandle cond;
    int max_runs;
};
cudaError_t launch_settle(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int par,
                          bool pdl = false, const LoopCtl *loop = nullptr);
// RESTART control: replaces an instance's inertial guess by the step's start
// positions when the guess inverts a tet (kernels.cu)
cudaError_t launch_guess_check(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st);
cudaError_t launch_epilogue(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, const int *pad2user);
// positions (user layout) <-> displacement pairs
cudaError_t launch_pack_positions(cudaStream_t s, const DevMesh &m, const float4 *uh, const float4 *ul,
                                  const int *pad2user, float *dst_user);
cudaError_t launch_unpack_positions(cudaStream_t s, const DevMesh &m, const float *src_user, const int *pad2user,
                                    float4 *uh, float4 *ul);
cudaError_t launch_pack(cudaStream_t s, int Np, const float4 *src, const int *pad2user, float *dst_user);
cudaError_t launch_unpack(cudaStream_t s, int Np, const float *src_user, const int *pad2user, float4 *dst);
cudaError_t launch_scatter_positions(cudaStream_t s, const DevMesh &m, int count, const int *ids_pad,
                                     const float *xyz, float4 *uh, float4 *ul);
// n_fp64_svd: when not null, counts the tets whose stretch-based stress took
// the FP64 SVD (det F < 1e-3); ul: the displacements' low words (when not
// null, a near-inverted tet forms its FP64 gradient from the exact pairs)
cudaError_t launch_eval_tets(cudaStream_t s, const DevMesh &m, const float4 *uh, int material, int clamp_cpu,
                             float *tf, float *energy, float *hd, unsigned int *n_fp64_svd = nullptr,
                             const float4 *ul = nullptr);
cudaError_t launch_gather(cudaStream_t s, const DevMesh &m, const float *tf, const float *hd, const int *pad2user,
                          float *force_user, float *hd_user);

// Makes a handle's device current for the rest of an entry point's scope and
// puts the caller's current device back on every return path: a call on a
// handle never changes which device the caller's own CUDA work goes to.
class DeviceScope {
  public:
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev_) != cudaSuccess) {
            cudaGetLastError();
            prev_ = -1;
        }
        if (prev_ == device) {
            prev_ = -1;  // already current: nothing to restore
            ok_ = true;
        } else {
            ok_ = cudaSetDevice(device) == cudaSuccess;
        }
    }
    ~DeviceScope() {
        if (prev_ >= 0) cudaSetDevice(prev_);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
    bool ok() const { return ok_; }

  private:
    int prev_ = -1;
    bool ok_ = false;
};

}  // namespace pbs

// Enters a handle's device for the enclosing entry point (see DeviceScope);
// returns PBS_E_CUDA when the device cannot be made current.
#define PBS_DEVICE_SCOPE(dev)                  \
    ::pbs::DeviceScope pbs_device_scope__(dev); \
    if (!pbs_device_scope__.ok()) return PBS_E_CUDA

struct pbs_handle;

namespace pbs {

// What an entry point outside the handle's own source file reads of it.
// Surface picking and drag forces (surface.cu): faces and rings in padded
// node ids.
int pick_blocks(int n_faces, int sms);
cudaError_t launch_pick_face(cudaStream_t s, const DevMesh &m, const DevState &st, int n_faces, const int4 *faces,
                             float3 orig, float3 dir, int n_blk, float *blk_d2, int *blk_id, int *out);
cudaError_t launch_drag_ring(cudaStream_t s, const DevMesh &m, const DevState &st, const int4 *faces,
                             const int *ring, int begin, int len, float3 drag, float4 *ext);

// Backward-Euler step (implicit.cu): a 3x3 block-CSR matrix over padded
// nodes (columns ascending per block row) and the conjugate-gradient state.
struct BsrView {
    const int *ptr, *col;
    float *val;      // 9 per block, row-major; or 1 per block (a I3) when scalar
    int scalar = 0;
};
struct CgState {
    double rz, rr, bb, alpha, beta;
    int iters, status, done, pad;
};
int cg_blocks(int Np);
cudaError_t launch_be_assemble(cudaStream_t s, const DevMesh &m, const DevState &st, int material, const BsrView &A,
                               float dt, float alpha, float beta, const float4 *ext, float4 *b, float4 *x,
                               float *dinv9);
// pnorm: stop on the preconditioned norm r.D^-1 r <= tol2 b.D^-1 b instead
// of |r|^2 <= tol2 |b|^2 (rows of very different scale, e.g. pinned nodes'
// 1e8 masses)
cudaError_t launch_cg_init(cudaStream_t s, int Np, const BsrView &A, const float *dinv9, const float4 *b,
                           const float4 *x, float4 *r, float4 *z, float4 *p, double *part, CgState *cs, double tol2,
                           int pnorm = 0);
cudaError_t launch_cg_iteration(cudaStream_t s, int Np, const BsrView &A, const float *dinv9, float4 *x, float4 *r,
                                float4 *z, float4 *p, float4 *q, double *part, CgState *cs, double tol2,
                                int max_iters, int pnorm = 0);
cudaError_t launch_be_finish(cudaStream_t s, const DevMesh &m, const DevState &st, const float4 *x, float dt);

// Strain-based PBD schedule: levels of mutually node-disjoint tets in the
// caller's order; group g (an instance) sweeps levels grp[g] .. grp[g+1]-1,
// level l holds tets lvl[l] .. lvl[l+1]-1 of the level-ordered copies.
struct PbdView {
    const int *grp, *lvl;
    const int4 *tet;              // padded node ids
    const float4 *d0, *d1, *d2;   // rows of Dm^-1
    float4 *px;                   // positions; .w = inverse mass
};
// The PBD rest data as the reference forms it in FP32: Dm^-1 rows of the
// level-ordered tets (order[j] = padded tet) and per node {1 / mass (0 when
// pinned), -gravity * mass}; share: scratch of Tp floats.
cudaError_t launch_pbd_rest(cudaStream_t s, const DevMesh &m, const int *order, int n, float density, float gravity,
                            float4 *d0, float4 *d1, float4 *d2, float *share, float2 *node);
cudaError_t launch_pbd_begin(cudaStream_t s, const DevMesh &m, const DevState &st, const float2 *node,
                             const float4 *ext, float dt, float4 *px, float4 *x0);
cudaError_t launch_pbd_sweeps(cudaStream_t s, const PbdView &v, int n_groups, int iterations, const float stretch[3],
                              const float shear[3]);
// The sweeps with an instance's positions in its 16-CTA cluster's
// distributed shared memory: codes = per tet corner (owner CTA << 16 |
// offset), gnode = per group {first padded node, slice, node count};
// pbd_dsmem_fits: whether 16-CTA clusters with smem_bytes a CTA can be
// resident (sets the kernel's attributes).
bool pbd_dsmem_fits(int smem_bytes);
cudaError_t launch_pbd_sweeps_dsmem(cudaStream_t s, const PbdView &v, const int4 *codes, const int4 *gnode,
                                    int n_groups, int smem_bytes, int iterations, const float stretch[3],
                                    const float shear[3]);
cudaError_t launch_dyn_end(cudaStream_t s, const DevMesh &m, const DevState &st, const float4 *px, const float4 *x0,
                           float dt, int divide_first);
cudaError_t launch_pd_assemble(cudaStream_t s, const DevMesh &m, const BsrView &A, float dt_matrix, float stiffness,
                               float *dinv9);
cudaError_t launch_pd_begin(cudaStream_t s, const DevMesh &m, const DevState &st, const float4 *ext, float dt,
                            float4 *q, float4 *px, float4 *x0);
// r = b - A p of the global step at iterate px (and d = 0), from the per-tet
// rotations; slot: scratch of one float4 a gather slot
cudaError_t launch_pd_residual(cudaStream_t s, const DevMesh &m, const float4 *px, float stiffness, float dt,
                               float dt_matrix, float4 *slot, const float4 *q, const float4 *x0, float4 *r, float4 *d);
cudaError_t launch_pd_apply(cudaStream_t s, int Np, float4 *p, const float4 *d);

struct HandleView {
    int device;
    cudaStream_t stream;
    int material;
    DevMesh mesh;
    const int *pad2user;  // padded node -> caller's node index, -1 for padding
};
void handle_view(const pbs_handle *h, HandleView *v);

}  // namespace pbs
