/*
 * phybs.h - C ABI of the GB300-native descent time step.
 *
 * One handle holds one packed set of tet meshes ("instances") resident on
 * the GPU, and advances all of them by one implicit-Euler step per
 * pbs_step() call: the step's energy is minimised by Jacobi-preconditioned
 * descent with Chebyshev acceleration and an energy line search every few
 * iterations.  This is the entry-point set of PhyBS's
 *   CUDAInterface (FVM/CUDAInterface.h:20-102)   and
 *   DescentOptimize (FVM/DescentOptimize.h:11-54)
 * as its step loop (FVM/fvm.cpp:35-47, 172-189, 216-217) drives them:
 * construct from a TetMesh, set the material, step, read positions back.
 *
 * Conventions
 *   - positions / forces: 3*N floats, interleaved xyz (Eigen 3xN column-major,
 *     the layout of TetMesh::getNodes().data()).
 *   - tets: 4*T int32, 0-based node ids, 4 consecutive ids per tet
 *     (TetMesh::getTets().data()).  Tets must be positively oriented.
 *   - every function returns PBS_OK (0) or a negative PBS_E_* code; the
 *     library never exits the process and never prints.
 *   - one handle = one CUDA stream on the current device; a handle is not
 *     thread-safe.  Calls are synchronous unless stated otherwise.  The
 *     handle's stream is non-blocking (it does not wait for the legacy
 *     default stream); every call makes the handle's device current and
 *     restores the caller's current device before it returns.
 *   - there is no CPU path: without a usable GB300 (sm_103) every call that
 *     needs the device fails with PBS_E_CUDA / PBS_E_NO_DEVICE.
 */
#ifndef PHYBS_H
#define PHYBS_H

#ifdef __cplusplus
extern "C" {
#endif

#define PBS_OK 0
#define PBS_E_INVALID_ARG (-1)
#define PBS_E_CUDA (-2)
#define PBS_E_NONFINITE (-3)   /* a step produced NaN/Inf energy or residual   */
#define PBS_E_ITER_CAP (-4)    /* the device-side pass cap ended a step         */
#define PBS_E_BAD_MESH (-5)    /* bad index, zero-volume or inverted rest tet   */
#define PBS_E_NO_DEVICE (-6)   /* no CUDA device, or not compute capability 10.3 */
#define PBS_E_OUT_OF_MEMORY (-7)
#define PBS_E_CAPACITY (-8)    /* a size beyond a documented fixed maximum      */
#define PBS_E_DEVICE_TIMEOUT (-9) /* a kernel's bounded wait on its own copies,
                                     or of the frame engine on a grid barrier,
                                     ran out (the step's results are invalid)   */

/* Pass engines of pbs_step (pbs_set_pass_engine). */
#define PBS_ENGINE_GRAPH 0
#define PBS_ENGINE_FRAME 1

/* Materials.  Both are the neo-Hookean energy
 *   Psi = mu/2 (I1 - 3) - mu ln J + lambda/2 (ln J)^2,
 * evaluated through the invariants (IsotropicNeohookeanMaterial.cpp:104)
 * or through the principal stretches of the modified SVD
 * (IsotropicMaterial.cpp:360-409, Xu et al. 2015). */
#define PBS_MATERIAL_NEOHOOKEAN 0
#define PBS_MATERIAL_STRETCH 1

/* Line-search rejection behaviour. */
#define PBS_CONTROL_REFERENCE 0 /* alpha *= shrink; iterations -= k - 8; redo k (DescentOptimize.cpp:111-122) */
#define PBS_CONTROL_RESTART 1   /* alpha *= shrink; restore x, restart the Chebyshev history and rho schedule;
                                   the iteration budget is unchanged                                          */

/* Energy clamp per tet. */
#define PBS_CLAMP_CPU 0 /* e > 1e-6 ? e : 0   (IsotropicNeohookeanMaterial.cpp:129) */
#define PBS_CLAMP_GPU 1 /* max(e, 0)          (CUDAInterface.cu:549)               */

typedef struct pbs_handle pbs_handle;

/* Mesh description (deep-copied by pbs_create; the caller keeps ownership). */
typedef struct pbs_mesh_desc {
    int n_nodes;
    const float *rest;       /* 3*n_nodes rest positions                          */
    const float *positions;  /* 3*n_nodes initial positions, or NULL for rest     */
    int n_tets;
    const int *tets;         /* 4*n_tets                                          */
    const int *pin_mask;     /* n_nodes, > 0 = pinned (fixed within a step), or NULL */
    int n_instances;         /* >= 1; instances are disjoint node/tet ranges      */
    const int *instance_node_ptr; /* n_instances+1, or NULL when n_instances == 1 */
    const int *instance_tet_ptr;  /* n_instances+1, or NULL when n_instances == 1 */
    float density;           /* kg/m^3, lumped mass = density * vol / 4 per corner */
    float gravity;           /* m/s^2 along -y (the reference uses 9.8)           */
} pbs_mesh_desc;

/* Step parameters.  pbs_default_params() returns the reference preset: the
 * constants of DescentOptimize.cpp:4-22,91-185 and CUDAInterface.cu:911-1006
 * (h = 0.03, 96 iterations, alpha 0.1 / 0.7 / 0.01, line search every 8,
 * Hessian diagonal every 32, rho profile {1:0.96, 7:0.991, 10:0.999},
 * damping 0.99, warm start 0.2, CPU energy clamp, gravity and external
 * forces counted twice in the gradient as DescentOptimize does). */
typedef struct pbs_step_params {
    float h;                  /* time step, s                                   */
    int max_iters;            /* the reference's `iterations`                   */
    float tol;                /* stop when |g| <= tol * |g_0| (FP64 norms); 0 = off */
    int control;              /* PBS_CONTROL_*                                  */
    float alpha0, alpha_min, alpha_shrink;
    int line_search_every;    /* energy check period (8)                        */
    int hessian_every;        /* Jacobi diagonal refresh period (32)            */
    int n_profile;            /* Chebyshev rho profile entries (<= 4)           */
    int profile_k[4];
    float profile_rho[4];
    float damping;            /* v = damping * (x - x0) / h                      */
    float warm_start;         /* x_init = x~ + warm_start * h * (v - v_old)      */
    float body_force_scale;  /* times gravity + external forces enter the gradient:
                                 2 = DescentOptimize.cpp:52 with IsotropicNeohookeanMaterial.cpp:98,
                                 1 = CUDAInterface.cu:600-602 (physical)          */
    int energy_clamp;         /* PBS_CLAMP_*                                     */
    int pass_cap;             /* hard cap on device passes per step; 0 = max_iters + 16 */
    float energy_slack;       /* line-search rounding allowance: reject only if
                                 E > E_old + energy_slack * 2^-24 * sqrt(sum of squared
                                 energy terms); 0 = the reference's strict E > E_old */
    float alpha_grow;         /* RESTART control: alpha <- min(alpha * alpha_grow, alpha0) at
                                 every accepted line-search check, so that one early rejection
                                 does not slow the whole step; 1 = the reference's alpha,
                                 which only shrinks */
    int incremental_stress;   /* neo-Hookean passes: 1 = evaluate P(F) - P(F_base) against
                                 an FP64 force at the step's initial guess (residual
                                 accurate far below 1e-6 of its initial value),
                                 0 = the full FP32 stress each pass (fewer operations) */
} pbs_step_params;

typedef struct pbs_stats {
    int passes;               /* iterations executed, including redone ones (max over instances); the
                                 graph engine also counts a pass that carried the state over
                                 unchanged because a non-finite residual forced an energy check */
    int iterations;           /* accepted iterations k at exit (max over instances) */
    int rejections;           /* line-search rejections (sum over instances)      */
    int converged;            /* instances that met tol                          */
    int status;               /* worst per-instance status (PBS_OK or PBS_E_*)    */
    float alpha;              /* instance 0 */
    float rho, omega;         /* instance 0 Chebyshev state */
    double energy;            /* instance 0 energy at its last check             */
    double residual_ratio;    /* instance 0 |g_k| / |g_0|                         */
    double device_ms;         /* device time of the last pbs_step (CUDA events)   */
    int graph_launches;       /* 16-pass bodies the last step's graph ran */
    int warm_start_used;      /* instances whose step started from the learned guess */
    int guess_fallbacks;      /* RESTART control: instances whose inertial guess inverted a
                                 tet, started from the step's start positions instead */
} pbs_stats;

void pbs_default_params(pbs_step_params *p);
const char *pbs_error_string(int code);

/* CUDAInterface::CUDAInterface (CUDAInterface.cu:641-740): copies the mesh to
 * the device, precomputes Dm^-1, volumes, lumped masses (FP64) and the
 * deterministic node -> (tet, corner) gather, and resets the state.  The
 * material starts as neo-Hookean with E = 5e5, nu = 0.45 (TetMesh.cpp:185)
 * until pbs_set_material is called. */
int pbs_create(const pbs_mesh_desc *desc, pbs_handle **out);
void pbs_destroy(pbs_handle *h);

/* Lame parameters as the reference forms them from (E, nu)
 * (IsotropicNeohookeanMaterial.cpp:15-16, CUDAInterface.cu:704-705):
 * mu = E / (2 (1 + nu)), lambda = 2 mu / (1 - 2 nu) when reference_formula
 * is nonzero, else the textbook lambda = 2 mu nu / (1 - 2 nu). */
void pbs_lame(float young, float poisson, int reference_formula, float *mu, float *lambda);

/* Material model and per-tet (count == n_tets) or uniform (count == 1) Lame
 * parameters (IsotropicMaterial::m_mus / m_lambdas). */
int pbs_set_material(pbs_handle *h, int model, const float *mu, const float *lambda, int count);

int pbs_set_params(pbs_handle *h, const pbs_step_params *p);
int pbs_get_params(pbs_handle *h, pbs_step_params *p);

/* One time step of every instance (CUDAInterface::doDescentOpt,
 * CUDAInterface.cu:911-1007 / DescentOptimize::doDescentOpt).  ext: 3*N
 * external forces for this step (copied in), or NULL for none.  The external
 * forces are cleared after the step, as fvm.cpp:188 does.  iters_out may be
 * NULL.  Returns PBS_E_NONFINITE / PBS_E_ITER_CAP when an instance ended that
 * way (the state is still advanced). */
int pbs_step(pbs_handle *h, const float *ext, int *iters_out);

/* Positions after the last step (the hostNode output of doDescentOpt). */
int pbs_read_positions(pbs_handle *h, float *out);
/* CUDAInterface::updateNodePositions (CUDAInterface.cu:771). */
int pbs_update_positions(pbs_handle *h, const float *positions);
/* Velocities (3*N) and the previous step's velocities, for snapshots. */
int pbs_read_velocities(pbs_handle *h, float *v, float *v_old);
int pbs_write_velocities(pbs_handle *h, const float *v, const float *v_old);
/* Overwrite the positions of `count` nodes (caller numbering; ids: count ints,
 * xyz: 3*count floats) before the next step.  This is how a caller prescribes
 * the motion of pinned nodes: the reference has no such call, its harness
 * writes TetMesh::getNodes() directly (pinned nodes stay where they are put
 * within a step, DescentOptimize.cpp:54-58 / CUDAInterface.cu:578-585). */
int pbs_set_node_positions(pbs_handle *h, int count, const int *ids, const float *xyz);
/* Initial guess for the next pbs_step only (3*N positions, caller order;
 * pinned nodes keep their prescribed positions).  The step treats it as it
 * treats the learned warm start's prediction: the guess is kept only if its
 * energy is not higher than the inertial guess's, and the step still iterates
 * to the same residual bar, measured against the inertial guess's gradient.
 * No counterpart in the reference, whose first iterate is always the
 * inertial guess. */
int pbs_set_guess(pbs_handle *h, const float *positions);
/* CUDAInterface::reset (CUDAInterface.cu:776): rest positions, zero velocities
 * (and an empty displacement history for the learned warm start). */
int pbs_reset(pbs_handle *h);
int pbs_get_stats(pbs_handle *h, pbs_stats *s);
/* The last step's figures of one packed instance (0 .. n_instances-1): its
 * own passes, iterations, rejections, convergence, status and residual ratio
 * (device_ms and graph_launches are the whole step's).  No counterpart in the
 * reference, which steps one mesh. */
int pbs_get_instance_stats(pbs_handle *h, int instance, pbs_stats *s);

/* Mesh sizes and the device-side gather structure, for parity checks.
 * row_ptr: n_nodes+1; entries: 4*n_tets, entry = 4*tet + corner, ordered per
 * node by ascending tet then corner. */
int pbs_get_sizes(pbs_handle *h, int *n_nodes, int *n_tets, int *n_instances);
int pbs_get_incidence(pbs_handle *h, int *row_ptr, int *entries);
/* Rest data as the device holds it: Dm^-1 row-major (9T), signed volume det/6
 * (T), lumped mass with pins = 1e8 (N), gravity_y = -g * lumped mass (N). */
int pbs_get_rest_data(pbs_handle *h, float *dm_inv9, float *signed_vol, float *mass, float *grav_y);

/* Evaluate the per-tet kernel at the given positions (NULL = current):
 * corner forces (12*T, corner-major xyz; the reference's P * AN columns and
 * their negated sum), clamped energy (T) and the 12 Jacobi-diagonal entries
 * (12*T).  Any output may be NULL. */
int pbs_eval_tets(pbs_handle *h, const float *positions, float *corner_forces, float *energy, float *hess_diag);
/* Parity probe: how many tets of the last pbs_eval_tets call had their stress
 * evaluated in FP64 from the exact displacements: near-inverted tets, det F <
 * 1e-3 (for the stretch-based material also any tet whose smallest singular
 * value is below 0.3: the FP64 SVD of the near-inverted tets the reference's
 * modified SVD, IsotropicMaterial.cpp:16-60, resolves). */
int pbs_eval_fp64_svd_count(pbs_handle *h, int *count);
/* Parity probe of the incremental stress's per-step base force: the elastic
 * node forces (3*N doubles, free nodes; pinned nodes get 0) at `positions`,
 * from the kernels pbs_step runs once a step at its initial guess (each tet's
 * neo-Hookean stress in double-float arithmetic, corner forces summed per
 * node in FP64 in incidence order), on the displacements' FP32 hi words as
 * the step's base uses them.  The per-node elastic force of
 * IsotropicNeohookeanMaterial::computeInnerForceFromPos
 * (IsotropicNeohookeanMaterial.cpp:93-114) without its gravity, external and
 * pin-spring terms, to about 1e-12 relative.  Neo-Hookean handles only
 * (PBS_E_INVALID_ARG otherwise). */
int pbs_eval_base_force(pbs_handle *h, const float *positions, double *forces);
/* Elastic forces (3*N) and Hessian diagonal (3*N) assembled by the
 * deterministic gather at the given positions (NULL = current). */
int pbs_eval_nodes(pbs_handle *h, const float *positions, float *forces, float *hess_diag);

/* Elastic forces (3*N, the caller's node order) at the given positions (3*N),
 * as pbs_eval_nodes computes them, for callers that cannot allocate device
 * memory in the call: a frame loop that must not stall (cudaMalloc and
 * cudaFree synchronise the whole device) or a host that keeps all device
 * memory in its own pool.  No counterpart in the reference.
 *   - positions and forces are DEVICE pointers on the handle's device; the
 *     two kernels are enqueued on the handle's stream (pbs_get_stream) and
 *     the call returns without waiting for them.  That stream is created
 *     non-blocking: it does not wait for the legacy default stream or any
 *     other stream of the caller.  Order the work that writes `positions`
 *     before the call, and the work that reads `forces` after it, against
 *     pbs_get_stream's stream (enqueue it there, or use events).
 *   - positions are not checked for finiteness (they stay on the device):
 *     a non-finite position gives non-finite forces, where pbs_eval_nodes
 *     would return PBS_E_INVALID_ARG.
 *   - allocates nothing: the per-tet corner-force scratch is one fixed
 *     24 MiB array in the library's device image, which bounds the mesh to
 *     PBS_EVAL_STATIC_MAX_TETS tets after padding (each instance's tet count
 *     rounded up to 256); larger handles fail with PBS_E_CAPACITY, host
 *     pointers with PBS_E_INVALID_ARG.
 *   - the first call on a device looks up that array's address (with the
 *     device current) and keeps it; make this first call before any stream
 *     capture.  After a cudaDeviceReset the next call looks it up again
 *     (make that one before any capture too).
 *   - every call on a device shares the array: calls whose kernels overlap
 *     on the GPU (different streams with no ordering between them) race and
 *     corrupt each other's forces.  Nothing in it needs to start at zero.
 *   - the caller's current device is left as it was. */
#define PBS_EVAL_STATIC_MAX_TETS 524288
int pbs_eval_nodes_static(pbs_handle *h, const float *positions, float *forces);

/* The CUDA stream (cudaStream_t) every call of this handle launches on, so a
 * caller can order its own work or record timing events on it. */
int pbs_get_stream(pbs_handle *h, void **stream);
/* Time the two kernels of one descent pass separately with CUDA events on the
 * handle's stream: runs `passes` passes from the current state (the state is
 * left as it was) and returns the mean milliseconds per launch of the per-tet
 * kernel and of the per-node kernel.  Fails when an instance stopped before
 * the last pass (its launches would time no work): with its status
 * (PBS_E_NONFINITE), or PBS_E_ITER_CAP when it stopped for another reason;
 * pbs_get_stats then describes that instance. */
int pbs_profile_kernels(pbs_handle *h, int passes, double *tet_ms, double *node_ms);

/* Chunk shape of the per-tet pass kernel picked by pbs_autotune. */
typedef struct pbs_tune_result {
    int chunk_threads;       /* threads per CTA                                   */
    int chunk_tets;          /* tets per chunk at most                            */
    int chunk_nodes;         /* nodes a chunk may touch at most                   */
    int chunk_staged;        /* 1: the chunk's per-tet rows are staged in shared
                                memory by asynchronous copies; 2: persistent CTAs
                                walk the chunks through two staging buffers fed by
                                bulk (TMA) copies (neo-Hookean only)              */
    int node_npt;            /* nodes per thread of the node kernel (1 or 2)      */
    int n_tried;             /* shapes timed                                      */
    double pass_ms;          /* per-tet + per-node kernel time of one pass, kept shape */
    double default_pass_ms;  /* the same for the default shape (256, 1024, 448)   */
} pbs_tune_result;
/* Autotuner of the pass kernels' block and tile shapes: rebuilds the pass
 * layout for each candidate chunk shape (threads per CTA, tets per chunk,
 * nodes per chunk, staging: rows read in the loop, staged in shared memory, or
 * the persistent double-buffered kernel), times
 * `passes` passes of it from the current state (then the node kernel with 1
 * and 2 nodes per thread) with
 * CUDA events and keeps the fastest.  Forces stay deterministic for a given
 * shape; another shape changes the order the corner forces are summed in, so
 * results can differ in the last bits.  Call between steps (it recaptures the
 * step graph).  No counterpart in the reference, whose launch shapes are
 * fixed. */
int pbs_autotune(pbs_handle *h, int passes, pbs_tune_result *out);
/* Sets a chunk shape directly (for instance one pbs_autotune picked on another
 * handle of the same mesh): threads per CTA 128, 256 or 512; tets per chunk
 * 1 .. 16384; nodes per chunk >= 4; staged 0, 1 or 2 (not with 512 threads;
 * used by neo-Hookean handles only); the shared memory it needs at most
 * 200 KB; node_npt 1 or 2 nodes per thread of the node kernel.  Call between
 * steps. */
int pbs_set_chunk_shape(pbs_handle *h, int threads, int chunk_tets, int chunk_nodes, int staged, int node_npt);
/* Pass engine of pbs_step.  PBS_ENGINE_GRAPH (the default): each pass is a
 * per-tet and a per-node kernel, 16 passes to a captured CUDA graph, and the
 * host reads the count of running instances between graphs.
 * PBS_ENGINE_FRAME: one cooperative launch runs all the passes of a step; its
 * CTAs stay resident for the whole step, grid barriers separate the tet and
 * node phases of a pass, and every CTA takes the line-search and stop
 * decisions from the same sums.  For one-instance handles whose chunk shape
 * is unstaged (staged 0) with 128 or 256 threads; PBS_E_INVALID_ARG
 * otherwise, and from pbs_step when a later shape or parameter change leaves
 * the handle outside that set.  The instance's energy and residual sums are
 * grouped per CTA instead of per chunk, so results agree with the graph
 * engine's to rounding; they are bit-reproducible run to run.  A barrier wait
 * that runs out (0.5 s) ends the step with PBS_E_DEVICE_TIMEOUT.
 * pbs_stats.graph_launches is 0 for a frame-engine step.  No counterpart in
 * the reference, which launches each kernel from the host. */
int pbs_set_pass_engine(pbs_handle *h, int engine);
/* L2 residency of the per-tet pass data (the tets' Dm^-1 rows and corner
 * records, 64 B a tet, read by every pass).  pbs_create takes the persisting-L2
 * set-aside of the calling process's CUDA context (at most that data's size,
 * at most what the device allows) and the per-tet kernels then launch with an
 * L2 access-policy window over that data (persisting hits, streaming misses);
 * pbs_destroy resets the persisting lines and sets the set-aside back to 0,
 * for the whole context.  enable = 0 launches without the window (for a
 * caller that shares L2 with other work, or to compare), 1 with it (the
 * default); PBS_E_INVALID_ARG when the device has no persisting L2.  Results
 * do not depend on it.  No counterpart in the reference. */
int pbs_set_l2_residency(pbs_handle *h, int enable);
int pbs_get_pass_engine(pbs_handle *h, int *engine);
/* pbs_profile_kernels for the frame engine: one frame launch of `passes`
 * passes from the current state (left as it was), timed with CUDA events;
 * returns the mean milliseconds per pass.  Fails as pbs_profile_kernels does,
 * and with PBS_E_INVALID_ARG where the frame engine does not apply. */
int pbs_profile_frame(pbs_handle *h, int passes, double *pass_ms);

/* ------------------------------------------------------------------------
 * Learned warm start.  A per-node MLP 24 -> 64 -> 64 -> 64 -> 3 (GELU; BF16
 * weights on the tensor cores, FP32 accumulation; 10,115 FP32 master
 * parameters: W1 64x24, b1, W2 64x64, b2, W3 64x64, b3, W4 3x64, b4, weights
 * row-major with one row per output).  It has no counterpart in the
 * reference: it predicts each step's correction to the inertial guess.
 * ------------------------------------------------------------------------ */
typedef struct pbs_mlp pbs_mlp;
int pbs_mlp_param_count(void);
/* theta: NPARAM initial values, or NULL for He initialisation from `seed`. */
int pbs_mlp_create(pbs_mlp **out, const float *theta, unsigned long long seed);
void pbs_mlp_destroy(pbs_mlp *t);
int pbs_mlp_get_params(pbs_mlp *t, float *theta);
int pbs_mlp_set_params(pbs_mlp *t, const float *theta);   /* also resets Adam */
/* Host arrays: X n x 24, Y n x 3. */
int pbs_mlp_forward(pbs_mlp *t, const float *X, int n, float *Y);
/* Gradient of the mean (over rows) squared error of the batch; grad NPARAM floats. */
int pbs_mlp_gradient(pbs_mlp *t, const float *X, const float *Y, int n, float *grad, float *loss);
/* Training set (copied to the device): X n x 24, Y n x 3, W n non-negative
 * sample weights or NULL (all 1; the loss is then the mean squared error,
 * otherwise sum_i W_i |y_i - Y_i|^2 / n over the minibatch).  Adam training
 * on minibatches. */
int pbs_mlp_set_data(pbs_mlp *t, const float *X, const float *Y, const float *W, int n);
int pbs_mlp_train(pbs_mlp *t, int steps, int batch, float lr, unsigned long long seed, float *losses);

/* Install (enabled = 1 or 2) or switch off (0) the warm start on a solver
 * handle.  theta: pbs_mlp_param_count() values; feat_mean / feat_std: the 24
 * feature standardisation constants; out_std: the 3 output scales (the
 * network predicts correction / (out_std * s), s the node's motion scale, see
 * pbs_warm_start_features).  The correction is added to the plain guess
 * (enabled = 1) or to the constant-acceleration extrapolation of the node's
 * last two displacements, u0 + 2 d1 - d2 (enabled = 2).  Each pbs_step then
 * evaluates the network on the plain guess's features, keeps the predicted
 * guess for an instance only if its energy is not higher than the plain
 * guess's, and measures the residual tolerance against the plain guess's
 * gradient either way. */
int pbs_set_warm_start(pbs_handle *h, const float *theta, const float *feat_mean, const float *feat_std,
                       const float *out_std, int enabled);
/* The 24 raw (unstandardised) features of every node for the next step with
 * external forces ext (or NULL), the plain initial guess x~ + warm_start
 * h (v - v_old) (x_init, 3*N, may be NULL) and each node's motion scale
 * s = (1 - damping) |d1| + |d1 - d2| + 1e-4 l (scale, N, may be NULL; d1, d2
 * the node's last two displacements, l the instance's mean edge length: the
 * plain guess's error under constant acceleration), which divides the length
 * features.  The state is not advanced. */
int pbs_warm_start_features(pbs_handle *h, const float *ext, float *features, float *x_init, float *scale);

/* Node-node 3N x 3N stiffness pattern of the mesh, bit-identical to
 * IsotropicMaterial::allocateGlobalStiffnessMatrix (IsotropicMaterial.cpp:554-644):
 * CSR row pointers (3N+1), column indices (nnz), the CSR slot of each diagonal
 * entry (3N) and the 48 slots per tet (kIDinCSRval).  Call with col == NULL to
 * get nnz only.  Host-side; needs no device. */
int pbs_stiffness_pattern(int n_nodes, int n_tets, const int *tets, int *nnz, int *row_ptr, int *col,
                          int *diag_idx, int *kid48);

/* ---- Linearly implicit (backward) Euler step ----
 * The reference's second GPU integrator, CUDAInterface::computeInnerforces +
 * computeGlobalStiffnessMatrix + doBackEuler (CUDAInterface.cu:784-884, driven
 * by fvm.cpp:179-183):
 *   (M (1 + alpha dt) + dt (dt + beta) K(x)) v' = M v + dt f(x),  x' = x + dt v'
 * f = elastic + gravity (+ ext, 3*N floats or NULL); a pinned node's force is
 * the spring 1e8 (X - x) and its mass 1e8; K = -df/dx (the neo-Hookean
 * Hessian, which the stretch-based material shares).  The reference uses
 * dt = 0.03, alpha = beta = 0.02.  K is assembled per 3x3 block row in a
 * fixed order (no atomics) and the system solved by block-Jacobi
 * preconditioned conjugate gradients from v, FP64 dot products, until
 * |r| <= tol |b| (the reference: a cuSOLVER sparse Cholesky).  Returns
 * PBS_E_ITER_CAP (state advanced with the last iterate) when max_iters did
 * not reach tol, PBS_E_NONFINITE (state unchanged) on a non-finite residual;
 * iters_out / residual_out (|r| / |b|) may be NULL.  Shares positions and
 * velocities with pbs_step. */
int pbs_backward_euler_step(pbs_handle *h, float dt, float alpha, float beta, const float *ext, float tol,
                            int max_iters, int *iters_out, double *residual_out);

/* ---- Surface picking and drag forces (the viewer's interactive load) ----
 * The reference's viewer picks a boundary face with a ray and drags it; the
 * drag becomes the external forces of the next steps (RenderWidget.cpp:154,194
 * -> TetMesh::pickFacebyRay / dragFaceRing, passed to doDescentOpt by
 * fvm.cpp:187-188).  These calls compute the same on the device from the
 * handle's current positions, bit-identical to the reference's FP32. */

/* Boundary triangles (3 * n_faces caller node ids, e.g. a tetgen .face file's,
 * in the file's orientation) replacing TetMesh::initFacesFromFile
 * (TetMesh.cpp:130-151).  Builds each face's ring as
 * TetMesh::computeBoundfaceRingIndices does (TetMesh.cpp:229-277): the face's
 * three nodes, then every other node that shares a surface edge with one of
 * them, ascending.  n_faces = 0 clears the surface. */
int pbs_set_surface(pbs_handle *h, const int *faces, int n_faces);
/* The ring of one face: its length in *size and up to `capacity` caller node
 * ids in ring (ring may be NULL to query the length). */
int pbs_get_face_ring(pbs_handle *h, int face, int *ring, int capacity, int *size);
/* TetMesh::pickFacebyRay (TetMesh.cpp:395-418) with the normals and centres of
 * computeBoundfaceNormals (TetMesh.cpp:378-393) at the current positions:
 * among the faces whose normal (x2 - x0) x (x1 - x0) opposes dir, the first
 * whose centre lies nearest the ray (orig, dir), within the length of face 0's
 * first edge; *face = -1 when none does.  orig and dir: 3 floats each. */
int pbs_pick_face(pbs_handle *h, const float *orig, const float *dir, int *face);
/* TetMesh::dragFaceRing (TetMesh.cpp:443-470): the external forces of a drag
 * of `face` along drag (3 floats) at the current positions, written to ext
 * (3 * N floats, caller order; zero off the ring) for the next pbs_step:
 * factor = min(|drag| / r * 100, 800) with r face 0's first edge, factor * m
 * * drag / |drag| on the face's nodes and half of it on the rest of the ring
 * (m: lumped mass, 1e8 for a pinned node). */
int pbs_drag_face_ring(pbs_handle *h, int face, const float *drag, float *ext);

/* ---- Strain-based position-based dynamics and projective dynamics ----
 * The reference's two CPU integrators besides the descent, selected in
 * fvm.cpp:162-171.  Both share positions and velocities with pbs_step; a step
 * starts from the FP32 positions pbs_read_positions returns and stores the
 * new ones exactly (up to the compensated split of the state). */

/* PosBaseDynamic::doStepStrainConstraints (PosBaseDynamic.cpp:12-53) with
 * solveStrainConstraints (:55-117), strain-based dynamics of Mueller et al.
 * 2014:
 *   p = x + dt (v + dt w f),  f = gravity + ext (3*N floats or NULL),
 *   w = 1 / mass (0 at a pinned node);
 *   `iterations` Gauss-Seidel sweeps over the tets in their caller order, each
 *   tet projecting its six Green-strain constraints S_ij = f_i . f_j
 *   (f_i = P Dm^-1 e_i, P the deformed edge matrix) onto S_ii = 1 (weight
 *   stretch[i]) and S_ij = 0 (weight shear[i + j - 1]); a constraint whose
 *   w-weighted gradient norm is below 1e-6 is skipped;
 *   v = (p - x) 0.99 / dt,  x = p.
 * The reference uses 5 sweeps, stretch = (1, 1, 1), shear = (0.8, 0.8, 0.8)
 * (NULL selects these) and the viewer's time step.  The sweeps run on the
 * device in the caller's tet order exactly: tets are grouped by dependency
 * level (a tet's level is one more than that of the last earlier tet sharing
 * a node), so a level's tets share no node and each sees precisely the
 * updates of the tets before it.  The arithmetic is FP32 without contraction
 * in the reference's operation order (the stretch multiplier in FP64, as the
 * reference's double literal makes it), so a step equals the serial CPU
 * sweep's bit for bit on the same rest data. */
int pbs_pbd_step(pbs_handle *h, float dt, int iterations, const float *stretch, const float *shear,
                 const float *ext);

/* ProjDynamic::doProjDynamics (ProjDynamic.cpp:442-480) with its solver
 * matrix (buildGlobalSolverMatrix, :48-100) and local projections
 * (projectLocalConstraints2 on 4 threads, :351-434):
 *   s = (x + dt v + dt^2 w f) m / dt^2   (f = gravity + ext, m the lumped
 *        mass, 1e8 at a pinned node, w = 1 / m, 0 at a pinned node);
 *   `iterations` times: R_t = U V^T of the SVD of each tet's F at the current
 *   iterate p (JacobiSVD with det U, det V fixed by flipping the first,
 *   largest-singular-value column: an inverted tet's R flips that direction),
 *   b = s + sum_t k vol_t A_t^T R_t, and p = A^-1 b with
 *   A = M / dt_m^2 + sum_t k vol_t A_t^T A_t (A_t maps corner positions to F);
 *   v = (p - x) / dt 0.99,  x = p.
 * The reference: k = 1e6, 5 iterations, dt = 0.03 for the right-hand side and
 * the integrator's time step for A (dt_matrix; 0 takes dt), and an MKL
 * Pardiso LDL^T factorisation of A.  Here A is assembled once per (dt_matrix,
 * k) as block rows and each global step solves for the correction d of the
 * current iterate p: r = b - A p formed per tet from edge differences
 * (M / dt^2 (x - p + dt v + dt^2 w f) + sum_t k vol_t A_t^T vec(R_t - F_t):
 * no absolute coordinate enters), A d = r by block-Jacobi
 * preconditioned conjugate gradients until (e^T D^-1 e)^1/2 <= tol
 * (r^T D^-1 r)^1/2 for the CG residual e, or max_cg iterations
 * (PBS_E_ITER_CAP, the state advanced), then p += d.  cg_iters_out: total CG
 * iterations of the step (may be NULL). */
int pbs_pd_step(pbs_handle *h, float dt, float dt_matrix, float stiffness, int iterations, const float *ext,
                float tol, int max_cg, int *cg_iters_out);

#ifdef __cplusplus
}
#endif
#endif /* PHYBS_H */
