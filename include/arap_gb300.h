/*
 * arap_gb300.h -- C ABI of the GB300 (sm_103a) embedded-deformation / ARAP
 * hot path: kNN skinning weights, node graph, Gauss-Newton solve over node
 * transforms, and skinning of Gaussians and density-grid samples.
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer owned by the caller unless the
 *     parameter name ends in "_host".  Nothing is retained after a call except
 *     inside an explicit handle (arap_solver, arap_solver_batch, arap_grid,
 *     arap_skin_plan).  The library keeps no global state: two handles used
 *     from two streams or threads never share a word.
 *   - Every call takes the cudaStream_t it enqueues on (0 = legacy default).
 *     Calls return after enqueueing; results are ready once the stream is.
 *   - Every call returns an int status (ARAP_OK = 0).  Errors raised on the
 *     device (non-finite values, timed-out barrier waits) go to a device
 *     status word: each handle owns one (read and cleared by
 *     arap_solver_status / arap_grid_status / arap_skin_plan_status, and by
 *     the calls that synchronise, such as arap_solver_solve with stats); the
 *     stateless calls that can raise one take an `int32_t* status` device
 *     word of the caller's (NULL: not recorded), read with arap_status_read.
 *     The first code raised wins until the word is read.
 *   - Points are float32 xyz triples; quaternions are (w, x, y, z) float32;
 *     node rotations are column-major 3x3 ("[0 3 6; 1 4 7; 2 5 8]"), exactly
 *     DeformGraph::rot (Deform.hpp:29-38).
 *   - "planes" layout: a per-item array with C components is stored as C
 *     contiguous planes of length P (component c of item i at [c*P + i]).
 */
#ifndef ARAP_GB300_H
#define ARAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* arap_stream_t; /* == cudaStream_t */

enum {
  ARAP_OK = 0,
  ARAP_NOT_CONVERGED = 1, /* iteration cap hit with early exit enabled (Deform.cpp:112-115 prints only) */
  ARAP_ENONFINITE = 2,    /* NaN/Inf produced (e.g. zero kNN radius, singular block) */
  ARAP_EBADINPUT = 3,     /* invalid sizes / indices / null pointers */
  ARAP_ETIMEOUT = 4,      /* a bounded device-side wait gave up */
  ARAP_ECUDA = 5,         /* a CUDA runtime call failed */
  ARAP_ENOMEM = 6,        /* an allocation failed: device memory inside a handle, or the PLY
                             loader's host buffer */
  ARAP_EUNSUPPORTED = 7   /* parameter outside the compiled range (e.g. k > 12) */
};

#define ARAP_KNN_MAX 12 /* KNN_MAX, helper.hpp:48 */

/* ----------------------------------------------------------------- kNN --- */

/* Node graph: for every node its k nearest OTHER nodes, ascending distance.
 * Replaces DeformGraph::setupEdges / findNearestNodes (Deform.hpp:84-95,
 * 153-185).  nodes_xyz [n*3]; neighbors_out [n*k] row-major (node-major).
 * Requires 1 <= k <= ARAP_KNN_MAX and n >= k+1. */
int arap_build_graph(const float* nodes_xyz, int n, int k, int32_t* neighbors_out,
                     arap_stream_t stream);

/* Skinning weights of P points against n nodes: the k nearest nodes and
 * w_j = (1 - d_j/d_{k+1})^2 / sum (Deform.hpp:187-208, used by
 * GaussianView::setupWeights* GaussianView.cpp:2818-2918).
 * points_xyz [P*3]; idx_out, w_out in planes layout [k][P] (entry j of point i
 * at [j*P + i]).  Distances are compared as float32 sqrt((dx*dx+dy*dy)+dz*dz);
 * exact ties go to the lower node index.  A point whose k+1 nearest nodes are
 * all at the same distance gets NaN weights (the reference's 0/0) and
 * ARAP_ENONFINITE in *status (device word, optional). */
int arap_compute_weights(const float* points_xyz, int P, const float* nodes_xyz, int n,
                         int k, int32_t* idx_out, float* w_out, int32_t* status,
                         arap_stream_t stream);
/* arap_compute_weights with the CTA size of its kernel chosen by the caller
 * (threads: 128, 256 or 512; 0 = 256), e.g. from arap_knn_autotune.  The
 * results do not depend on it. */
int arap_compute_weights_ex(const float* points_xyz, int P, const float* nodes_xyz, int n, int k,
                            int threads, int32_t* idx_out, float* w_out, int32_t* status,
                            arap_stream_t stream);
/* Autotuner of the kNN kernel: times the 128-, 256- and 512-thread CTAs on the
 * first min(P, 262144) points against the n nodes (each run once to warm up,
 * then timed with CUDA events on the stream) and returns the fastest in
 * *threads_out; ms_out [3] (optional) receives the three times.  Synchronises;
 * allocates and frees its own scratch outputs. */
int arap_knn_autotune(const float* points_xyz, int P, const float* nodes_xyz, int n, int k,
                      int* threads_out, float* ms_out, arap_stream_t stream);

/* --------------------------------------------------------------- solver --- */

/* PLAIN: FP32 residual, gradient and PCG, block-Jacobi preconditioning unless
   coarse_nodes is set.  MIXED: the iterate and grid-wide sums in FP64, the
   per-node residual, gradient and energy terms in float-float (about 48
   significant bits from FP32 operations), the PCG in FP32 with float-float
   sums, FP64 polar factors for near-degenerate Gaussians. */
enum { ARAP_PRECISION_PLAIN = 0, ARAP_PRECISION_MIXED = 1 };

typedef struct {
  float w_rot;            /* DeformGraph::w_rot (default 1),  Deform.hpp:56 */
  float w_reg;            /* DeformGraph::w_reg (default 10), Deform.hpp:57 */
  float w_con;            /* DeformGraph::w_con (default 100),Deform.hpp:58 */
  float weighting_factor; /* GaussianView::_weighting_factor (default 1) */
  int cons_on_center;     /* _constraints_on_center: one residual per block centre */
  int max_iters;          /* Gauss-Newton iterations (reference MAX_ITERS = 30) */
  int early_exit;         /* stop when |h| < (|x|+1e-6)*1e-6 (Deform.cpp:165) */
  int precision;          /* ARAP_PRECISION_PLAIN or ARAP_PRECISION_MIXED */
  float pcg_tol;          /* relative residual target of the inner PCG (<=0: default) */
  int pcg_max_iters;      /* inner PCG iteration cap (<=0: default) */
  int coarse_nodes;       /* two-level PCG: target free nodes per aggregate of the coarse
                             (per-aggregate affine) space; 0 = block-Jacobi only.  The
                             target is raised (by a quarter at a time) until there are
                             at most 80 aggregates (960 coarse unknowns). */
  int spin_limit;         /* polls of one grid-barrier wait inside the persistent solve
                             before it gives up with ARAP_ETIMEOUT (<=0: 2^23, about
                             a second); every CTA then leaves the kernel.  A solver
                             with a limit of its own runs on the batched-solve kernel
                             as a batch of one (the same results, a little slower) */
  float coarse_reuse;     /* two-level PCG: a Gauss-Newton iteration keeps the previous
                             iteration's coarse inverse when the last accepted step was
                             below this fraction of |x| and the last PCG took at most 1.5
                             times the iterations of the last one with a fresh inverse.
                             It changes the preconditioner only: every PCG still meets
                             pcg_tol.  0: the default, 0.05; < 0: invert every
                             iteration */
} arap_solve_config;

typedef struct {
  int status;             /* ARAP_* of the last solve */
  int gn_iterations;      /* Gauss-Newton iterations executed */
  int pcg_iterations;     /* total inner PCG iterations */
  int halvings;           /* total line-search step halvings */
  double initial_energy;  /* f.f at x = identity */
  double final_energy;    /* f.f at the returned x */
  int n_free, n_static, n_rows;
  int n_coarse;           /* coarse unknowns of the two-level preconditioner (0 = off) */
  double phase_ms[9];     /* device time in: [0] set-up, [1] gradient/preconditioner,
                             [2] coarse matrix build + inversion, [3] PCG, [4] line search
                             (CTA 0's view); [5] of which the coarse inversion; the
                             slowest CTA's own work (barrier waits excluded) inside
                             PCG: [6] products (J^T J) p, [7] vector update and
                             preconditioner, [8] coarse solves */
  int resident;           /* 1: every CTA's nodes and PCG vectors fit in its shared
                             memory (the resident two-level PCG with the V-cycle);
                             0: the non-resident PCG with the additive preconditioner */
  int coarse_fallbacks;   /* Gauss-Newton iterations whose coarse matrix had a pivot that
                             was not positive in float32 (nearly collinear nodes in an
                             aggregate): their PCG ran with block-Jacobi alone, which is
                             slower but still solves the same system */
  int iteration_halvings[64]; /* line-search step halvings of each of the first 64
                             Gauss-Newton iterations (Deform.cpp:144-156; 0 past
                             gn_iterations) */
  int coarse_inversions;  /* Gauss-Newton iterations that formed and inverted the coarse
                             matrix (the others kept the previous inverse, coarse_reuse) */
} arap_solve_stats;

typedef struct arap_solver arap_solver;

/* Fill *cfg with the reference's defaults (Deform.hpp:54-58,
 * GaussianView.hpp:429,459; MAX_ITERS Deform.cpp:3). */
void arap_solve_config_default(arap_solve_config* cfg);

/* Build a solve plan for one control-region configuration.  Replaces the
 * bookkeeping of the Deform constructor (Deform.hpp:414-455: row counts,
 * free/static sets from UpdateIndicies GaussianView.cpp:2010-2035,
 * BelongsToSameBlock Deform.cpp:20-32, SelectKeyControls Deform.cpp:34-75).
 *   neighbors   [n*k]  device, from arap_build_graph
 *   anchor_idx  [k][n] device planes: kNN of each node's own vertex
 *   anchor_w    [k][n] device planes  (cand_vertices[nodes[i].Vertex_index])
 *   block_offsets_host [n_blocks+1], block_nodes_host [...]: node ids of each
 *       block in block order (DeformGraph::indices_blocks)
 *   block_type_host [n_blocks]: 1 active, 0 pinned, -1 excluded (blocks_type)
 * The plan owns its device buffers; free with arap_solver_destroy. */
int arap_solver_create(arap_solver** out, int n, int k, const int32_t* neighbors,
                       const int32_t* anchor_idx, const float* anchor_w,
                       const int32_t* block_offsets_host, const int32_t* block_nodes_host,
                       const int32_t* block_type_host, int n_blocks,
                       const arap_solve_config* cfg, arap_stream_t stream);

/* One deformation solve (Deform::real_time_deform, Deform.cpp:77-169, then
 * DeformGraph::putFreeInputs Deform.hpp:140-151).
 *   node_pos [n*3]  current node positions (DeformGraph::nodes[i].Position)
 *   aims     [n*3]  control targets (GaussianView::aim_positions)
 *   rot_out  [n*9]  column-major R per node (identity for static nodes)
 *   trans_out[n*3]  t per node (zero for static nodes)
 *   stats_host      optional; when non-null the call synchronises the stream
 *                   and fills it. */
int arap_solver_solve(arap_solver* s, const float* node_pos, const float* aims,
                      float* rot_out, float* trans_out, arap_solve_stats* stats_host,
                      arap_stream_t stream);

/* Gradient of 0.5*|f(x)|^2 as the reference's Jacobian states it (J^T f,
 * Deform.cpp:120-122) at x [F*12] (free-node order, [R col-major | t]).
 * grad_out [F*12]; energy_host (optional, synchronises) = f.f. */
int arap_solver_energy_grad(arap_solver* s, const float* node_pos, const float* aims,
                            const double* x, double* grad_out, double* energy_host,
                            arap_stream_t stream);

/* Read and clear the solver's device status word (synchronises the stream):
 * ARAP_OK, or the first device-side error of its launches since the last
 * read (ARAP_ETIMEOUT, ARAP_ENONFINITE, ARAP_EUNSUPPORTED). */
int arap_solver_status(arap_solver* s, arap_stream_t stream);

/* Number of free nodes (columns/12) and the free node ids ascending. */
int arap_solver_free_count(const arap_solver* s);
int arap_solver_free_ids(const arap_solver* s, int32_t* free_ids_host);

void arap_solver_destroy(arap_solver* s);

/* No counterpart in the reference, whose viewer deforms one field at a time:
 * several independent solves in a few cooperative persistent launches (waves).
 * - Instances whose nodes fit in shared memory on some share of the grid (the
 *   resident two-level PCG) are packed into waves by that minimum share,
 *   largest first; the other instances share one wave. In each wave the
 *   co-resident grid (one CTA per SM) is split among its instances: each gets
 *   its minimum (at least one CTA), the rest go in proportion to (coupling
 *   items + free nodes)^balance_exponent (<= 0: 1).
 * - Each instance runs the same Gauss-Newton/PCG iteration as
 *   arap_solver_solve on its own CTAs, with its own grid barrier and its own
 *   solver's buffers. Results equal separate solves to rounding (reduction
 *   order).
 * - All solvers must share one precision, and count may not exceed the grid
 *   (ARAP_EUNSUPPORTED).
 * - A solver may belong to several batches but must not run in two launches
 *   at once. */
typedef struct arap_solver_batch arap_solver_batch;
int arap_solver_batch_create(arap_solver_batch** out, arap_solver* const* solvers, int count,
                             float balance_exponent, arap_stream_t stream);
/* node_pos, aims, rot_out, trans_out: host arrays of count device pointers,
 * with the meaning of arap_solver_solve's arguments. stats_host: NULL (no
 * synchronisation) or count entries (synchronises).
 * Without stats the call queues two copies (a pinned upload of the instances'
 * parameters, a barrier reset) and one cooperative launch per wave, all on `stream`.
 * It can therefore be captured in a CUDA graph. A replay reads the parameter
 * staging as left by the most recent call on this batch. */
int arap_solver_batch_solve(arap_solver_batch* batch, const float* const* node_pos, const float* const* aims,
                            float* const* rot_out, float* const* trans_out, arap_solve_stats* stats_host,
                            arap_stream_t stream);
/* Autotuner of the CTA split: times one batch solve for each balance exponent
 * in {0.75, 1, 1.25, 1.5, 2} (after an untimed one) and keeps the fastest.
 * Outputs are written by the trial solves. Synchronises. */
int arap_solver_batch_autotune(arap_solver_batch* batch, const float* const* node_pos, const float* const* aims,
                               float* const* rot_out, float* const* trans_out, float* best_exponent,
                               arap_stream_t stream);
/* cta_first_host [count+1]: prefix sums of the CTAs each instance gets in its
 * wave (instance i runs on cta_first[i+1] - cta_first[i] CTAs). */
int arap_solver_batch_ctas(const arap_solver_batch* batch, int32_t* cta_first_host);
void arap_solver_batch_destroy(arap_solver_batch* batch);

/* ------------------------------------------------------------ skinning --- */

/* Per-node transform table used by every skinning call: for node j
 * [R - I row-major 9 | g 3 | t 3 | 0] (16 floats).  Built from the solve
 * output and the node positions the solve used.  Blends evaluate
 * p' = p + [(sum w - 1) p + sum w ((R - I)(p - g) + t)], algebraically
 * DeformGraph::predict_mesh (Deform.hpp:230-249), rounded once. */
int arap_node_table(int n, const float* rot, const float* trans, const float* node_pos,
                    float* table_out, arap_stream_t stream);

/* Six endpoints per Gaussian mu +/- (s_a + 1e-3) * 2 * R(q) e_a
 * (GaussianView::GetEndPoints, GaussianView.cpp:4643-4668).
 * ends_out in planes layout [18][N] (endpoint e, component c at plane 3e+c;
 * e = 2a for +axis a, 2a+1 for -axis a).  ends_xyz_out (optional) receives the
 * same points endpoint-major as xyz triples [(e*N + i)*3 + c], the input
 * arap_compute_weights expects for the endpoint weights. */
int arap_end_points(int N, const float* pos, const float* rot, const float* scale,
                    float* ends_out, float* ends_xyz_out, arap_stream_t stream);

/* One frame of Gaussian skinning, fused:
 *   ED blend of the 6 endpoints (GaussianView::UpdatePosition,
 *   GaussianView.cpp:3022-3040; DeformGraph::predict_mesh Deform.hpp:230-249)
 *   then the per-Gaussian refit (UpdateAsSixPointsWithdrawBad,
 *   GaussianView.cpp:3081-3166): centre, M = (P - c) Q^+, polar R/K,
 *   quaternion, scale K_a/((s0_a+1e-3)*2)*s0_a, SH rotated by q q_old^-1.
 *   ends      [18][N] in/out (deformed in place, every Gaussian)
 *   ends_idx  [k][6][N], ends_w [k][6][N]: kNN of each endpoint, exactly what
 *             arap_compute_weights returns for the 6N endpoint-major points
 *             (neighbour j of endpoint e of Gaussian i at [(j*6 + e)*N + i])
 *   node_table[n*16] from arap_node_table
 *   scale0    [N*3]  scales at endpoint creation (scale_backup_vector)
 *   static_mask [N] (uint8, optional): 1 = skip refit (static_gaussians)
 *   pos_out [N*3], rot_inout [N*4] (in: q of the previous frame), scale_out [N*3]
 *   shs_inout [N*48] optional, cov_out [N*6] optional (xx,xy,xz,yy,yz,zz of
 *   R diag(s)^2 R^T).
 *   status    device word (optional): ARAP_ENONFINITE when a polar factor
 *             does not converge to a finite value. */
int arap_skin_gaussians(int N, int k, float* ends, const int32_t* ends_idx,
                        const float* ends_w, const float* node_table, const float* scale0,
                        const uint8_t* static_mask, float* pos_out, float* rot_inout,
                        float* scale_out, float* shs_inout, float* cov_out, int precision,
                        int32_t* status, arap_stream_t stream);

/* Skinning plan: no counterpart in the reference; a set-up-time layout of
 * the endpoint kNN for arap_skin_gaussians_planned.
 * - Per tile of 128 Gaussians it keeps the distinct nodes the tile's endpoints
 *   blend (at most 256), placed in shared-memory slots chosen so that the
 *   lanes of a warp rarely read two records from one bank, and each
 *   neighbour as an 8-bit slot index.
 * - Each endpoint's neighbours are ordered by node id; the tile's weights and
 *   slot indices form one contiguous block in the order a frame reads them.
 * Build it once after arap_compute_weights of the endpoints, and again
 * whenever ends_idx/ends_w or the Gaussian order change. Synchronises. */
typedef struct arap_skin_plan arap_skin_plan;
int arap_skin_plan_create(arap_skin_plan** out, int N, int k, const int32_t* ends_idx,
                          const float* ends_w, arap_stream_t stream);
/* tiles; tiles with more than 256 distinct nodes (skinned from the global table);
 * the most node records a tile of the others stages (its largest slot + 1). */
int arap_skin_plan_info(const arap_skin_plan* plan, int* tiles, int* overflow_tiles, int* max_nodes);
/* Read and clear the device status word of the plan's skinning launches
 * (synchronises the stream). */
int arap_skin_plan_status(arap_skin_plan* plan, arap_stream_t stream);
void arap_skin_plan_destroy(arap_skin_plan* plan);
/* arap_skin_gaussians with the plan's layout; the same results up to the
 * rounding of each blend's sum (its terms are added in node-id order, not
 * kNN order).
 * - A CTA copies its tile's block of weights and indices into shared memory
 *   with one bulk copy (TMA) and its node records once.
 * - ends_idx/ends_w are read only for tiles over 256 nodes (in kNN order, as
 *   arap_skin_gaussians). N and k are the plan's. */
int arap_skin_gaussians_planned(const arap_skin_plan* plan, float* ends, const int32_t* ends_idx,
                                const float* ends_w, const float* node_table, const float* scale0,
                                const uint8_t* static_mask, float* pos_out, float* rot_inout,
                                float* scale_out, float* shs_inout, float* cov_out, int precision,
                                arap_stream_t stream);

/* Adjoint of arap_skin_gaussians' mu and Sigma with respect to the node
 * transforms: given the upstream gradients grad_pos [N*3] and grad_cov [N*6]
 * (packed xx,xy,xz,yy,yz,zz, dL = sum_p grad_cov_p dSigma_p), ADDS dL/dR_j and
 * dL/dt_j into grad_node [n*12] ([dR column-major 9 | dt 3] per node; zero it
 * first).  ends_in are the endpoints the forward started from (before it
 * deformed them in place); node_table is the forward's table.  The blend and the
 * per-Gaussian polar factor are recomputed, not stored.  No reference
 * counterpart: the reference has no gradient of its skinning. */
int arap_skin_gaussians_backward(int N, int k, const float* ends_in, const int32_t* ends_idx,
                                 const float* ends_w, const float* node_table, const float* scale0,
                                 const uint8_t* static_mask, const float* grad_pos, const float* grad_cov,
                                 float* grad_node, int32_t* status, arap_stream_t stream);
/* arap_skin_gaussians_backward with a skinning plan of the same endpoints
 * (ends_idx/ends_w are read only when the plan has tiles over 256 nodes; then
 * the whole call is arap_skin_gaussians_backward).  Per tile the blend is
 * recomputed from the staged node records, and each node's gradient is summed
 * over the tile's references to it in the plan's fixed order, then added to
 * grad_node with one atomic per (tile, node, component).  The same result up
 * to float rounding of the sums.  Device errors go to the plan's status word. */
int arap_skin_gaussians_backward_planned(const arap_skin_plan* plan, const float* ends_in,
                                         const int32_t* ends_idx, const float* ends_w,
                                         const float* node_table, const float* scale0,
                                         const uint8_t* static_mask, const float* grad_pos,
                                         const float* grad_cov, float* grad_node, arap_stream_t stream);

/* Per-node unit quaternion of the Newton polar factor of R
 * (FastUpdateSamplesSH, GaussianView.cpp:3172-3181; FastgetOthogonalMatrix
 * helper.cpp:506-517).  quat_out [n*4] (w,x,y,z).  status: optional device
 * word, ARAP_ENONFINITE when an iteration does not stay finite. */
int arap_node_quaternions(int n, const float* rot, float* quat_out, int precision, int32_t* status,
                          arap_stream_t stream);

/* One frame of sample skinning, fused: ED blend of the sample position
 * (UpdatePositionforSamples GaussianView.cpp:3060-3077) and slerp-blended
 * rotation of the sample's 48-float feature (RotateSHs cudakdtree.cu:201-222).
 *   sample_pos [S*3] in/out, idx/w [k][S] planes, node_table, node_quat [n*4],
 *   feature [S*48] in/out (optional), static_mask [S] uint8 optional. */
int arap_skin_samples(int S, int k, float* sample_pos, const int32_t* idx, const float* w,
                      const float* node_table, const float* node_quat, float* feature,
                      const uint8_t* static_mask, arap_stream_t stream);

/* New node positions: ED blend of each node's position with its anchor kNN
 * (GaussianView.cpp:3042-3052).  node_pos_out must not alias node_table's
 * source positions. */
int arap_update_nodes(int n, int k, const float* node_pos, const int32_t* anchor_idx,
                      const float* anchor_w, const float* node_table, float* node_pos_out,
                      arap_stream_t stream);

/* Items whose k neighbours are all static (CheckStaticSamples,
 * GaussianView.cpp:2038-2070).  For Gaussians pass the 6 endpoint kNN as
 * groups=6 (a Gaussian is static only if all 6*k neighbours are).
 * node_is_static [n] uint8; mask_out [P] uint8. */
int arap_static_mask(int P, int k, int groups, const int32_t* idx,
                     const uint8_t* node_is_static, uint8_t* mask_out, arap_stream_t stream);

/* ----------------------------------------------------- control targets --- */

/* Control-target generators on the active blocks (type 1), in place on aims:
 *   translate: aims += delta                (UpdateAimPosition GaussianView.cpp:2920-2933)
 *   twist:     rotate about an axis through the active centroid by radian
 *              (UpdateAimPositionTwist 2935-2959, PointRotateByAxis helper.cpp:1077-1100)
 *   scale:     centre + s*(aim - centre)    (UpdateAimPositionScale 2961-2983)
 * active_nodes [n_active] (device): node ids of the active blocks in block
 * order; a node listed twice is moved twice, as the reference loops do.  The
 * centroid is the mean of node_pos over the same list. */
int arap_aims_translate(float* aims, const int32_t* active_nodes, int n_active, float dx,
                        float dy, float dz, arap_stream_t stream);
int arap_aims_twist(float* aims, const float* node_pos, const int32_t* active_nodes,
                    int n_active, float ax, float ay, float az, float radian,
                    arap_stream_t stream);
int arap_aims_scale(float* aims, const float* node_pos, const int32_t* active_nodes,
                    int n_active, float s, arap_stream_t stream);

/* ----------------------------------------------------------------- grid --- */

typedef struct {
  float min_xyz[3];  /* scene box (getOverallAABB, GaussianView.cpp:3601-3631) */
  float max_xyz[3];
  float step;        /* cell edge: max over axes of extent / grid_num */
  float interval;    /* sample spacing: step / 4 (SAMPLES_PER_GRID, helper.hpp:56) */
  int grid_num;
  int n_valid;       /* occupied cells (non-empty lists) */
  long long n_pairs; /* total (cell, Gaussian) entries */
} arap_grid_info;

typedef struct arap_grid arap_grid;

/* Bin N Gaussians into the grid_num^3 grid: every cell covered by a
 * Gaussian's box (centre +/- R s_3d, s_3d = sqrt(-2 ln((1/255)/opacity)) s,
 * widened by `padding` cells; GaussianView.cpp:3961-4019 and
 * GetBoxesGsGrid cudakdtree.cu:425-451) lists that Gaussian.  Lists are in
 * ascending Gaussian order, as the reference's serial fill
 * (GaussianView.cpp:4077-4100) leaves them.  rot = (w,x,y,z) [N*4]; scale and
 * opacity activated.  The handle owns its device arrays; synchronises. */
int arap_grid_build(arap_grid** out, int N, const float* pos, const float* rot, const float* scale,
                    const float* opacity, int grid_num, int padding, arap_grid_info* info_host,
                    arap_stream_t stream);

/* Device arrays owned by the handle: cell_offsets [g^3+1] (exclusive prefix
 * of the per-cell counts, grid_gs_prefix_sum shifted by one), cell_lists
 * [n_pairs] (grided_gs_idx), valid_cells [n_valid] ascending (valid_grid_idx). */
int arap_grid_arrays(const arap_grid* grid, const int32_t** cell_offsets, const int32_t** cell_lists,
                     const int32_t** valid_cells);

/* Read and clear the grid's device status word (synchronises the stream). */
int arap_grid_status(arap_grid* grid, arap_stream_t stream);

/* Stable order of N Gaussians by the grid cell of their centre (cell index
 * x*g^2 + y*g + z ascending, original order within a cell): the reorder the
 * reference applies before binning (GaussianView.cpp:3918-3953).  order_out
 * [N]: order_out[r] = original index of the Gaussian placed at rank r.
 * Synchronises. */
int arap_grid_center_order(const arap_grid* grid, int N, const float* pos, int32_t* order_out,
                           arap_stream_t stream);

/* Size of the static device scratch array of arap_grid_center_order_noalloc. */
#define ARAP_CENTER_SCRATCH_BYTES (8u << 20)

/* No counterpart in the reference: an addition of this library for callers
 * that may not allocate device memory while they run (a frame loop where the
 * device-wide synchronisation of cudaMalloc/cudaFree would stall rendering, or
 * a process whose device memory is fully reserved by its own allocator).
 * Same arguments and result as arap_grid_center_order, but no allocation: the
 * scratch (cell [N], per-cell counters, offsets and flags [4 g^3 + 2], occupied
 * cells [g^3], scan sums) is carved from one static device array of
 * ARAP_CENTER_SCRATCH_BYTES, about 4 N + 20 g^3 bytes in all; larger requests
 * return ARAP_EUNSUPPORTED before any device work.  A cell holding more than
 * 16384 centres is merge-sorted with the rest of the array (4 bytes per
 * centre of such cells), ARAP_EUNSUPPORTED when that does not fit.  Every
 * call looks up the array's address (cudaGetSymbolAddress) on the current
 * device; the first lookup on a device loads the module there, so make the
 * first call before any stream capture.  Calls that overlap on the GPU (other
 * streams, other host threads) share the array and race: serialise them.
 * Synchronises. */
int arap_grid_center_order_noalloc(const arap_grid* grid, int N, const float* pos, int32_t* order_out,
                                   arap_stream_t stream);

/* 64 samples per occupied cell, cell-major, sample s at
 * min + cell*step + (0.5 + (s/16, s/4%4, s%4)) * interval
 * (GaussianView.cpp:4104-4133).  samples_out [n_valid*64*3]. */
int arap_grid_samples(const arap_grid* grid, float* samples_out, arap_stream_t stream);

/* Adaptive low-pass filter per occupied cell (GetAdaLpfRatio,
 * GaussianView.cpp:4670-4751): lpf * M M^T, M the least-squares linear map of
 * the unit cube's corners onto the cell's corner samples / 3.
 * samples [n_valid*64*3]; out [n_valid*9] row-major. */
int arap_grid_ada_lpf(const arap_grid* grid, const float* samples, float lpf, float* out,
                      arap_stream_t stream);

/* Gaussian-mixture density at the grid samples, this library's definition of
 * CudaRasterizer::forward3d_grid (call sites GaussianView.cpp:4222-4249):
 *   sigma(x) = sum_i a_i exp(-1/2 d^T (S_i + L)^-1 d),  F(x) = sum_i (...) SH_i
 * over the sample's cell list, S_i = R diag(s)^2 R^T, L = the cell's adaptive
 * 3x3 (ada, [n_valid*9]) or lpf * I when ada is null.
 * sigma_out [n_valid*64], feature_out [n_valid*64*48]. */
int arap_grid_density(const arap_grid* grid, const float* pos, const float* rot, const float* scale,
                      const float* opacity, const float* shs, const float* samples, const float* ada,
                      float lpf, float* sigma_out, float* feature_out, arap_stream_t stream);

/* Stage-II alignment, the library's definition of the step the viewer runs
 * through the un-vendored rasteriser (L1loss3d + backward3d_grid,
 * GaussianView.cpp:4398-4448).  Attributes are raw: pos [N*3], rot [N*4]
 * (w x y z, normalised when used), log_scale [N*3], logit_opacity [N],
 * shs [N*48], for the N Gaussians the grid was built over (its cell lists are
 * used as built).  At each sample of the occupied cells (samples as
 * arap_grid_samples), with the filter ada / lpf as arap_grid_density:
 *   loss = sum |sigma - aim_sigma| + feature_weight * sum |F - aim_feature|_1
 * over the samples of cells with cell_active[v] != 0 (all when null), sign(0)
 * = 0.  Writes the gradient to the raw attributes (grad_* shaped as the
 * attributes; each Gaussian's pairs summed in ascending cell order, so the
 * result is deterministic).  loss_host (nullable, synchronises): [2] = shape
 * and feature loss.  The first call allocates 58 floats per (cell, Gaussian)
 * pair plus 2 per occupied cell, kept with the grid. */
int arap_stage2_loss_grad(const arap_grid* grid, const float* pos, const float* rot, const float* log_scale,
                          const float* logit_opacity, const float* shs, const float* samples, const float* ada,
                          float lpf, const float* aim_sigma, const float* aim_feature,
                          const uint8_t* cell_active, float feature_weight, float* grad_pos, float* grad_rot,
                          float* grad_log_scale, float* grad_logit_opacity, float* grad_shs, double* loss_host,
                          arap_stream_t stream);

/* One Adam step (update3d's role, GaussianView.cpp:4451-4476) of the raw
 * attributes of the Gaussians with moved[i] != 0 (all when null), step >= 1
 * counting from 1, beta1 0.9, beta2 0.999, eps 1e-8.  lr_host [5]: rates for
 * opacity, SH, mean, quaternion, log-scale (the viewer's defaults are
 * 0, 0.002, 0.005, 0.1, 0.0001, GaussianView.hpp:418).  m, v [N*59]: moments
 * per Gaussian in the order opacity | SH 48 | mean 3 | quaternion 4 |
 * log-scale 3, zero before the first step. */
int arap_stage2_adam(int N, int step, const float* lr_host, const uint8_t* moved, float* logit_opacity,
                     float* shs, float* pos, float* rot, float* log_scale, const float* grad_logit_opacity,
                     const float* grad_shs, const float* grad_pos, const float* grad_rot,
                     const float* grad_log_scale, float* m, float* v, arap_stream_t stream);

/* Cell flags of the Stage-II loop over the grid's occupied cells, both
 * nullable (at least one given):
 * - empty_out [n_valid] (JudgeEmptyGrid, GaussianView.cpp:4272-4316): 1 for a
 *   cell that neither holds target density (its 64 aim_opacity values, summed
 *   in order in float, exceed 1e-6) nor is a face neighbour of such a cell;
 * - converged_io [n_valid] (ExpandOpRange, GaussianView.cpp:4319-4360): every
 *   cell that is a face neighbour of a cell not converged becomes not
 *   converged (0); flags are bytes, nonzero = converged.
 * aim_opacity [n_valid*64] is needed for empty_out. */
int arap_stage2_cell_flags(const arap_grid* grid, const float* aim_opacity, uint8_t* empty_out,
                           uint8_t* converged_io, arap_stream_t stream);

void arap_grid_destroy(arap_grid* grid);

/* ------------------------------------------------------------ render --- */

/* Headless rasteriser of N Gaussians into a device image, the published 3D
 * Gaussian splatting forward standing in for the un-vendored
 * CudaRasterizer::forward the viewer draws the deformed field with
 * (GaussianView.cpp:1066-1127); no window or GL interop.  Activated
 * attributes as the skinning writes them: pos [N*3], shs [N*48] (interleaved
 * rgb per coefficient, the first (sh_degree+1)^2 used), opacity [N], scale
 * [N*3], rot [N*4] (w x y z, 16-byte aligned).  view_host, proj_host [16]:
 * row-major world->camera and world->clip matrices (camera looks along +z);
 * campos_host [3]; background_host [3].  image_out [3*height*width] planes;
 * final_t_out [height*width] (nullable): the transmittance left;
 * n_contrib_out (nullable): the Gaussians composited per pixel.  A tile's
 * list of up to 16384 Gaussians is sorted in shared memory, a longer one in
 * global memory (chunk sorts and merges), with the same order.
 * Allocates stream-ordered scratch and synchronises. */
int arap_render(int N, const float* pos, const float* shs, const float* opacity, const float* scale,
                const float* rot, float scale_modifier, int sh_degree, const float* view_host,
                const float* proj_host, const float* campos_host, float tan_fovx, float tan_fovy, int width,
                int height, const float* background_host, float* image_out, float* final_t_out,
                int32_t* n_contrib_out, arap_stream_t stream);

/* -------------------------------------------------------------- PLY IO --- */

/* 3D Gaussian splatting binary PLY files, host memory only (no device call;
 * usable without a GPU). Replaces the viewer's loadPly / loadPly_Origin /
 * savePly (GaussianView.cpp:43-339). A file is accepted when it is binary
 * little-endian with one `vertex` element of float properties holding x y z,
 * f_dc_0..2, f_rest_* for SH degree 0..3, opacity, scale_0..2, rot_0..3 and
 * optionally `index`; anything else is ARAP_EBADINPUT (the viewer aborts). */
int arap_ply_info(const char* path, int64_t* count, int* sh_degree, int* has_index);

/* Loads count splats (as reported by arap_ply_info) into activated SoA arrays:
 * pos [count*3], shs [count*48] (rgb per coefficient, bands above the file's
 * degree zero), opacity [count] (logistic of the stored logit), scale
 * [count*3] (exp of the stored log), rot [count*4] (normalised, w x y z as
 * stored). morton_order != 0 reorders the splats by the viewer's 21-bit-per-axis
 * Morton code over the bounding box (ties in file order), as loadPly does.
 * box_min/box_max [3] (nullable): the bounding box. index [count] (nullable;
 * requires the property): the rounded `index` property.  Runs on up to 16
 * host threads; the result does not depend on their number. */
int arap_ply_load(const char* path, int64_t count, int morton_order, float* pos, float* shs, float* opacity,
                  float* scale, float* rot, float* box_min, float* box_max, int32_t* index);

/* Saves the splats inside [box_min, box_max] (bounds included) that are not
 * flagged in too_small [count] (nullable), as savePly does: SH degree 3,
 * normals zero, scale stored as log, opacity as logit, rot as given.
 * written (nullable): the number of splats written. */
int arap_ply_save(const char* path, int64_t count, const float* pos, const float* shs, const float* opacity,
                  const float* scale, const float* rot, const float* box_min, const float* box_max,
                  const uint8_t* too_small, int64_t* written);

/* --------------------------------------------------------------- misc --- */

/* Read and clear a caller-owned device status word (an int32 the caller
 * allocated and zeroed, passed as `status` to the stateless calls): returns
 * the first ARAP_* code raised into it since it was last cleared.
 * Synchronises the stream. */
int arap_status_read(int32_t* status_dev, arap_stream_t stream);

/* Library version string. */
const char* arap_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ARAP_GB300_H */
