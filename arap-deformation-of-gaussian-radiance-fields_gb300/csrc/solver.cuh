// Plan and parameter layout of the persistent Gauss-Newton / PCG solver.
#pragma once

#include "arap_common.cuh"

namespace arap {

constexpr int kGJBlock = 32;         // pivot block of the coarse Gauss-Jordan inversion (one warp)
constexpr int kMaxCoarseAggs = 80;   // aggregates of the coarse space (12 unknowns each)
constexpr int kMaxCoarse = 12 * kMaxCoarseAggs;

// Coupling items of one free node j (all rows of J that touch x_j besides its
// own rotation rows).  int4 {kind, a, b, c}:
//   ITEM_OUT    regularisation rows (j -> k), k = Neighbor[t] of j
//               a = free rank of k (-1 if static), b = node k, c = bits(scale)
//   ITEM_IN     regularisation rows (i -> j) of a free node i
//               a = free rank of i, b = node i, c = bits(scale)
//   ITEM_STATIC rows (i -> j) of a static node i: f = -w t_j
//               a = -1, b = node i, c = 0
//   ITEM_CON    constraint group g whose member anchors contain j
//               a = member-anchor slot (u*k + t), b = g, c = 0
// The low 4 bits of the kind word hold the kind; the bits above hold the
// coarse aggregate of node a's free rank (ITEM_OUT / ITEM_IN) when the
// two-level preconditioner is on.
enum { ITEM_OUT = 0, ITEM_IN = 1, ITEM_STATIC = 2, ITEM_CON = 3 };

struct SolveParams {
  int n, k, F, G, U, n_items;
  const int32_t* free_ids;   // [F]
  const int32_t* rank;       // [n]
  const int32_t* item_off;   // [F+1]
  const int4* items;         // [n_items]
  const int32_t* grp_off;    // [G+1] member slots per group
  const int32_t* grp_member; // [U] node id of member u
  const float* grp_mult;     // [G] number of members (|S_b| or 1)
  const int32_t* tsrc_off;   // [G+1] target sources per group
  const int32_t* tsrc;       // aims indices (first min(20,|b|) block entries, or the node)
  const int32_t* mem_rank;   // [U*k] free rank of anchor l (-1 when not free)
  const int32_t* mem_node;   // [U*k] anchor node l
  const float* mem_w;        // [U*k] anchor weight a_cl
  float4* mem_geo;           // [U*k] per frame {a, v_c - g_l}
  float4* grp_target;        // [G] per frame {target xyz, mult}
  double* grp_f;             // [G*3] constraint residual of each group at the current x
  float4* item_cq;           // [n_items] per solve, ITEM_CON only: {sum a (v_c - g_j), sum a} over
                             // the group's anchors equal to the item's node (first item of a run)
  const float* node_pos;     // [n*3]
  const float* aims;         // [n*3]
  double* x;                 // [F*12] Gauss-Newton iterate
  float* xf;                 // [F*12] float copy of x
  float2* xo;                // [F*12] x - [I | 0] as float-float (hi, lo): the mixed form's residual
  float* h;                  // [F*12] step
  float* r;                  // [F*12] PCG residual
  float* z;                  // [F*12] u_f = Dinv r (fine part of the preconditioned residual)
  float* p0;                 // [F*12] search direction p
  float* p1;                 // [F*12] s = (J^T J) p
  float* q;                  // [F*12] w = (J^T J) u
  float* u;                  // [F*12] preconditioned residual u = u_f + P zc
  float* dinv;               // [F*144] inverse of the 12x12 diagonal block of J^T J
  double* partials;          // [2 * kReduceSlots * gridDim] barrier partial sums
  GridBarrier* bar;
  double* stats;             // [8] device-side stats (see solver.cu)
  float* rot_out;            // [n*9]
  float* trans_out;          // [n*3]
  const double* x_in;        // grad-only mode: evaluation point
  double* grad_out;          // grad-only mode: J^T f
  double wr, wg, wc;         // square roots of w_rot, w_reg, w_con (Deform.hpp:452-454)
  float wrf, wgf, wcf;       // the same rounded to float (FP64 conversions are slow on this part)
  float wr_lo, wg_lo, wc_lo; // and their rounding errors (float-float weights)
  float wf;                  // weighting factor
  const int32_t* order;      // [F] processing order of the free nodes (cost-balanced)
  int max_iters, early_exit, pcg_max;
  float pcg_tol;
  float coarse_reuse;        // keep the coarse inverse while the last step < coarse_reuse |x|
  int mode;                  // 0 solve, 1 gradient/energy only
  int refine;                // mixed precision: FP64 refinement sweeps per solve
  // two-level preconditioner (coarse space: one affine ED transform per
  // aggregate; node j of aggregate a gets dR_j = dR_a, dt_j = dR_a (g_j - g_pa) + dT_a)
  int NA, NC;                // aggregates, coarse unknowns (12 NA); NA = 0 disables it
  const int32_t* agg;        // [F] aggregate of each free node
  const int32_t* pivot;      // [NA] node id of each aggregate's reference node
  const int32_t* agg_count;  // [NA] free nodes per aggregate
  double* Qd;                // [NA*NA*16] 4x4 kernels of the coarse blocks
  float* Cw;                 // [2*NC*NC] coarse matrix / Gauss-Jordan ping-pong
  float* Cinv;               // [NC*NC] inverse of the coarse matrix
  double* rotagg;            // [2*NA*81] per-aggregate sums of J_rot^T J_rot (GN-iteration parity)
  double* rc;                // [2*NC] restricted residual, double-buffered
  float* zc;                 // [NC] coarse correction
  const int32_t* mem_agg;    // [U*k] aggregate of each free anchor (-1 otherwise)
  float4* dpiv;              // [F] per solve: g_j - g_pivot(agg(j))
  // J_g u of each constraint group by linearity when the two-level
  // preconditioner is on: u = u_f + P zc gives J_g u = J_g u_f + sum_a V_ga . zc_a
  const int32_t* gca_off;    // [G+1] distinct aggregates of each group's free anchors
  const int32_t* gca;        // aggregate ids
  float4* gcv;               // per solve: V_ga = sum over anchors in a of w (v_c - g_pivot(a), 1)
  float4* uzg;               // [G] w_con J_g u_f, refreshed after each update
  // CTA-resident node tables: each CTA keeps the fixed data of the free nodes
  // it processes (coupling items with their geometry, diagonal-block
  // inverses, aggregate offsets) in dynamic shared memory, for as many of its
  // nodes as stage_cap bytes hold; the rest are read from the global tables
  const int4* con_info;      // [F] {coarse-list entries, constraint items, aggregates coupled to the node,
                             // member-anchor slots of its constraint items' groups} (0 without a coarse level)
  int stage_cap;             // dynamic shared memory of the launch, bytes (0: nothing staged)
  int resident;              // every CTA holds all of its nodes, with their PCG vectors (two-level PCG only)
};

// Shared-memory bytes of one staged node: its 12x12 inverse block (576), two
// node records (32) and its aggregate offset (16), plus 32 per coupling item
// (item + geometry) and 20 per coarse-list entry of its constraint items.
constexpr int kStageNodeBytes = 576 + 32 + 16;
constexpr int kStageItemBytes = 32;
constexpr int kStageListBytes = 20;
// Resident mode adds per node its PCG vectors (8 x 12 floats), the float copy
// of x (12) and its 9x9 rotation block (rows padded to 12), per coupling item
// the other node's aggregate offset (16), per constraint item its group id
// and the group's w_con J_g v with the range of its member-anchor slots (28),
// per such slot its anchor's free rank and geometry (20), per aggregate
// coupled to the node its id
// and the node's 12x12 block of (J^T J)_{reg,con} P on it (580), and per CTA
// its rows of the coarse inverse.
constexpr int kResVecs = 8;
constexpr int kResNodeBytes = kResVecs * 48 + 48 + 9 * 48;
constexpr int kResItemBytes = 16;
constexpr int kResConBytes = 28;  // group id, w_con J_g v, slot range of the group
constexpr int kResSlotBytes = 20; // member-anchor slot of a constraint item's group: free rank, geometry
constexpr int kResAggBytes = 576 + 48 + 4;  // block, the aggregate's zc (staged per iteration), id

}  // namespace arap
