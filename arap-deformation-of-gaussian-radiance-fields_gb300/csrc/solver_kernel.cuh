// The persistent Gauss-Newton kernel: one cooperative launch runs the whole
// Deform::optimize loop (Deform.cpp:95-169) -- gradient and energy, block
// preconditioner, PCG for (J^T J) h = -J^T f, halving line search, stop test
// -- and writes the node transforms (Deform.hpp:140-151).
#pragma once

#include "solver_device.cuh"

namespace arap {

// stats slots written by CTA 0; ST_T_PREP..ST_T_CINV are nanoseconds spent in
// each phase (global timer, read by thread 0 of CTA 0 after the phase's
// barrier); ST_T_W_* are the largest per-CTA sums of work time inside PCG
// (from leaving one barrier to entering the next), combined with atomicMax
// on the bit patterns of non-negative doubles.
enum {
  ST_ITERS = 0, ST_PCG = 1, ST_HALV = 2, ST_E0 = 3, ST_E = 4, ST_CONV = 5, ST_NONFINITE = 6,
  ST_T_PREP = 8, ST_T_GRAD = 9, ST_T_COARSE = 10, ST_T_PCG = 11, ST_T_LS = 12, ST_T_CINV = 13,
  ST_T_W_SPMV = 14, ST_T_W_UPD = 15, ST_T_W_CSOLVE = 16, ST_CFALL = 17, ST_CINV_N = 18
};
constexpr int ST_HALV_IT = 24;  // cumulative halvings after each of the first kHalvIters GN iterations
constexpr int kHalvIters = 64;
constexpr int kStatSlots = ST_HALV_IT + kHalvIters;

// Entry e of x as the float-float offset x - [I | 0] (P.xo), for the mixed
// form's residual.
__device__ __forceinline__ void put_xo(const SolveParams& P, int e, double v) {
  const int c = e % 12;
  const double d = v - ((c == 0 || c == 4 || c == 8) ? 1.0 : 0.0);
  const float hi = __double2float_rn(d);
  P.xo[e] = make_float2(hi, __double2float_rn(d - (double)hi));
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Shared scratch of the persistent kernel, reused phase by phase (phases are
// separated by grid barriers, which include __syncthreads).
constexpr int kGJRows = 8;  // rows of a CTA's strip handled together
constexpr int kScratchFloats = kGJBlock * (kGJBlock + 1) + kGJRows * (kGJBlock + 1) + kGJRows * kGJBlock;
static_assert(kScratchFloats >= kMaxCoarse, "scratch holds the restricted residual");

// Inverse of the coarse matrix in Cw[0] by blocked Gauss-Jordan (float32, no
// pivoting: the matrix is symmetric positive definite).  For each pivot block
// K (kGJBlock = 32 wide, the last one padded with the identity), warp 0 of
// every CTA inverts A_KK in registers (lane j holds column j; the pivot
// column is published in shared memory, one warp barrier per pivot; the same
// bits in every CTA), then every CTA updates its own strip of rows:
//   A_KK <- A_KK^-1, A_Kj <- A_KK^-1 A_Kj, A_iK <- -W_iK,
//   A_ij <- A_ij - W_iK A_Kj,  W = A_iK A_KK^-1,
// with W of the strip in shared memory and the column A_Kj streamed from L2 in
// one batch per column.  Reads Cw[src] and writes Cw[1-src] (Cinv for the
// last block), so one grid barrier per block suffices.  Returns false on a
// barrier failure; *ok = 0 when a pivot was not positive.
template <class G>
__device__ bool coarse_invert(const SolveParams& P, G& gs, int* ok, float* sm) {
  constexpr int KB = kGJBlock, KP = kGJBlock + 1;
  static_assert(KB == 32, "one lane per pivot column");
  float(*pv0)[KP] = reinterpret_cast<float(*)[KP]>(sm);
  float(*wrow)[KP] = reinterpret_cast<float(*)[KP]>(sm + KB * KP);
  // per strip row: -W_iK, or the row of A_KK^-1 for rows inside K (16-byte rows)
  float(*wsel)[KB] = reinterpret_cast<float(*)[KB]>(sm + KB * KP + kGJRows * KP);
  static_assert((KB * KP + kGJRows * KP) % 4 == 0, "float4 rows");
  const int NC = P.NC;
  const size_t NC2 = (size_t)NC * NC;
  const int tid = threadIdx.x, bd = blockDim.x;
  const int R = (NC + (int)gs.nb - 1) / (int)gs.nb;
  const int r_begin = min(NC, (int)gs.bid * R), r_end = min(NC, r_begin + R);
  int src_i = 0;
  *ok = 1;
  __shared__ int s_bad;
  for (int K0 = 0; K0 < NC; K0 += KB) {
    const int kb = min(KB, NC - K0);
    const float* src = P.Cw + src_i * NC2;
    float* dst = (K0 + kb >= NC) ? P.Cinv : P.Cw + (1 - src_i) * NC2;
    if (tid < 32) {
      // column `lane` of the pivot block, padded with the identity, inverted
      // in place by warp 0 (Gauss-Jordan without pivoting): per pivot m, lane
      // m publishes its column (the old A[*][m]) in shared memory
      // (double-buffered in wrow's space, so one warp barrier per pivot) and
      // every lane updates its column from it.  Every CTA gets the same bits.
      const int lane = tid;
      float* bc = &wrow[0][0];  // [2][32]
      float col[KB];
#pragma unroll
      for (int i = 0; i < KB; ++i)
        col[i] = (i < kb && lane < kb) ? __ldcg(src + (size_t)(K0 + i) * NC + K0 + lane) : (i == lane ? 1.f : 0.f);
      int bad = 0;
#pragma unroll
      for (int m = 0; m < KB; ++m) {
        float4* pub = reinterpret_cast<float4*>(bc + (m & 1) * KB);
        if (lane == m) {
#pragma unroll
          for (int i4 = 0; i4 < KB / 4; ++i4)
            pub[i4] = make_float4(col[4 * i4], col[4 * i4 + 1], col[4 * i4 + 2], col[4 * i4 + 3]);
        }
        __syncwarp();
        const float* cm = bc + (m & 1) * KB;
        const float pvt = cm[m];
        bad |= !(pvt > 0.f);
        const float ip = __frcp_rn(pvt);
        const float cmj = col[m];
#pragma unroll
        for (int i = 0; i < KB; ++i) {
          const float cim = cm[i];
          if (i == m)
            col[i] = (lane == m) ? ip : cmj * ip;
          else
            col[i] = (lane == m) ? -cim * ip : fmaf(-cim * ip, cmj, col[i]);
        }
      }
#pragma unroll
      for (int i = 0; i < KB; ++i) pv0[i][lane] = col[i];
      if (lane == 0) s_bad = bad;
    }
    __syncthreads();
    if (s_bad) *ok = 0;
    for (int r0 = r_begin; r0 < r_end; r0 += kGJRows) {
      const int nr = min(kGJRows, r_end - r0);
      for (int t = tid; t < kGJRows * KB; t += bd) {
        const int rr = t / KB, m = t % KB;
        wrow[rr][m] = (rr < nr && m < kb) ? __ldcg(src + (size_t)(r0 + rr) * NC + K0 + m) : 0.f;
      }
      __syncthreads();
      float wv = 0.f;
      if (tid < kGJRows * KB) {
        const int rr = tid / KB, n = tid % KB;
#pragma unroll 16
        for (int m = 0; m < KB; ++m) wv = fmaf(wrow[rr][m], pv0[m][n], wv);
      }
      if (tid < kGJRows * KB) {
        const int rr = tid / KB, n = tid % KB;
        const int iK = r0 + rr - K0;
        wsel[rr][n] = (iK >= 0 && iK < kb) ? pv0[iK][n] : -wv;
      }
      __syncthreads();
      for (int j = tid; j < NC; j += bd) {
        const int jK = j - K0;
        const bool inJ = jK >= 0 && jK < kb;
        float out[kGJRows];
        if (inJ) {
          // A_KK^-1 inside the pivot block, -W_iK elsewhere: both are in wsel
#pragma unroll
          for (int rr = 0; rr < kGJRows; ++rr) out[rr] = wsel[rr][jK];
        } else {
          float akj[KB];
#pragma unroll
          for (int m = 0; m < KB; ++m) akj[m] = m < kb ? __ldcg(src + (size_t)(K0 + m) * NC + j) : 0.f;
#pragma unroll
          for (int rr = 0; rr < kGJRows; ++rr) {
            const int iK = r0 + rr - K0;
            const bool inI = iK >= 0 && iK < kb;
            float v = (inI || rr >= nr) ? 0.f : __ldcg(src + (size_t)(r0 + rr) * NC + j);
            const float4* w4 = reinterpret_cast<const float4*>(&wsel[rr][0]);
#pragma unroll
            for (int m4 = 0; m4 < KB / 4; ++m4) {
              const float4 ww = w4[m4];
              v = fmaf(ww.x, akj[4 * m4], v);
              v = fmaf(ww.y, akj[4 * m4 + 1], v);
              v = fmaf(ww.z, akj[4 * m4 + 2], v);
              v = fmaf(ww.w, akj[4 * m4 + 3], v);
            }
            out[rr] = v;
          }
        }
#pragma unroll
        for (int rr = 0; rr < kGJRows; ++rr)
          if (rr < nr) dst[(size_t)(r0 + rr) * NC + j] = out[rr];
      }
      __syncthreads();
    }
    if (!gs.sync()) return false;
    src_i ^= 1;
  }
  return true;
}

// zc = Cinv rc (one warp per row, the row loaded as float4s in one batch, rc
// staged in shared memory), zero the other restriction buffer, and the group
// products w_con J_g u_f.  Every thread of the CTA calls it.
constexpr int kRowVec = (kMaxCoarse / 4 + 31) / 32;  // float4 loads per lane of a row
template <class G>
__device__ __forceinline__ void coarse_solve(const SolveParams& P, const G& gs, const double* rc,
                                             double* rc_other, int ok, float* s_rc) {
  const int lane = threadIdx.x & 31;
  const int gw = (int)(gs.bid * blockDim.x + threadIdx.x) >> 5;
  const int nw = (int)(gs.nb * blockDim.x) >> 5;
  const int NC = P.NC, n4 = NC / 4;
  for (int e = threadIdx.x; e < NC; e += blockDim.x) s_rc[e] = (float)__ldcg(rc + e);
  __syncthreads();
  const float4* s4 = reinterpret_cast<const float4*>(s_rc);
  for (int i = gw; i < NC; i += nw) {
    float a = 0.f;
    if (ok) {
      const float4* row = reinterpret_cast<const float4*>(P.Cinv + (size_t)i * NC);
      float4 v[kRowVec];
#pragma unroll
      for (int q = 0; q < kRowVec; ++q) {
        const int c = lane + 32 * q;
        v[q] = c < n4 ? __ldcg(row + c) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int q = 0; q < kRowVec; ++q) {
        const int c = lane + 32 * q;
        if (c < n4) {
          const float4 r4 = s4[c];
          a = fmaf(v[q].x, r4.x, fmaf(v[q].y, r4.y, fmaf(v[q].z, r4.z, fmaf(v[q].w, r4.w, a))));
        }
      }
    }
    a = warp_sum(a);
    if (lane == 0) P.zc[i] = a;
  }
  for (int e = gs.bid * blockDim.x + threadIdx.x; e < NC; e += gs.nb * blockDim.x) rc_other[e] = 0.0;
  // w_con J_g u_f for the next products, on the warps the rows leave idle
  for (int g = nw - 1 - gw; g < P.G; g += nw) con_jz_group(P, g);
}

// The whole solve on a group of nbk co-resident CTAs; bid is this CTA's index
// in the group.
template <typename RT, bool kCfgLimit>
__device__ __forceinline__ void solve_body(const SolveParams& P, int bid, int nbk) {
  __shared__ __align__(16) float s_scratch[kScratchFloats];
  const int lane = threadIdx.x & 31;
  const int gw = (bid * (int)blockDim.x + (int)threadIdx.x) >> 5;
  const int nw = (nbk * (int)blockDim.x) >> 5;
  const int gt = bid * (int)blockDim.x + (int)threadIdx.x;
  const int nt = nbk * (int)blockDim.x;
  const int F = P.F, k = P.k;
  // node order position p belongs to CTA p % nbk: the costliest nodes (the
  // order is by cost, descending) are spread over all SMs
  const int wib = threadIdx.x >> 5;
  GridSyncT<kCfgLimit> gs{P.bar, P.partials, 0u, (unsigned int)nbk, (unsigned int)bid};
  // phase timers, thread 0's only, kept in shared memory rather than registers
  // that would stay live through the whole kernel.  acc: prep, grad, coarse,
  // pcg, line search, inversion (ns).  work: PCG work of this CTA per phase
  // kind (products, update, coarse solve), from leaving a barrier to the last
  // warp of the CTA finishing its share (each warp posts its finish time to
  // wend; thread 0 reads the latest after the barrier).
  __shared__ struct {
    unsigned long long mark, w0, wend, inv0;
    double acc[6];
    unsigned long long work[3];
    int pend;
  } s_clk;
  if (threadIdx.x == 0) {
    s_clk.mark = global_ns();
    s_clk.wend = 0ull;
    s_clk.pend = -1;
    for (int q = 0; q < 6; ++q) s_clk.acc[q] = 0.0;
    for (int q = 0; q < 3; ++q) s_clk.work[q] = 0ull;
  }
  auto work_flush = [&]() {
    if (threadIdx.x == 0 && s_clk.pend >= 0) {
      s_clk.work[s_clk.pend] += s_clk.wend - s_clk.w0;
      s_clk.pend = -1;
    }
  };
  auto work_begin = [&]() {
    work_flush();
    if (threadIdx.x == 0) s_clk.w0 = global_ns();
  };
  auto work_end = [&](int slot) {
    if (lane == 0) atomicMax(&s_clk.wend, global_ns());
    if (threadIdx.x == 0) s_clk.pend = slot;
  };
  auto lap = [&](int slot) {
    if (threadIdx.x == 0) {
      const unsigned long long now = global_ns();
      s_clk.acc[slot] += (double)(now - s_clk.mark);
      s_clk.mark = now;
    }
  };

  // ---- per-frame geometry: member anchors, group targets, x = identity
  for (int slot = gt; slot < P.U * k; slot += nt) {
    const int c = P.grp_member[slot / k];
    const int l = P.mem_node[slot];
    P.mem_geo[slot] = make_float4(P.mem_w[slot], P.node_pos[3 * c] - P.node_pos[3 * l],
                                  P.node_pos[3 * c + 1] - P.node_pos[3 * l + 1],
                                  P.node_pos[3 * c + 2] - P.node_pos[3 * l + 2]);
  }
  for (int g = gt; g < P.G; g += nt) {
    // centre = float sum of the listed aims / count (Deform.cpp:56-64)
    const int a0 = P.tsrc_off[g], a1 = P.tsrc_off[g + 1];
    float cx = 0.f, cy = 0.f, cz = 0.f;
    for (int a = a0; a < a1; ++a) {
      const int s = P.tsrc[a];
      cx += P.aims[3 * s];
      cy += P.aims[3 * s + 1];
      cz += P.aims[3 * s + 2];
    }
    const float m = (float)(a1 - a0);
    P.grp_target[g] = make_float4(cx / m, cy / m, cz / m, P.grp_mult[g]);
  }
  for (int e = gt; e < F * 12; e += nt) {
    const int c = e % 12;
    const double v = P.mode == 1 ? P.x_in[e] : ((c == 0 || c == 4 || c == 8) ? 1.0 : 0.0);
    P.x[e] = v;
    P.xf[e] = (float)v;
    put_xo(P, e, v);
  }
  const bool coarse = P.NA > 0 && P.mode == 0;
  const bool resident = coarse && P.resident != 0;
  if (coarse) {
    for (int r = gt; r < F; r += nt) {
      const int j = P.free_ids[r];
      const int pv = P.pivot[P.agg[r]];
      P.dpiv[r] = make_float4(P.node_pos[3 * j] - P.node_pos[3 * pv], P.node_pos[3 * j + 1] - P.node_pos[3 * pv + 1],
                              P.node_pos[3 * j + 2] - P.node_pos[3 * pv + 2], 0.f);
    }
    for (int e = gt; e < P.NA * P.NA * 16; e += nt) P.Qd[e] = 0.0;
    for (int e = gt; e < 2 * P.NC; e += nt) P.rc[e] = 0.0;
    for (int e = gt; e < 2 * P.NA * 81; e += nt) P.rotagg[e] = 0.0;
    // V_ga of every group and aggregate of its free anchors
    for (int g = gt; g < P.G; g += nt) {
      const int s0 = P.grp_off[g], s1 = P.grp_off[g + 1];
      for (int f = P.gca_off[g]; f < P.gca_off[g + 1]; ++f) {
        const int a = P.gca[f];
        const int pv = P.pivot[a];
        float4 V = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int u = s0; u < s1; ++u) {
          const int c = P.grp_member[u];
          for (int t = 0; t < k; ++t) {
            const int slot = u * k + t;
            const int rk = P.mem_rank[slot];
            if (rk < 0 || P.agg[rk] != a) continue;
            const float w = P.mem_w[slot];
            V.x = fmaf(w, P.node_pos[3 * c] - P.node_pos[3 * pv], V.x);
            V.y = fmaf(w, P.node_pos[3 * c + 1] - P.node_pos[3 * pv + 1], V.y);
            V.z = fmaf(w, P.node_pos[3 * c + 2] - P.node_pos[3 * pv + 2], V.z);
            V.w += w;
          }
        }
        P.gcv[f] = V;
      }
    }
  }
  if (gt == 0)
    for (int q = ST_T_W_SPMV; q <= ST_CFALL; ++q) P.stats[q] = 0.0;
  if (!gs.sync()) return;
  stage_build(P, bid, nbk);
  // diagonal-block share of every constraint item (fixed for this solve): the
  // group's anchors equal to the item's node, summed into the first item of
  // the node's run of that group
  for (int e = gt; e < P.n_items; e += nt) {
    const int4 m = P.items[e];
    if ((m.x & 15) != ITEM_CON) continue;
    const int g = m.z;
    const int j = P.mem_node[m.y];
    const int b0 = P.item_off[P.rank[j]];
    bool first = true;
    if (e > b0) {
      const int4 pm = P.items[e - 1];
      first = !((pm.x & 15) == ITEM_CON && pm.z == g);
    }
    float4 cq = make_float4(0.f, 0.f, 0.f, 0.f);
    if (first) {
      const int s0 = P.grp_off[g], s1 = P.grp_off[g + 1];
      for (int u = s0; u < s1; ++u)
        for (int t = 0; t < k; ++t) {
          const int slot = u * k + t;
          if (P.mem_node[slot] != j) continue;
          const float4 gg = P.mem_geo[slot];
          cq.x = fmaf(gg.x, gg.y, cq.x);
          cq.y = fmaf(gg.x, gg.z, cq.y);
          cq.z = fmaf(gg.x, gg.w, cq.z);
          cq.w += gg.x;
        }
    }
    P.item_cq[e] = cq;
  }
  if (!coarse && !gs.sync()) return;
  if (coarse) {
    // coarse matrix P^T (J^T J at x = I) P, fixed for this solve
    for (int oi = gw; oi < F; oi += nw) coarse_rows_node(P, __ldg(P.order + oi));
    for (int g = gt; g < P.G; g += nt) coarse_rows_group(P, g);
    if (!gs.sync()) return;
  }

  lap(0);
  double e_first = 0.0, e_last = 0.0;
  int iters = 0, pcg_total = 0, halvings = 0, converged = 0;
  // reuse of the coarse inverse: the last accepted step and |x| before it,
  // whether an inverse is held (and its pivots were positive), PCG iterations
  // of the last system and of the last one solved with a fresh inverse
  double step_prev = 0.0, normv_prev = 0.0;
  int inv_held = 0, inv_ok = 0, pcg_prev = 0, pcg_fresh = 0, n_inv = 0;
  bool fresh = false;
  for (int it = 0; it < P.max_iters; ++it) {
    // ---- gradient -J^T f, energy, preconditioner, PCG start (h=0, r=g, z=M^-1 g)
    double red[3] = {0.0, 0.0, 0.0};
    // constraint residuals, one warp per group, for the nodes' products
    for (int g = gw; g < P.G; g += nw) {
      RT f[3];
      con_residual_warp<RT>(P, g, RT(0), f);
      if (lane == 0) {
        store_grp_f<RT>(P, g, 0, f[0]);
        store_grp_f<RT>(P, g, 1, f[1]);
        store_grp_f<RT>(P, g, 2, f[2]);
        red[0] += double(f[0]) * double(f[0]) + double(f[1]) * double(f[1]) + double(f[2]) * double(f[2]);
      }
    }
    if (!gs.sync()) return;
    for (int ws = wib; ws * nbk + bid < F; ws += kSolveWarps) {
      const bool stg = ws < s_stg.n;
      const int r = stg ? stg_node()[ws].x : __ldg(P.order + ws * nbk + bid);
      RT g_lane;  // this lane's entry of (J^T f)_r (lanes 0..11)
      float Q[10];
      double en;
      residual_node<RT, PASS_GRAD>(P, r, RT(0), g_lane, Q, en);
      if (lane == 0) red[0] += en;
      if (P.mode == 1) {
        if (lane < 12) P.grad_out[12 * (size_t)r + lane] = (double)g_lane;
        continue;
      }
      if (stg)
        build_dinv<true>(P, r, ws, Q);
      else
        build_dinv<false>(P, r, 0, Q);
      if (coarse) coarse_rot_node(P, r, P.rotagg + (it & 1) * 81 * P.NA);
      const float gc = lane < 12 ? -(float)g_lane : 0.f;
      const float zc = stg ? apply_dinv<true>(P, r, ws, gc) : apply_dinv<false>(P, r, 0, gc);
      // (the resident PCG restricts r - A z1 itself)
      if (coarse && !resident) coarse_restrict(P, r, gc, P.rc);
      if (lane < 12) {
        const size_t o = 12 * (size_t)r + lane;
        P.r[o] = gc;
        P.z[o] = zc;
        P.h[o] = 0.f;
        red[2] += (double)gc * (double)gc;
        if (resident && stg) {
          stg_vec(ws, RV_R)[lane] = gc;
          stg_vec(ws, RV_UF)[lane] = zc;
          stg_vec(ws, RV_H)[lane] = 0.f;
          stg_xf(ws)[lane] = __ldcg(P.xf + o);
        }
      }
      if (resident && stg) {
        __syncwarp();
        rot_block(P, ws);
      }
    }
    for (int e = gt; e < F * 12; e += nt) {
      const double v = __ldcg(P.x + e);
      red[1] += v * v;
    }
    if (!gs.template reduce<3>(red)) return;
    lap(1);
    const double e_old = red[0];
    const double normv = sqrt(red[1]);
    if (it == 0) e_first = e_old;
    e_last = e_old;
    if (P.mode == 1) {
      if (gt == 0) P.stats[ST_E] = e_old;
      return;
    }

    // ---- PCG on (J^T J) h = g in the Chronopoulos-Gear form, one reduction
    // per iteration:
    //   (1) p = u + beta p, s = w + beta s, h += alpha p, r -= alpha s,
    //       u_f = Dinv r and its restriction P^T r; plain barrier
    //   (2) two-level only: zc = Cinv P^T r and w_con J_g u_f; plain barrier
    //   (3) u = u_f + P zc, w = (J^T J) u; gamma = r.u, delta = w.u, r.r
    //   beta = gamma / gamma_old, alpha = gamma / (delta - beta gamma / alpha_old)
    const double rr0 = red[2];
    // the PCG scalars are float-float (hi, lo) pairs: its sums are
    // float-float reductions of float terms, and FP64 arithmetic (~64-cycle
    // latency, divisions many times that) would sit on every iteration's
    // critical path.  The recurrence den = delta - beta gamma / alpha cancels
    // near convergence, which plain float does not survive.
    float rr = (float)rr0;
    int coarse_ok = 0;
    if (coarse) {
      // The coarse inverse is the preconditioner's only: the PCG solves the
      // same system to the same tolerance with any of them.  So the previous
      // iteration's inverse is kept while the last accepted step was below
      // coarse_reuse of |x| (the orthogonality blocks, the only part of the
      // coarse matrix that depends on x, have barely moved) and the last PCG
      // took at most 1.5 times the iterations of the last one run with a
      // fresh inverse.  Every CTA takes the same decision (the norms are the
      // same bits everywhere).
      fresh = !(inv_held && inv_ok && step_prev < (double)P.coarse_reuse * normv_prev &&
                2 * pcg_prev <= 3 * pcg_fresh);
      // coarse matrix at this x: fixed kernels + current orthogonality blocks
      const double* rot_now = P.rotagg + (it & 1) * 81 * P.NA;
      double* rot_next = P.rotagg + ((it + 1) & 1) * 81 * P.NA;
      const size_t NC2 = (size_t)P.NC * P.NC;
      if (fresh)
        for (size_t e = gt; e < NC2; e += nt) P.Cw[e] = coarse_entry_x(P, rot_now, (int)(e / P.NC), (int)(e % P.NC));
      for (int e = gt; e < 81 * P.NA; e += nt) rot_next[e] = 0.0;
      if (!gs.sync()) return;
      if (fresh) {
        if (threadIdx.x == 0) s_clk.inv0 = global_ns();
        if (!coarse_invert(P, gs, &coarse_ok, s_scratch)) return;
        if (threadIdx.x == 0) s_clk.acc[5] += (double)(global_ns() - s_clk.inv0);
        inv_held = 1;
        inv_ok = coarse_ok;
        ++n_inv;
      } else {
        coarse_ok = inv_ok;
      }
      // a pivot of the coarse inversion that is not positive: this
      // iteration's PCG runs with block-Jacobi alone; counted in the stats
      if (!coarse_ok && gt == 0) P.stats[ST_CFALL] += 1.0;
      if (resident) {
        // this CTA's rows of the coarse inverse (rows bid, bid + nbk, ...)
        const int NC = P.NC, n4 = NC / 4;
        for (int e = threadIdx.x; e < s_stg.nrows * n4; e += blockDim.x) {
          const int j = e / n4, q = e - j * n4;
          reinterpret_cast<float4*>(stg_crow(j, NC))[q] =
              __ldcg(reinterpret_cast<const float4*>(P.Cinv + (size_t)(bid + j * nbk) * NC) + q);
        }
        __syncthreads();
      }
      lap(2);
    }
    const float tol2 = (float)((double)P.pcg_tol * (double)P.pcg_tol * rr0);
    const int half = lane >> 4, l16 = lane & 15;
    // products: u = u_f + P zc (formed on the fly for every node a product
    // touches), w = (J^T J) u, and gamma = r.u, delta = w.u, r.r in one
    // reduction
    auto products = [&](float2 (&s3)[3]) -> bool {
      float f3[3] = {0.f, 0.f, 0.f};
      work_begin();
      // the coarse correction zc (12 floats per aggregate, shared by its
      // ~64 nodes) is read from a shared-memory copy
      if (coarse) {
        for (int e = threadIdx.x; e < P.NC; e += blockDim.x) s_zc[e] = __ldcg(P.zc + e);
        __syncthreads();
      }
      for (int hs0 = 2 * wib; hs0 * nbk + bid < F; hs0 += 2 * kSolveWarps) {
        const int oi = (hs0 + half) * nbk + bid;
        const bool valid = oi < F;
        // staged or not, for both halves of the warp alike
        const bool stg = hs0 < s_stg.n;
        const int r = valid ? (stg ? stg_node()[hs0 + half].x : __ldg(P.order + oi)) : 0;
        const float rv = (valid && l16 < 12) ? __ldcg(P.r + 12 * (size_t)r + l16) : 0.f;
        float acc[12], uj[12];
        if (stg)
          spmv_node_stg(P, hs0 + half, r, valid, acc, uj);
        else
          spmv_node(P, r, valid, acc, uj);
        if (valid && l16 < 12) {
          float uc = 0.f, wv = 0.f;
#pragma unroll
          for (int i = 0; i < 12; ++i)
            if (i == l16) {
              uc = uj[i];
              wv = acc[i];
            }
          const size_t o = 12 * (size_t)r + l16;
          P.u[o] = uc;
          P.q[o] = wv;
          f3[0] = fmaf(rv, uc, f3[0]);
          f3[1] = fmaf(wv, uc, f3[1]);
          f3[2] = fmaf(rv, rv, f3[2]);
        }
      }
      work_end(0);
      return gs.template reduce_f<3>(f3, s3);
    };
    int cur = 0;  // rc buffer holding P^T r of the current residual
    int pi = 0;
    if (resident) {
      // ---- two-level PCG with the CTA's nodes resident in shared memory and
      // the symmetric two-grid preconditioner (vc_* in solver_device.cuh):
      //   (1) update of own nodes, z1 = D^-1 r; plain barrier
      //   (2) A z1 and the restriction of r - A z1; plain barrier
      //   (3) zc = C^-1 P^T (r - A z1) over the CTA's rows of C^-1; plain barrier
      //   (4) z2 = z1 + P zc, A z2, z3 = D^-1 (r - A z2), u = z2 + z3; plain barrier
      //   (5) A z3, w = A z2 + A z3; gamma, delta, r.r in one reduction
      const int ns = s_stg.n;
      // (J^T J) v of the CTA's nodes (v = slot vector RV_UF here and in P.z):
      // the regularisation rows into RV_W, w_con J_g v of the CTA's constraint
      // items into their staged slots; the first 64 items' loads are issued
      // before the node products so that both take one round trip
      auto full_products = [&]() {
        const int qw = (int)(threadIdx.x >> 3);
        const int ncon = s_stg.ncon;
        GroupLoad G;
        group_issue(P, qw, qw < ncon, G);
        for (int hs0 = 2 * wib; hs0 < ns; hs0 += 2 * kSolveWarps) reg_product_store(P, hs0 + half, hs0 + half < ns, RV_UF);
        group_finish(P, qw, qw < ncon, G);
        for (int c0 = kSolveThreads / 8; c0 < ncon; c0 += kSolveThreads / 8) {
          const int ci = c0 + qw;
          GroupLoad G2;
          group_issue(P, ci, ci < ncon, G2);
          group_finish(P, ci, ci < ncon, G2);
        }
        __syncthreads();
      };
      // vc: the V-cycle; otherwise the additive form D^-1 + P C^-1 P^T on the
      // same phases (restriction of r, no post-smoothing, no phase 5)
      auto apply_m = [&](float2 (&s3)[3], bool vc) -> bool {
        double* rcw = P.rc + cur * P.NC;
        work_begin();
        full_products();
        for (int hs0 = 2 * wib; hs0 < ns; hs0 += 2 * kSolveWarps) vc_restrict(P, hs0 + half, hs0 + half < ns, rcw, vc);
        work_end(2);
        if (!gs.sync()) return false;
        work_begin();
#pragma unroll
        for (int q = 0; q < kRcPerThread; ++q) {
          const int e = threadIdx.x + q * kSolveThreads;
          if (e < P.NC) s_scratch[e] = (float)__ldcg(rcw + e);
        }
        __syncthreads();
        coarse_rows_res(P, bid, nbk, coarse_ok, s_scratch);
        double* rco = P.rc + (cur ^ 1) * P.NC;
        for (int e = gt; e < P.NC; e += nt) rco[e] = 0.0;
        work_end(2);
        if (!gs.sync()) return false;
        work_begin();
        // zc of every coupled aggregate of the CTA's nodes
        for (int e = threadIdx.x; e < 12 * s_stg.nent; e += blockDim.x) {
          const int en = e / 12, i = e - 12 * en;
          stg_zz(en)[i] = __ldcg(P.zc + 12 * stg_mag()[en] + i);
        }
        __syncthreads();
        for (int hs0 = 2 * wib; hs0 < ns; hs0 += 2 * kSolveWarps) vc_precond(P, hs0 + half, hs0 + half < ns, vc);
        float f3[3] = {0.f, 0.f, 0.f};
        if (vc) {
          work_end(1);
          if (!gs.sync()) return false;
          work_begin();
          full_products();
          for (int hs0 = 2 * wib; hs0 < ns; hs0 += 2 * kSolveWarps) vc_finish(P, hs0 + half, hs0 + half < ns, f3);
          work_end(0);
        } else {
          for (int hs0 = 2 * wib; hs0 < ns; hs0 += 2 * kSolveWarps)
            vc_finish_additive(P, hs0 + half, hs0 + half < ns, f3);
          work_end(1);
        }
        cur ^= 1;
        return gs.template reduce_f<3>(f3, s3);
      };
      // The V-cycle is positive definite only while the block-Jacobi smoother
      // converges (rho(D^-1 A) < 2; about 6 on some constraint-centre
      // problems).  A breakdown (gamma or the C-G denominator not positive
      // before convergence; the same bits in every CTA) restarts this step's
      // PCG with the additive form, which is always positive definite.
      for (int vc = 1; vc >= 0; --vc) {
        bool broke = false;
        float2 s3[3];
        if (!apply_m(s3, vc != 0)) return;
        float2 gam = s3[0];
        rr = s3[2].x;
        bool go = rr > tol2 && gam.x > 0.f && s3[1].x > 0.f;
        broke = !go && rr > tol2;
        float2 alpha_d = go ? dd_div(gam, s3[1]) : make_float2(0.f, 0.f);
        float beta = 0.f;
        for (int kk = 0; go && pi < P.pcg_max; ++kk) {
          const float alpha = alpha_d.x;
          work_begin();
          for (int hs0 = 2 * wib; hs0 < ns; hs0 += 2 * kSolveWarps)
            vc_update(P, hs0 + half, hs0 + half < ns, alpha, beta, kk == 0);
          work_end(1);
          if (!gs.sync()) return;
          ++pi;
          if (!apply_m(s3, vc != 0)) return;
          rr = s3[2].x;
          if (rr <= tol2 || pi >= P.pcg_max) break;
          const float2 gam_new = s3[0];
          if (!(gam_new.x > 0.f)) {
            broke = true;
            break;
          }
          const float2 bd = dd_div(gam_new, gam);
          const float2 den = dd_sub(s3[1], dd_div(dd_mul(bd, gam_new), alpha_d));
          if (!(den.x > 0.f)) {
            broke = true;
            break;
          }
          beta = bd.x;
          alpha_d = dd_div(gam_new, den);
          gam = gam_new;
        }
        if (!broke || !vc) break;
        for (int hs0 = 2 * wib; hs0 < ns; hs0 += 2 * kSolveWarps) vc_restart(P, hs0 + half, hs0 + half < ns);
        if (!gs.sync()) return;
      }
    } else {
    if (coarse) {
      work_begin();
      coarse_solve(P, gs, P.rc, P.rc + P.NC, coarse_ok, s_scratch);
      work_end(2);
      if (!gs.sync()) return;
    }
    float2 s3[3];
    if (!products(s3)) return;
    float2 gam = s3[0];
    rr = s3[2].x;
    bool go = rr > tol2 && gam.x > 0.f && s3[1].x > 0.f;
    float2 alpha_d = go ? dd_div(gam, s3[1]) : make_float2(0.f, 0.f);
    float beta = 0.f;
    while (go && pi < P.pcg_max) {
      const float alpha = alpha_d.x;
      // p = u + beta p, s = w + beta s (s = (J^T J) p), h += alpha p,
      // r -= alpha s, u_f = Dinv r and its restriction
      const bool first = pi == 0;
      double* rc_next = P.rc + (cur ^ 1) * P.NC;
      work_begin();
      for (int hs0 = 2 * wib; hs0 * nbk + bid < F; hs0 += 2 * kSolveWarps) {
        const int oi = (hs0 + half) * nbk + bid;
        const bool valid = oi < F;
        const bool stg = hs0 < s_stg.n;
        const int r = valid ? (stg ? stg_node()[hs0 + half].x : __ldg(P.order + oi)) : 0;
        float rv = 0.f;
        if (valid && l16 < 12) {
          const size_t o = 12 * (size_t)r + l16;
          const float uo = __ldcg(P.u + o), wo = __ldcg(P.q + o);
          const float pn = first ? uo : fmaf(beta, __ldcg(P.p0 + o), uo);
          const float sn = first ? wo : fmaf(beta, __ldcg(P.p1 + o), wo);
          P.p0[o] = pn;
          P.p1[o] = sn;
          P.h[o] = fmaf(alpha, pn, __ldcg(P.h + o));
          rv = fmaf(-alpha, sn, __ldcg(P.r + o));
          P.r[o] = rv;
        }
        const float zv = stg ? apply_dinv_h_stg(hs0 + half, valid, rv) : apply_dinv_h(P, r, valid, rv);
        if (coarse) {
          if (stg)
            coarse_restrict_h_stg(hs0 + half, valid, rv, rc_next);
          else
            coarse_restrict_h(P, r, valid, rv, rc_next);
        }
        if (valid && l16 < 12) P.z[12 * (size_t)r + l16] = zv;
      }
      work_end(1);
      if (!gs.sync()) return;
      ++pi;
      cur ^= 1;
      if (coarse) {
        work_begin();
        coarse_solve(P, gs, P.rc + cur * P.NC, P.rc + (cur ^ 1) * P.NC, coarse_ok, s_scratch);
        work_end(2);
        if (!gs.sync()) return;
      }
      if (!products(s3)) return;
      rr = s3[2].x;
      if (rr <= tol2 || pi >= P.pcg_max) break;
      const float2 gam_new = s3[0];
      if (!(gam_new.x > 0.f)) break;
      const float2 bd = dd_div(gam_new, gam);
      const float2 den = dd_sub(s3[1], dd_div(dd_mul(bd, gam_new), alpha_d));
      if (!(den.x > 0.f)) break;
      beta = bd.x;
      alpha_d = dd_div(gam_new, den);
      gam = gam_new;
    }
    }
    // both restriction buffers start the next gradient pass at zero
    if (coarse)
      for (int e = gt; e < 2 * P.NC; e += nt) P.rc[e] = 0.0;
    pcg_total += pi;
    pcg_prev = pi;
    if (fresh) pcg_fresh = pi;
    work_flush();
    lap(3);

    // ---- line search: x + 2^-m h, m = 0..49 (Deform.cpp:144-156)
    RT scale = RT(1);
    bool accepted = false;
    double hh = 0.0;
    for (int ls = 0; ls < 50; ++ls) {
      double en2[2] = {0.0, 0.0};
      for (int ws = wib; ws * nbk + bid < F; ws += kSolveWarps) {
        const int r = __ldg(P.order + ws * nbk + bid);
        RT g_unused;
        float Q[10];
        double en;
        residual_node<RT, PASS_ENERGY>(P, r, scale, g_unused, Q, en);
        if (lane == 0) en2[0] += en;
      }
      for (int g = gw; g < P.G; g += nw) {
        RT f[3];
        con_residual_warp<RT>(P, g, scale, f);
        if (lane == 0)
          en2[0] += double(f[0]) * double(f[0]) + double(f[1]) * double(f[1]) + double(f[2]) * double(f[2]);
      }
      if (ls == 0) {
        for (int e = gt; e < F * 12; e += nt) {
          const double v = __ldcg(P.h + e);
          en2[1] += v * v;
        }
      }
      if (!gs.template reduce<2>(en2)) return;
      if (ls == 0) hh = en2[1];
      if (en2[0] > e_old) {
        scale *= RT(0.5);
        ++halvings;
      } else {
        accepted = true;
        e_last = en2[0];
        break;
      }
    }
    if (accepted) {
      for (int e = gt; e < F * 12; e += nt) {
        const double v = __ldcg(P.x + e) + (double)scale * (double)__ldcg(P.h + e);
        P.x[e] = v;
        P.xf[e] = (float)v;
        put_xo(P, e, v);
      }
    }
    const double normh = (double)scale * sqrt(hh);
    step_prev = normh;
    normv_prev = normv;
    if (gt == 0 && it < kHalvIters) P.stats[ST_HALV_IT + it] = halvings;
    iters = it + 1;
    if (!gs.sync()) return;
    lap(4);
    if (P.early_exit && normh < (normv + 1e-6) * 1e-6) {
      converged = 1;
      break;
    }
  }

  // ---- putFreeInputs / resetRT: node transforms for every node
  int nonfinite = 0;
  for (int node = gt; node < P.n; node += nt) {
    const int rk = P.rank[node];
    float* ro = P.rot_out + 9 * (size_t)node;
    float* to = P.trans_out + 3 * (size_t)node;
    if (rk >= 0) {
      const double* xp = P.x + 12 * (size_t)rk;
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        const double v = __ldcg(xp + i);
        ro[i] = (float)v;
        if (!isfinite(v)) nonfinite = 1;
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const double v = __ldcg(xp + 9 + i);
        to[i] = (float)v;
        if (!isfinite(v)) nonfinite = 1;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 9; ++i) ro[i] = (i == 0 || i == 4 || i == 8) ? 1.f : 0.f;
      to[0] = to[1] = to[2] = 0.f;
    }
  }
  if (nonfinite) raise_status(&P.bar->status, ARAP_ENONFINITE);
  if (gt == 0) {
    P.stats[ST_ITERS] = iters;
    P.stats[ST_PCG] = pcg_total;
    P.stats[ST_CINV_N] = n_inv;
    P.stats[ST_HALV] = halvings;
    P.stats[ST_E0] = e_first;
    P.stats[ST_E] = e_last;
    P.stats[ST_CONV] = converged;
    for (int q = 0; q < 6; ++q) P.stats[ST_T_PREP + q] = s_clk.acc[q];
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q)
      atomicMax(reinterpret_cast<unsigned long long*>(P.stats + ST_T_W_SPMV + q),
                (unsigned long long)__double_as_longlong((double)s_clk.work[q]));
}

template <typename RT>
__global__ void __launch_bounds__(kSolveThreads) gn_solve_kernel(SolveParams P) {
  solve_body<RT, false>(P, blockIdx.x, gridDim.x);
}

// Batched solves: CTAs cta_first[i] .. cta_first[i+1]-1 of the cooperative
// grid run instance i with their own barrier; the instance's parameters are
// copied into shared memory.  Its barrier waits take each instance's
// configured spin limit, so a single solver with a spin limit of its own runs
// here as a batch of one.
template <typename RT>
__global__ void __launch_bounds__(kSolveThreads)
    gn_solve_batch_kernel(const SolveParams* __restrict__ params, const int* __restrict__ cta_first, int count) {
  __shared__ SolveParams s_P;
  __shared__ int s_inst;
  if (threadIdx.x == 0) {
    int i = 0;
    while (i + 1 < count && cta_first[i + 1] <= (int)blockIdx.x) ++i;
    s_inst = i;
  }
  __syncthreads();
  const int i = s_inst;
  {
    const int* src = reinterpret_cast<const int*>(params + i);
    int* dst = reinterpret_cast<int*>(&s_P);
    for (int q = threadIdx.x; q < (int)(sizeof(SolveParams) / sizeof(int)); q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  solve_body<RT, true>(s_P, (int)blockIdx.x - cta_first[i], cta_first[i + 1] - cta_first[i]);
}

}  // namespace arap
