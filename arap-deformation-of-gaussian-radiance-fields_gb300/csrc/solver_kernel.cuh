// The persistent Gauss-Newton kernel: one cooperative launch runs the whole
// Deform::optimize loop (Deform.cpp:95-169) -- gradient and energy, block
// preconditioner, PCG for (J^T J) h = -J^T f, halving line search, stop test
// -- and writes the node transforms (Deform.hpp:140-151).
#pragma once

#include "solver_device.cuh"

namespace arap {

// stats slots written by CTA 0; ST_T_* are nanoseconds spent in each phase
// (global timer, read by thread 0 of CTA 0 after the phase's barrier)
enum {
  ST_ITERS = 0, ST_PCG = 1, ST_HALV = 2, ST_E0 = 3, ST_E = 4, ST_CONV = 5, ST_NONFINITE = 6,
  ST_T_PREP = 8, ST_T_GRAD = 9, ST_T_COARSE = 10, ST_T_PCG = 11, ST_T_LS = 12
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <int N>
__device__ __forceinline__ bool reduce_all(const SolveParams& P, double (&v)[N], double (&out)[N]) {
  block_sum<N>(v);
  return grid_sync_reduce<N>(P.bar, P.partials, P.results, v, out);
}

// Inverse of the coarse matrix in Cw[0] by blocked Gauss-Jordan (float32, no
// pivoting: the matrix is symmetric positive definite).  For each pivot block
// K: CTA 0 inverts A_KK in shared memory; every CTA forms W = A_:K A_KK^-1;
// then A_KK <- A_KK^-1, A_Kj <- A_KK^-1 A_Kj, A_iK <- -W_iK,
// A_ij <- A_ij - W_iK A_Kj.  Three grid barriers per block.  Returns false on a
// barrier failure; *ok = 0 when a pivot block was not positive definite.
__device__ bool coarse_invert(const SolveParams& P, int* ok) {
  __shared__ float s_piv[kGJBlock][kGJBlock + 1];
  __shared__ float s_row[kGJBlock], s_col[kGJBlock];
  __shared__ int s_bad;
  const int NC = P.NC;
  const size_t NC2 = (size_t)NC * NC;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = gridDim.x * blockDim.x;
  int src_i = 0;
  *ok = 1;
  for (int K0 = 0; K0 < NC; K0 += kGJBlock) {
    const int kb = min(kGJBlock, NC - K0);
    const float* src = P.Cw + src_i * NC2;
    float* dst = P.Cw + (1 - src_i) * NC2;
    const bool last = K0 + kb >= NC;
    double bad[1] = {0.0}, obad[1];
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) s_bad = 0;
      for (int t = threadIdx.x; t < kb * kb; t += blockDim.x)
        s_piv[t / kb][t % kb] = __ldcg(src + (size_t)(K0 + t / kb) * NC + K0 + t % kb);
      for (int m = 0; m < kb; ++m) {
        __syncthreads();
        if (threadIdx.x < kb) {
          s_row[threadIdx.x] = s_piv[m][threadIdx.x];
          s_col[threadIdx.x] = s_piv[threadIdx.x][m];
        }
        __syncthreads();
        const float pv = s_row[m];
        if (!(pv > 0.f)) {
          if (threadIdx.x == 0) s_bad = 1;
          continue;
        }
        const float ip = 1.f / pv;
        for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
          const int i = t / kb, j = t % kb;
          float v;
          if (i == m && j == m)
            v = ip;
          else if (i == m)
            v = s_row[j] * ip;
          else if (j == m)
            v = -s_col[i] * ip;
          else
            v = s_piv[i][j] - s_col[i] * s_row[j] * ip;
          s_piv[i][j] = v;
        }
      }
      __syncthreads();
      for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) P.Pgj[t] = s_piv[t / kb][t % kb];
      bad[0] = s_bad;
    }
    if (!grid_sync_reduce<1>(P.bar, P.partials, P.results, bad, obad)) return false;
    if (obad[0] != 0.0) *ok = 0;
    for (size_t e = gt; e < (size_t)NC * kb; e += nt) {
      const int i = (int)(e / kb), n = (int)(e % kb);
      if (i >= K0 && i < K0 + kb) continue;
      float w = 0.f;
      for (int m = 0; m < kb; ++m) w = fmaf(__ldcg(src + (size_t)i * NC + K0 + m), __ldcg(P.Pgj + m * kb + n), w);
      P.Wgj[(size_t)i * kb + n] = w;
    }
    double d0[1] = {0.0}, o0[1];
    if (!grid_sync_reduce<1>(P.bar, P.partials, P.results, d0, o0)) return false;
    for (size_t e = gt; e < NC2; e += nt) {
      const int i = (int)(e / NC), j = (int)(e % NC);
      const int iK = i - K0, jK = j - K0;
      const bool inI = iK >= 0 && iK < kb, inJ = jK >= 0 && jK < kb;
      float v;
      if (inI && inJ) {
        v = __ldcg(P.Pgj + iK * kb + jK);
      } else if (inI) {
        v = 0.f;
        for (int m = 0; m < kb; ++m) v = fmaf(__ldcg(P.Pgj + iK * kb + m), __ldcg(src + (size_t)(K0 + m) * NC + j), v);
      } else if (inJ) {
        v = -__ldcg(P.Wgj + (size_t)i * kb + jK);
      } else {
        v = __ldcg(src + e);
        for (int m = 0; m < kb; ++m) v = fmaf(-__ldcg(P.Wgj + (size_t)i * kb + m), __ldcg(src + (size_t)(K0 + m) * NC + j), v);
      }
      if (last)
        P.Cinv[e] = v;
      else
        dst[e] = v;
    }
    if (!grid_sync_reduce<1>(P.bar, P.partials, P.results, d0, o0)) return false;
    src_i ^= 1;
  }
  return true;
}

// zc = Cinv rc (one warp per row), zero the other restriction buffer, and
// this thread's share of rc . zc.
__device__ __forceinline__ bool coarse_solve(const SolveParams& P, const double* rc, double* rc_other,
                                             double (&part)[1], int ok) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int NC = P.NC;
  for (int i = gw; i < NC; i += nw) {
    double acc = 0.0;
    const float* row = P.Cinv + (size_t)i * NC;
    if (ok)
      for (int j = lane; j < NC; j += 32) acc += (double)__ldcg(row + j) * __ldcg(rc + j);
    acc = warp_sum(acc);
    if (lane == 0) {
      P.zc[i] = (float)acc;
      part[0] += __ldcg(rc + i) * acc;
    }
  }
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < NC; e += gridDim.x * blockDim.x) rc_other[e] = 0.0;
  return true;
}

template <typename RT>
__global__ void __launch_bounds__(kSolveThreads) gn_solve_kernel(SolveParams P) {
  __shared__ float s_D[kSolveWarps][144];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = gridDim.x * blockDim.x;
  const int F = P.F, k = P.k;
  unsigned long long t_mark = global_ns();
  double t_acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // prep, grad, coarse, pcg, line search
  auto lap = [&](int slot) {
    const unsigned long long now = global_ns();
    t_acc[slot] += (double)(now - t_mark);
    t_mark = now;
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
  }
  const bool coarse = P.NA > 0 && P.mode == 0;
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
  }
  {
    double d0[1] = {0.0}, o0[1];
    if (!grid_sync_reduce<1>(P.bar, P.partials, P.results, d0, o0)) return;
  }
  if (coarse) {
    // coarse matrix P^T (J^T J at x = I) P, fixed for this solve
    for (int oi = gw; oi < F; oi += nw) coarse_rows_node(P, __ldg(P.order + oi));
    for (int g = gt; g < P.G; g += nt) coarse_rows_group(P, g);
    double d0[1] = {0.0}, o0[1];
    if (!grid_sync_reduce<1>(P.bar, P.partials, P.results, d0, o0)) return;
  }

  lap(0);
  double e_first = 0.0, e_last = 0.0;
  int iters = 0, pcg_total = 0, halvings = 0, converged = 0;
  for (int it = 0; it < P.max_iters; ++it) {
    // ---- gradient -J^T f, energy, preconditioner, PCG start (h=0, r=g, z=M^-1 g)
    double red[4] = {0.0, 0.0, 0.0, 0.0}, out[4];
    for (int oi = gw; oi < F; oi += nw) {
      const int r = __ldg(P.order + oi);
      RT acc[12];
      float Q[10];
      double en;
      residual_node<RT, PASS_GRAD>(P, r, RT(0), acc, Q, en);
      if (lane == 0) red[0] += en;
      if (P.mode == 1) {
        if (lane < 12) {
          double a = 0.0;
#pragma unroll
          for (int i = 0; i < 12; ++i)
            if (i == lane) a = (double)acc[i];
          P.grad_out[12 * (size_t)r + lane] = a;
        }
        continue;
      }
      build_dinv(P, r, Q, s_D[wib]);
      if (coarse) coarse_rot_node(P, r, P.rotagg + (it & 1) * 81 * P.NA);
      float gc = 0.f;
#pragma unroll
      for (int i = 0; i < 12; ++i)
        if (i == lane) gc = -(float)acc[i];
      const float zc = apply_dinv(P, r, gc);
      if (coarse) coarse_restrict(P, r, gc, P.rc);
      if (lane < 12) {
        const size_t o = 12 * (size_t)r + lane;
        P.g[o] = gc;
        P.r[o] = gc;
        P.z[o] = zc;
        P.h[o] = 0.f;
        red[2] += (double)gc * (double)zc;
        red[3] += (double)gc * (double)gc;
      }
    }
    for (int g = gt; g < P.G; g += nt) {
      RT f[3];
      con_residual<RT>(P, g, RT(0), f);
      red[0] += double(f[0]) * double(f[0]) + double(f[1]) * double(f[1]) + double(f[2]) * double(f[2]);
    }
    for (int e = gt; e < F * 12; e += nt) {
      const double v = __ldcg(P.x + e);
      red[1] += v * v;
    }
    if (!reduce_all<4>(P, red, out)) return;
    lap(1);
    const double e_old = out[0];
    const double normv = sqrt(out[1]);
    if (it == 0) e_first = e_old;
    e_last = e_old;
    if (P.mode == 1) {
      if (gt == 0) P.stats[ST_E] = e_old;
      return;
    }

    // ---- PCG on (J^T J) h = g: two barriers per iteration, plus one for the
    // coarse solve when the two-level preconditioner is on
    double rz = out[2];
    const double rr0 = out[3];
    double rr = rr0;
    int coarse_ok = 0;
    if (coarse) {
      // coarse matrix at this x: fixed kernels + current orthogonality blocks
      const double* rot_now = P.rotagg + (it & 1) * 81 * P.NA;
      double* rot_next = P.rotagg + ((it + 1) & 1) * 81 * P.NA;
      const size_t NC2 = (size_t)P.NC * P.NC;
      for (size_t e = gt; e < NC2; e += nt) P.Cw[e] = coarse_entry_x(P, rot_now, (int)(e / P.NC), (int)(e % P.NC));
      for (int e = gt; e < 81 * P.NA; e += nt) rot_next[e] = 0.0;
      double d0[1] = {0.0}, o0[1];
      if (!grid_sync_reduce<1>(P.bar, P.partials, P.results, d0, o0)) return;
      if (!coarse_invert(P, &coarse_ok)) return;
      if (!coarse_ok && gt == 0) raise_status(ARAP_ENONFINITE);
      lap(2);
    }
    if (coarse) {
      double rzc[1] = {0.0}, orc[1];
      if (!coarse_solve(P, P.rc, P.rc + P.NC, rzc, coarse_ok)) return;
      if (!reduce_all<1>(P, rzc, orc)) return;
      rz += orc[0];
    }
    const double tol2 = (double)P.pcg_tol * (double)P.pcg_tol * rr0;
    float beta = 0.f;
    int pi = 0;
    const int half = lane >> 4, l16 = lane & 15;
    const int nhw = 2 * nw;
    while (rr > tol2 && pi < P.pcg_max && rz > 0.0) {
      const bool first = pi == 0;
      float* pcur = (pi & 1) ? P.p1 : P.p0;
      const float* pold = (pi & 1) ? P.p0 : P.p1;
      double pq[1] = {0.0}, opq[1];
      for (int base = 2 * gw; base < F; base += nhw) {
        const int oi = base + half;
        const bool valid = oi < F;
        const int r = valid ? __ldg(P.order + oi) : 0;
        float acc[12], pj[12];
        spmv_node(P, r, valid, first, beta, pold, acc, pj);
        if (valid && l16 < 12) {
          float pc = 0.f, qc = 0.f;
#pragma unroll
          for (int i = 0; i < 12; ++i)
            if (i == l16) {
              pc = pj[i];
              qc = acc[i];
            }
          const size_t o = 12 * (size_t)r + l16;
          pcur[o] = pc;
          P.q[o] = qc;
          pq[0] += (double)pc * (double)qc;
        }
      }
      if (!reduce_all<1>(P, pq, opq)) return;
      if (!(opq[0] > 0.0)) break;
      const float alpha = (float)(rz / opq[0]);
      double* rc_next = P.rc + ((pi + 1) & 1) * P.NC;
      double rzr[2] = {0.0, 0.0}, orz[2];
      for (int base = 2 * gw; base < F; base += nhw) {
        const int oi = base + half;
        const bool valid = oi < F;
        const int r = valid ? __ldg(P.order + oi) : 0;
        float rc = 0.f;
        if (valid && l16 < 12) {
          const size_t o = 12 * (size_t)r + l16;
          P.h[o] = fmaf(alpha, __ldcg(pcur + o), __ldcg(P.h + o));
          rc = fmaf(-alpha, __ldcg(P.q + o), __ldcg(P.r + o));
          P.r[o] = rc;
        }
        const float zc = apply_dinv_h(P, r, valid, rc);
        if (coarse) coarse_restrict_h(P, r, valid, rc, rc_next);
        if (valid && l16 < 12) {
          P.z[12 * (size_t)r + l16] = zc;
          rzr[0] += (double)rc * (double)zc;
          rzr[1] += (double)rc * (double)rc;
        }
      }
      if (!reduce_all<2>(P, rzr, orz)) return;
      ++pi;
      rr = orz[1];
      if (rr <= tol2 || pi >= P.pcg_max) break;
      double rz_new = orz[0];
      if (coarse) {
        double rzc[1] = {0.0}, orc[1];
        if (!coarse_solve(P, rc_next, P.rc + (pi & 1 ? 0 : 1) * P.NC, rzc, coarse_ok)) return;
        if (!reduce_all<1>(P, rzc, orc)) return;
        rz_new += orc[0];
      }
      beta = (float)(rz_new / rz);
      rz = rz_new;
    }
    pcg_total += pi;
    lap(3);

    // ---- line search: x + 2^-m h, m = 0..49 (Deform.cpp:144-156)
    RT scale = RT(1);
    bool accepted = false;
    double hh = 0.0;
    for (int ls = 0; ls < 50; ++ls) {
      double en2[2] = {0.0, 0.0}, oen[2];
      for (int oi = gw; oi < F; oi += nw) {
      const int r = __ldg(P.order + oi);
        RT acc[12];
        float Q[10];
        double en;
        residual_node<RT, PASS_ENERGY>(P, r, scale, acc, Q, en);
        if (lane == 0) en2[0] += en;
      }
      for (int g = gt; g < P.G; g += nt) {
        RT f[3];
        con_residual<RT>(P, g, scale, f);
        en2[0] += double(f[0]) * double(f[0]) + double(f[1]) * double(f[1]) + double(f[2]) * double(f[2]);
      }
      if (ls == 0) {
        for (int e = gt; e < F * 12; e += nt) {
          const double v = __ldcg(P.h + e);
          en2[1] += v * v;
        }
      }
      if (!reduce_all<2>(P, en2, oen)) return;
      if (ls == 0) hh = oen[1];
      if (oen[0] > e_old) {
        scale *= RT(0.5);
        ++halvings;
      } else {
        accepted = true;
        e_last = oen[0];
        break;
      }
    }
    if (accepted) {
      for (int e = gt; e < F * 12; e += nt) {
        const double v = __ldcg(P.x + e) + (double)scale * (double)__ldcg(P.h + e);
        P.x[e] = v;
        P.xf[e] = (float)v;
      }
    }
    const double normh = (double)scale * sqrt(hh);
    iters = it + 1;
    {
      double d0[1] = {0.0}, o0[1];
      if (!reduce_all<1>(P, d0, o0)) return;
    }
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
  if (nonfinite) raise_status(ARAP_ENONFINITE);
  if (gt == 0) {
    P.stats[ST_ITERS] = iters;
    P.stats[ST_PCG] = pcg_total;
    P.stats[ST_HALV] = halvings;
    P.stats[ST_E0] = e_first;
    P.stats[ST_E] = e_last;
    P.stats[ST_CONV] = converged;
    for (int q = 0; q < 5; ++q) P.stats[ST_T_PREP + q] = t_acc[q];
  }
}

}  // namespace arap
