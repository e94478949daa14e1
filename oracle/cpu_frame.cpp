// CPU baseline of the deformation frame: a C++/OpenMP FP64 restatement of the
// reference's CPU path, used as the timed CPU baseline and as a second oracle.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
// legs of bench.py load this library; the product (libarap_gb300.so) never
// does.  Parity unpinned against executed reference code (the reference needs
// Eigen 3 and SIBR, which are not installed); it is checked against the numpy
// oracle (oracle/ed.py, oracle/skin.py) on the same inputs.
//
// What it restates (reference paths relative to the project):
//   Deform bookkeeping        Deform.hpp:414-455, Deform.cpp:6-75
//   residual CalcEnergyFunc   Deform.cpp:378-581
//   Jacobian FastCalcJacobiMat Deform.cpp:180-376 (CSR rows; duplicates summed
//                             as setFromTriplets does)
//   optimize                  Deform.cpp:95-169: J^T J, g = -J^T f, a direct
//                             sparse Cholesky solve, halving line search,
//                             optional early exit
//   ED blend                  Deform.hpp:230-249 (float accumulation)
//   UpdatePosition / UpdatePositionforSamples   GaussianView.cpp:2986-3077
//   UpdateAsSixPointsWithdrawBad + getOthogonalMatrixWithK
//                             GaussianView.cpp:3081-3166, helper.cpp:429-440
//   FastUpdateSamplesSH + RotateSHs  GaussianView.cpp:3169-3186,
//                             helper.cpp:506-517, cudakdtree.cu:113-222
//
// The sparse solve stands in for Eigen's SimplicialCholesky (Deform.cpp:
// 103-133), which is not available here.  It is a block Cholesky L L^T over
// the 12 unknowns of each free node: a minimum-degree ordering of the node
// graph of J^T J, a node-level elimination tree and column structures, and a
// left-looking numeric factorisation on dense 12x12 blocks.  Independent
// subtrees of the elimination tree are factorised in parallel; the top of the
// tree is factorised column by column with the column's updates split over
// the threads.  The reference analyses the pattern and factorises twice per
// Gauss-Newton iteration (solver.compute, then solver.factorize); this
// restatement orders and analyses once per solve and factorises once per
// iteration, so its time is a lower bound on that work.
//
// The 3x3 polar split uses a one-sided Jacobi SVD (Hestenes 1958) in FP64;
// R = U V^T and K = diag(V S V^T) do not depend on which SVD algorithm is
// used for a nonsingular M.  SH bands 1-3 are rotated with the Ivanic-
// Ruedenberg recurrence (J. Phys. Chem. 100 (1996) 6342).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <queue>
#include <vector>

#include <omp.h>

namespace {

using Clock = std::chrono::steady_clock;
double secs(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

// ------------------------------------------------------------ problem ----

struct Problem {
  int n = 0, k = 0, F = 0, S = 0;
  const float* g = nullptr;       // [n][3]
  const int32_t* nb = nullptr;    // [n][k]
  const int32_t* aidx = nullptr;  // [n][k]
  const double* aw = nullptr;     // [n][k]
  const float* aims = nullptr;    // [n][3]
  std::vector<int> free_ids, static_ids, rank;
  std::vector<double> reg_scale;  // [F][k]
  bool center = false;
  std::vector<int> ctrl_nodes;                    // non-centre mode
  std::vector<std::vector<int>> center_sets;      // centre mode
  std::vector<float> center_aims;                 // [sets][3]
  double sw_rot = 1, sw_reg = 1, sw_con = 1;
  long long n_rows = 0;
  int rows_rot = 0;
  long long rows_reg = 0, rows_sta = 0;
};

// Deform.hpp:414-455, Deform.cpp:6-75, GaussianView.cpp:2010-2035.
int make_problem(Problem& P, int n, int k, const float* node_pos, const int32_t* nbr, const int32_t* aidx,
                 const double* aw, const float* aims, int n_blocks, const int32_t* block_ptr,
                 const int32_t* block_ids, const int32_t* block_type, int cons_on_center, float weighting_factor,
                 float w_rot, float w_reg, float w_con) {
  P.n = n;
  P.k = k;
  P.g = node_pos;
  P.nb = nbr;
  P.aidx = aidx;
  P.aw = aw;
  P.aims = aims;
  std::vector<char> is_static(n, 0);
  for (int b = 0; b < n_blocks; ++b)
    if (block_type[b] < 0)
      for (int t = block_ptr[b]; t < block_ptr[b + 1]; ++t) {
        const int v = block_ids[t];
        if (v < 0 || v >= n) return 3;
        is_static[v] = 1;
      }
  P.rank.assign(n, -1);
  for (int v = 0; v < n; ++v) {
    if (is_static[v]) {
      P.static_ids.push_back(v);
    } else {
      P.rank[v] = (int)P.free_ids.size();
      P.free_ids.push_back(v);
    }
  }
  P.F = (int)P.free_ids.size();
  P.S = (int)P.static_ids.size();
  // BelongsToSameBlock skips blocks of type -1 (Deform.cpp:20-32)
  std::vector<std::vector<char>> memb;
  for (int b = 0; b < n_blocks; ++b) {
    if (block_type[b] == -1) continue;
    std::vector<char> m(n, 0);
    for (int t = block_ptr[b]; t < block_ptr[b + 1]; ++t) m[block_ids[t]] = 1;
    memb.push_back(std::move(m));
  }
  const double wf = (double)weighting_factor;
  P.reg_scale.assign((size_t)P.F * k, 1.0);
  for (int f = 0; f < P.F; ++f)
    for (int j = 0; j < k; ++j) {
      const int a = P.free_ids[f], c = nbr[(size_t)a * k + j];
      bool same = false;
      for (auto& m : memb) same = same || (m[a] && m[c]);
      if (same) P.reg_scale[(size_t)f * k + j] = wf;
    }
  P.center = cons_on_center != 0;
  int n_ctrl_rows = 0;
  if (P.center) {
    // SelectKeyControls (Deform.cpp:34-75): the set of the first min(20, |b|)
    // ids; the centre aim is the float mean of their aims
    for (int b = 0; b < n_blocks; ++b) {
      if (block_type[b] == -1) continue;
      const int sz = block_ptr[b + 1] - block_ptr[b];
      const int m = std::min(20, sz);
      std::vector<int> s(block_ids + block_ptr[b], block_ids + block_ptr[b] + m);
      float c[3] = {0.f, 0.f, 0.f};
      for (int t = 0; t < m; ++t)
        for (int d = 0; d < 3; ++d) c[d] = c[d] + aims[3 * (size_t)s[t] + d];
      std::sort(s.begin(), s.end());
      s.erase(std::unique(s.begin(), s.end()), s.end());
      P.center_sets.push_back(s);
      for (int d = 0; d < 3; ++d) P.center_aims.push_back(c[d] / (float)m);
    }
    n_ctrl_rows = 3 * (int)P.center_sets.size();
  } else {
    for (int b = 0; b < n_blocks; ++b)
      if (block_type[b] != -1)
        for (int t = block_ptr[b]; t < block_ptr[b + 1]; ++t) P.ctrl_nodes.push_back(block_ids[t]);
    n_ctrl_rows = 3 * (int)P.ctrl_nodes.size();
  }
  P.sw_rot = std::sqrt((double)w_rot);
  P.sw_reg = std::sqrt((double)w_reg);
  P.sw_con = std::sqrt((double)w_con);
  P.rows_rot = 6 * P.F;
  P.rows_reg = 3LL * P.F * k;
  P.rows_sta = 3LL * P.S * k;
  P.n_rows = P.rows_rot + P.rows_reg + P.rows_sta + n_ctrl_rows;
  return 0;
}

inline void rmul(const double* X, const double v[3], double out[3]) {  // R v, R column-major in X[0:9]
  for (int r = 0; r < 3; ++r) out[r] = X[r] * v[0] + X[3 + r] * v[1] + X[6 + r] * v[2];
}

// sum_j w_cj (R_j (v_c - g_j) + g_j + t_j) over the anchor kNN (free j);
// w_cj v_c for a static j (Deform.cpp:540-573).
void blend_constraint(const Problem& P, const double* x, int c, double nv[3]) {
  const int k = P.k;
  const double ve[3] = {P.g[3 * (size_t)c], P.g[3 * (size_t)c + 1], P.g[3 * (size_t)c + 2]};
  nv[0] = nv[1] = nv[2] = 0.0;
  for (int j = 0; j < k; ++j) {
    const int a = P.aidx[(size_t)c * k + j];
    const double w = P.aw[(size_t)c * k + j];
    const int r = P.rank[a];
    double term[3];
    if (r >= 0) {
      const double* X = x + 12 * (size_t)r;
      const double gj[3] = {P.g[3 * (size_t)a], P.g[3 * (size_t)a + 1], P.g[3 * (size_t)a + 2]};
      const double d[3] = {ve[0] - gj[0], ve[1] - gj[1], ve[2] - gj[2]};
      double m[3];
      rmul(X, d, m);
      for (int q = 0; q < 3; ++q) term[q] = m[q] + gj[q] + X[9 + q];
    } else {
      for (int q = 0; q < 3; ++q) term[q] = ve[q];
    }
    for (int q = 0; q < 3; ++q) nv[q] += w * term[q];
  }
}

// CalcEnergyFunc (Deform.cpp:378-581).
void residual(const Problem& P, const double* x, double* f) {
  const int F = P.F, k = P.k;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < F; ++i) {
    const double* X = x + 12 * (size_t)i;
    const double *c0 = X, *c1 = X + 3, *c2 = X + 6;
    auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    double* r = f + 6 * (size_t)i;
    r[0] = P.sw_rot * dot(c0, c1);
    r[1] = P.sw_rot * dot(c0, c2);
    r[2] = P.sw_rot * dot(c1, c2);
    r[3] = P.sw_rot * (dot(c0, c0) - 1.0);
    r[4] = P.sw_rot * (dot(c1, c1) - 1.0);
    r[5] = P.sw_rot * (dot(c2, c2) - 1.0);
    const int a = P.free_ids[i];
    const double gj[3] = {P.g[3 * (size_t)a], P.g[3 * (size_t)a + 1], P.g[3 * (size_t)a + 2]};
    for (int j = 0; j < k; ++j) {
      const int c = P.nb[(size_t)a * k + j];
      const int rc = P.rank[c];
      const double gk[3] = {P.g[3 * (size_t)c], P.g[3 * (size_t)c + 1], P.g[3 * (size_t)c + 2]};
      const double d[3] = {gk[0] - gj[0], gk[1] - gj[1], gk[2] - gj[2]};
      double m[3];
      rmul(X, d, m);
      const double s = P.sw_reg * P.reg_scale[(size_t)i * k + j];
      double* o = f + P.rows_rot + 3 * ((size_t)i * k + j);
      for (int q = 0; q < 3; ++q) {
        const double tk = rc >= 0 ? x[12 * (size_t)rc + 9 + q] : 0.0;
        o[q] = (m[q] + gj[q] + X[9 + q] - gk[q] - tk) * s;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < P.S; ++i) {
    const int a = P.static_ids[i];
    for (int j = 0; j < k; ++j) {
      const int rc = P.rank[P.nb[(size_t)a * k + j]];
      double* o = f + P.rows_rot + P.rows_reg + 3 * ((size_t)i * k + j);
      for (int q = 0; q < 3; ++q) o[q] = P.sw_reg * -(rc >= 0 ? x[12 * (size_t)rc + 9 + q] : 0.0);
    }
  }
  double* con = f + P.rows_rot + P.rows_reg + P.rows_sta;
  if (P.center) {
    for (size_t s = 0; s < P.center_sets.size(); ++s) {
      double acc[3] = {0, 0, 0};
      for (int c : P.center_sets[s]) {
        double nv[3];
        blend_constraint(P, x, c, nv);
        for (int q = 0; q < 3; ++q) acc[q] += P.sw_con * (nv[q] - (double)P.center_aims[3 * s + q]);
      }
      for (int q = 0; q < 3; ++q) con[3 * s + q] = acc[q];
    }
  } else {
    const int C = (int)P.ctrl_nodes.size();
#pragma omp parallel for schedule(static)
    for (int t = 0; t < C; ++t) {
      const int c = P.ctrl_nodes[t];
      double nv[3];
      blend_constraint(P, x, c, nv);
      for (int q = 0; q < 3; ++q) con[3 * (size_t)t + q] = P.sw_con * (nv[q] - (double)P.aims[3 * (size_t)c + q]);
    }
  }
}

double dot(const double* a, const double* b, size_t n) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long long i = 0; i < (long long)n; ++i) s += a[i] * b[i];
  return s;
}

// --------------------------------------------------------- Jacobian ----
// FastCalcJacobiMat (Deform.cpp:180-376) in CSR: every row's (column, value)
// pairs, duplicates summed (setFromTriplets), columns ascending.
struct Csr {
  long long rows = 0;
  int cols = 0;
  std::vector<long long> ptr;
  std::vector<int> col;
  std::vector<double> val;
};

void jacobian(const Problem& P, const double* x, Csr& J) {
  const int F = P.F, k = P.k;
  const long long R = P.n_rows;
  J.rows = R;
  J.cols = 12 * F;
  // row lengths (before duplicates are merged)
  std::vector<long long>& ptr = J.ptr;
  ptr.assign(R + 1, 0);
  for (int i = 0; i < F; ++i) {
    for (int r = 0; r < 3; ++r) ptr[6 * (size_t)i + r + 1] = 6;
    for (int r = 3; r < 6; ++r) ptr[6 * (size_t)i + r + 1] = 3;
  }
  for (int i = 0; i < F; ++i)
    for (int j = 0; j < k; ++j) {
      const bool fr = P.rank[P.nb[(size_t)P.free_ids[i] * k + j]] >= 0;
      for (int q = 0; q < 3; ++q) ptr[P.rows_rot + 3 * ((size_t)i * k + j) + q + 1] = 4 + (fr ? 1 : 0);
    }
  for (int i = 0; i < P.S; ++i)
    for (int j = 0; j < k; ++j) {
      const bool fr = P.rank[P.nb[(size_t)P.static_ids[i] * k + j]] >= 0;
      for (int q = 0; q < 3; ++q) ptr[P.rows_rot + P.rows_reg + 3 * ((size_t)i * k + j) + q + 1] = fr ? 1 : 0;
    }
  const long long cbase = P.rows_rot + P.rows_reg + P.rows_sta;
  auto anchors_free = [&](int c) {
    int m = 0;
    for (int j = 0; j < k; ++j) m += P.rank[P.aidx[(size_t)c * k + j]] >= 0;
    return m;
  };
  if (P.center) {
    for (size_t s = 0; s < P.center_sets.size(); ++s) {
      int m = 0;
      for (int c : P.center_sets[s]) m += anchors_free(c);
      for (int q = 0; q < 3; ++q) ptr[cbase + 3 * (long long)s + q + 1] = 4LL * m;
    }
  } else {
    for (size_t t = 0; t < P.ctrl_nodes.size(); ++t) {
      const int m = anchors_free(P.ctrl_nodes[t]);
      for (int q = 0; q < 3; ++q) ptr[cbase + 3 * (long long)t + q + 1] = 4LL * m;
    }
  }
  for (long long r = 0; r < R; ++r) ptr[r + 1] += ptr[r];
  J.col.resize(ptr[R]);
  J.val.resize(ptr[R]);
  int* col = J.col.data();
  double* val = J.val.data();
  const double w = P.sw_rot;
  // rotation rows (Deform.cpp:189-220)
#pragma omp parallel for schedule(static)
  for (int i = 0; i < F; ++i) {
    const double* X = x + 12 * (size_t)i;
    const int cb = 12 * i;
    static const int spec[6][2][3] = {{{0, 1, 2}, {3, 4, 5}}, {{3, 4, 5}, {0, 1, 2}},
                                      {{0, 1, 2}, {6, 7, 8}}, {{6, 7, 8}, {0, 1, 2}},
                                      {{3, 4, 5}, {6, 7, 8}}, {{6, 7, 8}, {3, 4, 5}}};
    for (int r = 0; r < 3; ++r) {
      const long long p = ptr[6 * (size_t)i + r];
      // two spec entries per row, columns ascending by construction order:
      // first entry's columns are lower
      for (int h = 0; h < 2; ++h)
        for (int c = 0; c < 3; ++c) {
          col[p + 3 * h + c] = cb + spec[2 * r + h][0][c];
          val[p + 3 * h + c] = X[spec[2 * r + h][1][c]] * w;
        }
    }
    for (int j = 0; j < 3; ++j) {
      const long long p = ptr[6 * (size_t)i + 3 + j];
      for (int c = 0; c < 3; ++c) {
        col[p + c] = cb + 3 * j + c;
        val[p + c] = 2.0 * X[3 * j + c] * w;
      }
    }
  }
  // regularisation rows, free side (Deform.cpp:222-266): the float32 node
  // difference, and no weight_scale on the t_i column
  const double wr = P.sw_reg;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < F; ++i) {
    const int a = P.free_ids[i];
    for (int j = 0; j < k; ++j) {
      const int c = P.nb[(size_t)a * k + j];
      const int rc = P.rank[c];
      const double s = P.reg_scale[(size_t)i * k + j];
      float dfl[3];
      for (int q = 0; q < 3; ++q) dfl[q] = P.g[3 * (size_t)c + q] - P.g[3 * (size_t)a + q];
      for (int q = 0; q < 3; ++q) {
        const long long r = P.rows_rot + 3 * ((size_t)i * k + j) + q;
        long long p = ptr[r];
        // entries: 12i+q+3c (c=0..2), 12i+q+9, and 12rc+q+9; sorted
        int cs[5];
        double vs[5];
        int m = 0;
        for (int cc = 0; cc < 3; ++cc) {
          cs[m] = 12 * i + q + 3 * cc;
          vs[m++] = (double)dfl[cc] * wr * s;
        }
        cs[m] = 12 * i + q + 9;
        vs[m++] = wr;
        if (rc >= 0) {
          cs[m] = 12 * rc + q + 9;
          vs[m++] = -wr * s;
        }
        // insertion sort by column (rc != i, so no duplicates)
        for (int u = 1; u < m; ++u)
          for (int v = u; v > 0 && cs[v - 1] > cs[v]; --v) {
            std::swap(cs[v - 1], cs[v]);
            std::swap(vs[v - 1], vs[v]);
          }
        for (int u = 0; u < m; ++u) {
          col[p] = cs[u];
          val[p++] = vs[u];
        }
      }
    }
  }
  // static side (Deform.cpp:268-297)
#pragma omp parallel for schedule(static)
  for (int i = 0; i < P.S; ++i) {
    const int a = P.static_ids[i];
    for (int j = 0; j < k; ++j) {
      const int rc = P.rank[P.nb[(size_t)a * k + j]];
      if (rc < 0) continue;
      for (int q = 0; q < 3; ++q) {
        const long long p = ptr[P.rows_rot + P.rows_reg + 3 * ((size_t)i * k + j) + q];
        col[p] = 12 * rc + 9 + q;
        val[p] = -wr;
      }
    }
  }
  // constraints (Deform.cpp:299-371): float32 difference v - g_j
  const double wc = P.sw_con;
  auto con_entries = [&](int c, int q, std::vector<std::pair<int, double>>& out) {
    for (int j = 0; j < k; ++j) {
      const int a = P.aidx[(size_t)c * k + j];
      const int r = P.rank[a];
      if (r < 0) continue;
      const double wj = P.aw[(size_t)c * k + j];
      for (int cc = 0; cc < 3; ++cc) {
        const float dd = P.g[3 * (size_t)c + cc] - P.g[3 * (size_t)a + cc];
        out.emplace_back(12 * r + 3 * cc + q, wj * (double)dd * wc);
      }
      out.emplace_back(12 * r + 9 + q, wj * wc);
    }
  };
  auto write_row = [&](long long r, std::vector<std::pair<int, double>>& e) {
    std::sort(e.begin(), e.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    long long p = ptr[r];
    const long long end = ptr[r + 1];
    size_t u = 0;
    while (u < e.size()) {
      int c = e[u].first;
      double v = 0.0;
      while (u < e.size() && e[u].first == c) v += e[u++].second;
      col[p] = c;
      val[p++] = v;
    }
    // merged duplicates leave the tail short: pad with explicit zeros
    while (p < end) {
      col[p] = col[p - 1];
      val[p++] = 0.0;
    }
  };
  if (P.center) {
    for (size_t s = 0; s < P.center_sets.size(); ++s)
      for (int q = 0; q < 3; ++q) {
        std::vector<std::pair<int, double>> e;
        for (int c : P.center_sets[s]) con_entries(c, q, e);
        write_row(cbase + 3 * (long long)s + q, e);
      }
  } else {
    const int C = (int)P.ctrl_nodes.size();
#pragma omp parallel for schedule(static)
    for (int t = 0; t < C; ++t) {
      std::vector<std::pair<int, double>> e;
      for (int q = 0; q < 3; ++q) {
        e.clear();
        con_entries(P.ctrl_nodes[t], q, e);
        write_row(cbase + 3 * (long long)t + q, e);
      }
    }
  }
}

// y = J^T v (row-parallel with per-thread accumulators would race; use CSC)
struct Csc {
  std::vector<long long> ptr;
  std::vector<long long> row;
  std::vector<long long> src;  // index of the entry in the CSR arrays
};

void transpose_pattern(const Csr& J, Csc& T) {
  const int n = J.cols;
  T.ptr.assign(n + 1, 0);
  for (long long p = 0; p < J.ptr[J.rows]; ++p) T.ptr[J.col[p] + 1]++;
  for (int c = 0; c < n; ++c) T.ptr[c + 1] += T.ptr[c];
  T.row.resize(J.ptr[J.rows]);
  T.src.resize(J.ptr[J.rows]);
  std::vector<long long> cur(T.ptr.begin(), T.ptr.end() - 1);
  for (long long r = 0; r < J.rows; ++r)
    for (long long p = J.ptr[r]; p < J.ptr[r + 1]; ++p) {
      const long long d = cur[J.col[p]]++;
      T.row[d] = r;
      T.src[d] = p;
    }
}

void jt_mul(const Csr& J, const Csc& T, const double* v, double* y) {
#pragma omp parallel for schedule(static)
  for (int c = 0; c < J.cols; ++c) {
    double s = 0.0;
    for (long long p = T.ptr[c]; p < T.ptr[c + 1]; ++p) s += J.val[T.src[p]] * v[T.row[p]];
    y[c] = s;
  }
}

// ------------------------------------------------- block sparse Cholesky ----
// Node-level structure: A = J^T J in 12x12 blocks over the free nodes.
constexpr int B = 12;
constexpr int BB = B * B;

struct BlockMatrix {     // symmetric, both triangles stored by block column
  int F = 0;
  std::vector<int> ptr;  // [F+1], block column j holds rows idx[ptr[j]..ptr[j+1])
  std::vector<int> idx;  // row node of each block (sorted, includes j)
  std::vector<double> val;  // [blocks][12][12]: block (row node, column node), row-major
};

// The node-level pattern of J^T J: two free nodes couple when a row of J
// touches both.
void a_pattern(const Csr& J, int F, BlockMatrix& A) {
  std::vector<std::vector<int>> adj(F);
  std::vector<int> nodes;
  for (long long r = 0; r < J.rows; ++r) {
    nodes.clear();
    for (long long p = J.ptr[r]; p < J.ptr[r + 1]; ++p) nodes.push_back(J.col[p] / B);
    std::sort(nodes.begin(), nodes.end());
    nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
    for (int a : nodes)
      for (int b : nodes) adj[a].push_back(b);
  }
  A.F = F;
  A.ptr.assign(F + 1, 0);
  for (int j = 0; j < F; ++j) {
    auto& v = adj[j];
    v.push_back(j);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    A.ptr[j + 1] = A.ptr[j] + (int)v.size();
  }
  A.idx.resize(A.ptr[F]);
  for (int j = 0; j < F; ++j) std::copy(adj[j].begin(), adj[j].end(), A.idx.begin() + A.ptr[j]);
  A.val.assign((size_t)A.ptr[F] * BB, 0.0);
}

// A = J^T J numerically, block column by block column (no write races).
void a_numeric(const Csr& J, const Csc& T, BlockMatrix& A) {
  const int F = A.F;
#pragma omp parallel
  {
    std::vector<int> where(F, -1);
#pragma omp for schedule(dynamic, 16)
    for (int j = 0; j < F; ++j) {
      for (int t = A.ptr[j]; t < A.ptr[j + 1]; ++t) where[A.idx[t]] = t;
      double* base = A.val.data();
      for (int t = A.ptr[j]; t < A.ptr[j + 1]; ++t) std::memset(base + (size_t)t * BB, 0, sizeof(double) * BB);
      for (int cl = 0; cl < B; ++cl) {
        const int c = B * j + cl;
        for (long long p = T.ptr[c]; p < T.ptr[c + 1]; ++p) {
          const long long r = T.row[p];
          const double v = J.val[T.src[p]];
          for (long long q = J.ptr[r]; q < J.ptr[r + 1]; ++q) {
            const int c2 = J.col[q];
            double* blk = base + (size_t)where[c2 / B] * BB;
            blk[(c2 % B) * B + cl] += J.val[q] * v;
          }
        }
      }
      for (int t = A.ptr[j]; t < A.ptr[j + 1]; ++t) where[A.idx[t]] = -1;
    }
  }
}

// Minimum-degree ordering of the node graph (exact degrees on the
// elimination graph, lowest node id first among equal degrees).
std::vector<int> min_degree(const BlockMatrix& A) {
  const int F = A.F;
  std::vector<std::vector<int>> adj(F);
  for (int j = 0; j < F; ++j)
    for (int t = A.ptr[j]; t < A.ptr[j + 1]; ++t)
      if (A.idx[t] != j) adj[j].push_back(A.idx[t]);
  std::vector<char> gone(F, 0);
  using Item = std::pair<int, int>;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
  for (int j = 0; j < F; ++j) pq.push({(int)adj[j].size(), j});
  std::vector<int> order;
  order.reserve(F);
  std::vector<int> tmp;
  while (!pq.empty()) {
    const auto [d, v] = pq.top();
    pq.pop();
    if (gone[v] || d != (int)adj[v].size()) continue;
    gone[v] = 1;
    order.push_back(v);
    const std::vector<int> nv = adj[v];
    for (int u : nv) {
      tmp.clear();
      std::set_union(adj[u].begin(), adj[u].end(), nv.begin(), nv.end(), std::back_inserter(tmp));
      auto& au = adj[u];
      au.clear();
      for (int w : tmp)
        if (w != u && w != v) au.push_back(w);
      pq.push({(int)au.size(), u});
    }
    adj[v].clear();
  }
  return order;
}

// Geometric nested dissection of the node graph: split the node set at the
// median of its widest coordinate, take as separator the nodes of the lower
// half with a neighbour in the upper half, order both halves recursively and
// the separator last.  Small sets are ordered by minimum degree.
void nd_recurse(const BlockMatrix& A, const float* xyz, std::vector<int>& set, std::vector<int>& side,
                std::vector<int>& out) {
  const int m = (int)set.size();
  if (m <= 48) {
    // local minimum degree on the induced subgraph
    std::vector<int> loc(set);
    std::vector<std::vector<int>> adj(m);
    for (int a = 0; a < m; ++a) side[loc[a]] = a + 1;  // mark membership with local id + 1
    for (int a = 0; a < m; ++a) {
      const int v = loc[a];
      for (int t = A.ptr[v]; t < A.ptr[v + 1]; ++t) {
        const int u = A.idx[t];
        if (u != v && side[u] > 0) adj[a].push_back(side[u] - 1);
      }
    }
    for (int a = 0; a < m; ++a) side[loc[a]] = 0;
    std::vector<char> gone(m, 0);
    std::vector<int> tmp;
    for (int step = 0; step < m; ++step) {
      int best = -1;
      for (int a = 0; a < m; ++a)
        if (!gone[a] && (best < 0 || adj[a].size() < adj[best].size())) best = a;
      gone[best] = 1;
      out.push_back(loc[best]);
      const std::vector<int> nv = adj[best];
      for (int u : nv) {
        tmp.clear();
        std::set_union(adj[u].begin(), adj[u].end(), nv.begin(), nv.end(), std::back_inserter(tmp));
        adj[u].clear();
        for (int w : tmp)
          if (w != u && w != best) adj[u].push_back(w);
      }
      adj[best].clear();
    }
    return;
  }
  float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
  for (int v : set)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], xyz[3 * (size_t)v + d]);
      hi[d] = std::max(hi[d], xyz[3 * (size_t)v + d]);
    }
  int ax = 0;
  for (int d = 1; d < 3; ++d)
    if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
  std::vector<int> srt(set);
  std::nth_element(srt.begin(), srt.begin() + m / 2, srt.end(), [&](int a, int b) {
    const float pa = xyz[3 * (size_t)a + ax], pb = xyz[3 * (size_t)b + ax];
    return pa < pb || (pa == pb && a < b);
  });
  // side: 1 lower half, 2 upper half (of this set only)
  for (int t = 0; t < m; ++t) side[srt[t]] = t < m / 2 ? 1 : 2;
  std::vector<int> left, right, sep;
  for (int t = 0; t < m / 2; ++t) {
    const int v = srt[t];
    bool cut = false;
    for (int u = A.ptr[v]; u < A.ptr[v + 1] && !cut; ++u) cut = side[A.idx[u]] == 2;
    (cut ? sep : left).push_back(v);
  }
  for (int t = m / 2; t < m; ++t) right.push_back(srt[t]);
  for (int v : set) side[v] = 0;
  std::sort(left.begin(), left.end());
  std::sort(right.begin(), right.end());
  std::sort(sep.begin(), sep.end());
  nd_recurse(A, xyz, left, side, out);
  nd_recurse(A, xyz, right, side, out);
  for (int v : sep) out.push_back(v);
}

std::vector<int> nested_dissection(const BlockMatrix& A, const float* xyz) {
  std::vector<int> all(A.F), side(A.F, 0), out;
  for (int i = 0; i < A.F; ++i) all[i] = i;
  out.reserve(A.F);
  nd_recurse(A, xyz, all, side, out);
  return out;
}

struct Factor {
  int F = 0;
  std::vector<int> perm, iperm;    // perm[new] = old
  std::vector<int> parent;         // elimination tree (new indices), -1 at roots
  std::vector<int> sptr, sidx;     // struct(j): rows > j (new indices), sorted
  std::vector<int> rptr, rk, rpos; // row lists: columns k < j with j in struct(k), position there
  std::vector<size_t> loff;        // block offset of column j in L (diag first)
  std::vector<double> L;
  std::vector<int> sub_roots;      // roots of the subtrees factorised in parallel
  std::vector<std::vector<int>> sub_cols;
  std::vector<int> top_cols;       // the rest, grouped by level
  std::vector<int> level_ptr;      // top_cols[level_ptr[l] .. level_ptr[l+1]) form level l
  std::vector<long long> rwork;    // prefix over row-list entries of the updates each applies
  std::vector<int> aj_perm;        // A's block column for new column j
};

void analyse(const BlockMatrix& A, const float* xyz, int ordering, Factor& L, int nthreads) {
  const int F = A.F;
  L.F = F;
  L.perm = ordering == 1 ? nested_dissection(A, xyz) : min_degree(A);
  L.iperm.assign(F, 0);
  for (int i = 0; i < F; ++i) L.iperm[L.perm[i]] = i;
  // symbolic factorisation: struct(j) = A's rows > j in column j, united
  // with the structs of j's children minus j
  std::vector<std::vector<int>> st(F);
  std::vector<std::vector<int>> children(F);
  L.parent.assign(F, -1);
  std::vector<int> tmp;
  for (int j = 0; j < F; ++j) {
    const int oj = L.perm[j];
    std::vector<int> s;
    for (int t = A.ptr[oj]; t < A.ptr[oj + 1]; ++t) {
      const int i = L.iperm[A.idx[t]];
      if (i > j) s.push_back(i);
    }
    std::sort(s.begin(), s.end());
    for (int c : children[j]) {
      tmp.clear();
      std::set_union(s.begin(), s.end(), st[c].begin(), st[c].end(), std::back_inserter(tmp));
      s.swap(tmp);
    }
    s.erase(std::remove(s.begin(), s.end(), j), s.end());
    if (!s.empty()) {
      L.parent[j] = s[0];
      children[s[0]].push_back(j);
    }
    st[j] = std::move(s);
  }
  L.sptr.assign(F + 1, 0);
  for (int j = 0; j < F; ++j) L.sptr[j + 1] = L.sptr[j] + (int)st[j].size();
  L.sidx.resize(L.sptr[F]);
  for (int j = 0; j < F; ++j) std::copy(st[j].begin(), st[j].end(), L.sidx.begin() + L.sptr[j]);
  // row lists
  std::vector<int> cnt(F + 1, 0);
  for (int j = 0; j < F; ++j)
    for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) cnt[L.sidx[t] + 1]++;
  L.rptr.assign(F + 1, 0);
  for (int i = 0; i < F; ++i) L.rptr[i + 1] = L.rptr[i] + cnt[i + 1];
  L.rk.resize(L.rptr[F]);
  L.rpos.resize(L.rptr[F]);
  std::vector<int> cur(L.rptr.begin(), L.rptr.end() - 1);
  for (int j = 0; j < F; ++j)
    for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) {
      const int i = L.sidx[t];
      L.rk[cur[i]] = j;
      L.rpos[cur[i]++] = t - L.sptr[j];
    }
  L.loff.assign(F + 1, 0);
  for (int j = 0; j < F; ++j) L.loff[j + 1] = L.loff[j] + 1 + (size_t)(L.sptr[j + 1] - L.sptr[j]);
  L.L.assign(L.loff[F] * BB, 0.0);
  // split: subtrees of at most total/(4 threads) cost go to the parallel
  // phase; their ancestors form the top, factorised in order
  std::vector<double> cost(F), sub(F);
  for (int j = 0; j < F; ++j) {
    double m = 1.0 + (L.sptr[j + 1] - L.sptr[j]);
    cost[j] = m * m;
  }
  for (int j = 0; j < F; ++j) {
    sub[j] += cost[j];
    if (L.parent[j] >= 0) sub[L.parent[j]] += sub[j];
  }
  double total = 0.0;
  for (int j = 0; j < F; ++j)
    if (L.parent[j] < 0) total += sub[j];
  const double cap = total / (4.0 * std::max(1, nthreads));
  std::vector<char> top(F, 0);
  std::vector<int> stack;
  for (int j = 0; j < F; ++j)
    if (L.parent[j] < 0) stack.push_back(j);
  L.sub_roots.clear();
  while (!stack.empty()) {
    const int j = stack.back();
    stack.pop_back();
    if (sub[j] <= cap || children[j].empty()) {
      L.sub_roots.push_back(j);
    } else {
      top[j] = 1;
      for (int c : children[j]) stack.push_back(c);
    }
  }
  std::sort(L.sub_roots.begin(), L.sub_roots.end(), [&](int a, int b) { return sub[a] > sub[b]; });
  L.sub_cols.assign(L.sub_roots.size(), {});
  for (size_t s = 0; s < L.sub_roots.size(); ++s) {
    std::vector<int>& cols = L.sub_cols[s];
    stack.assign(1, L.sub_roots[s]);
    while (!stack.empty()) {
      const int j = stack.back();
      stack.pop_back();
      cols.push_back(j);
      for (int c : children[j]) stack.push_back(c);
    }
    std::sort(cols.begin(), cols.end());
  }
  // levels of the top part: 1 + the highest level among its top children
  std::vector<int> level(F, 0);
  int max_level = 0;
  for (int j = 0; j < F; ++j)
    if (top[j]) {
      int lv = 0;
      for (int c : children[j])
        if (top[c]) lv = std::max(lv, level[c] + 1);
      level[j] = lv;
      max_level = std::max(max_level, lv);
    }
  L.top_cols.clear();
  L.level_ptr.assign(1, 0);
  for (int lv = 0; lv <= max_level; ++lv) {
    for (int j = 0; j < F; ++j)
      if (top[j] && level[j] == lv) L.top_cols.push_back(j);
    L.level_ptr.push_back((int)L.top_cols.size());
  }
  L.rwork.assign(L.rptr[F] + 1, 0);
  for (int t = 0; t < L.rptr[F]; ++t) {
    const int kc = L.rk[t];
    L.rwork[t + 1] = L.rwork[t] + (L.sptr[kc + 1] - L.sptr[kc] - L.rpos[t]);
  }
}

// 12x12 kernels (row-major)
bool chol12(double* D) {  // lower Cholesky in place
  for (int j = 0; j < B; ++j) {
    double d = D[j * B + j];
    for (int t = 0; t < j; ++t) d -= D[j * B + t] * D[j * B + t];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    D[j * B + j] = d;
    for (int i = j + 1; i < B; ++i) {
      double s = D[i * B + j];
      for (int t = 0; t < j; ++t) s -= D[i * B + t] * D[j * B + t];
      D[i * B + j] = s / d;
    }
    for (int t = j + 1; t < B; ++t) D[j * B + t] = 0.0;
  }
  return true;
}

inline void trsm_rt(double* __restrict__ X, const double* __restrict__ Ld) {  // X <- X L^-T
  for (int r = 0; r < B; ++r)
    for (int c = 0; c < B; ++c) {
      double s = X[r * B + c];
      for (int t = 0; t < c; ++t) s -= X[r * B + t] * Ld[c * B + t];
      X[r * B + c] = s / Ld[c * B + c];
    }
}

// C -= A Bt with Bt = B^T given (row-major 12x12): four rows of C are
// accumulated at once, each a sum of axpys of Bt's rows, so every row of Bt
// loaded feeds four rows of FMAs.
inline void gemm_nn_sub(double* __restrict__ C, const double* __restrict__ A, const double* __restrict__ Bt) {
  for (int r0 = 0; r0 < B; r0 += 4) {
    double acc[4][B];
    for (int u = 0; u < 4; ++u)
      for (int c = 0; c < B; ++c) acc[u][c] = 0.0;
    for (int t = 0; t < B; ++t) {
      const double a0 = A[(r0 + 0) * B + t], a1 = A[(r0 + 1) * B + t], a2 = A[(r0 + 2) * B + t],
                   a3 = A[(r0 + 3) * B + t];
      for (int c = 0; c < B; ++c) {
        const double b = Bt[t * B + c];
        acc[0][c] += a0 * b;
        acc[1][c] += a1 * b;
        acc[2][c] += a2 * b;
        acc[3][c] += a3 * b;
      }
    }
    for (int u = 0; u < 4; ++u)
      for (int c = 0; c < B; ++c) C[(r0 + u) * B + c] -= acc[u][c];
  }
}

// Scatter A's column into W and apply the updates of the columns in row j's
// list [r0, r1) into W (W = diag block then one block per struct entry).
void gather_updates(const Factor& L, int j, int r0, int r1, const int* relpos, double* W) {
  alignas(64) double Bt[BB];
  for (int t = r0; t < r1; ++t) {
    const int kc = L.rk[t], p = L.rpos[t];
    const double* Lk = L.L.data() + L.loff[kc] * BB;
    const int* sk = L.sidx.data() + L.sptr[kc];
    const int nk = L.sptr[kc + 1] - L.sptr[kc];
    const double* Ljk = Lk + (size_t)(1 + p) * BB;
    for (int r = 0; r < B; ++r)
      for (int c = 0; c < B; ++c) Bt[c * B + r] = Ljk[r * B + c];
    for (int q = p; q < nk; ++q) {
      const int i = sk[q];
      double* dst = W + (size_t)(i == j ? 0 : 1 + relpos[i]) * BB;
      gemm_nn_sub(dst, Lk + (size_t)(1 + q) * BB, Bt);
    }
  }
}

void init_column(const BlockMatrix& A, const Factor& L, int j, const int* relpos, double* W) {
  const int oj = L.perm[j];
  const size_t nb = L.sptr[j + 1] - L.sptr[j];
  std::memset(W, 0, sizeof(double) * (1 + nb) * BB);
  for (int t = A.ptr[oj]; t < A.ptr[oj + 1]; ++t) {
    const int i = L.iperm[A.idx[t]];
    if (i < j) continue;
    const double* src = A.val.data() + (size_t)t * BB;
    double* dst = W + (size_t)(i == j ? 0 : 1 + relpos[i]) * BB;
    for (int e = 0; e < BB; ++e) dst[e] += src[e];
  }
}

bool finish_column(const Factor& L, int j, double* W) {
  if (!chol12(W)) return false;
  const int nb = L.sptr[j + 1] - L.sptr[j];
  for (int b = 0; b < nb; ++b) trsm_rt(W + (size_t)(1 + b) * BB, W);
  return true;
}

double g_t_phase1 = 0.0, g_t_phase2 = 0.0;

bool factorize(const BlockMatrix& A, Factor& L, int nthreads) {
  const int F = L.F;
  const auto tp1 = Clock::now();
  std::atomic<bool> ok{true};
  // phase 1: independent subtrees
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<int> relpos(F, -1);
#pragma omp for schedule(dynamic, 1)
    for (int s = 0; s < (int)L.sub_roots.size(); ++s) {
      for (int j : L.sub_cols[s]) {
        for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) relpos[L.sidx[t]] = t - L.sptr[j];
        double* W = L.L.data() + L.loff[j] * BB;
        init_column(A, L, j, relpos.data(), W);
        gather_updates(L, j, L.rptr[j], L.rptr[j + 1], relpos.data(), W);
        if (!finish_column(L, j, W)) ok = false;
      }
    }
  }
  // phase 2: the top of the tree by levels (a level's columns depend only on
  // earlier levels).  A level with at least as many columns as threads is
  // split by columns; a smaller level is factorised column by column with
  // each column's updates split over the threads by work, into private
  // accumulators that are then summed.
  const auto tp2 = Clock::now();
  std::vector<int> shared_relpos(F, -1);
  std::vector<std::vector<double>> privs(nthreads);
#pragma omp parallel num_threads(nthreads)
  {
    const int nt = omp_get_num_threads(), tid = omp_get_thread_num();
    std::vector<int> relpos(F, -1);
    std::vector<double>& priv = privs[tid];
    for (size_t lv = 0; lv + 1 < L.level_ptr.size(); ++lv) {
      const int c0 = L.level_ptr[lv], c1 = L.level_ptr[lv + 1];
      if (c1 - c0 >= nt) {
#pragma omp for schedule(dynamic, 1)
        for (int c = c0; c < c1; ++c) {
          const int j = L.top_cols[c];
          for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) relpos[L.sidx[t]] = t - L.sptr[j];
          double* W = L.L.data() + L.loff[j] * BB;
          init_column(A, L, j, relpos.data(), W);
          gather_updates(L, j, L.rptr[j], L.rptr[j + 1], relpos.data(), W);
          if (!finish_column(L, j, W)) ok = false;
        }
        continue;
      }
      for (int c = c0; c < c1; ++c) {
        const int j = L.top_cols[c];
        const int nb = L.sptr[j + 1] - L.sptr[j];
        double* W = L.L.data() + L.loff[j] * BB;
        const size_t wsz = (size_t)(1 + nb) * BB;
        if (L.rwork[L.rptr[j + 1]] - L.rwork[L.rptr[j]] < 256) {
          // too little work to share: one thread, one barrier
#pragma omp single
          {
            for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) relpos[L.sidx[t]] = t - L.sptr[j];
            init_column(A, L, j, relpos.data(), W);
            gather_updates(L, j, L.rptr[j], L.rptr[j + 1], relpos.data(), W);
            if (!finish_column(L, j, W)) ok = false;
          }
          continue;
        }
#pragma omp single
        {
          for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) shared_relpos[L.sidx[t]] = t - L.sptr[j];
          init_column(A, L, j, shared_relpos.data(), W);
        }
        // this thread's share of the row list, balanced by update count
        const int r0 = L.rptr[j], r1 = L.rptr[j + 1];
        const long long w0 = L.rwork[r0], wt = L.rwork[r1] - w0;
        const long long lo = w0 + wt * tid / nt, hi = w0 + wt * (tid + 1) / nt;
        const int a = (int)(std::lower_bound(L.rwork.begin() + r0, L.rwork.begin() + r1, lo) - L.rwork.begin());
        const int b = (int)(std::lower_bound(L.rwork.begin() + r0, L.rwork.begin() + r1, hi) - L.rwork.begin());
        if (priv.size() < wsz) priv.resize(wsz);
        std::memset(priv.data(), 0, sizeof(double) * wsz);
        gather_updates(L, j, a, std::min(b, r1), shared_relpos.data(), priv.data());
#pragma omp barrier
#pragma omp for schedule(static)
        for (long long e = 0; e < (long long)wsz; ++e) {
          double sum = 0.0;
          for (int u = 0; u < nt; ++u) sum += privs[u][e];
          W[e] += sum;
        }
#pragma omp single
        if (!chol12(W)) ok = false;
#pragma omp for schedule(static)
        for (int bb = 0; bb < nb; ++bb) trsm_rt(W + (size_t)(1 + bb) * BB, W);
      }
    }
  }
  g_t_phase1 += secs(tp1, tp2);
  g_t_phase2 += secs(tp2, Clock::now());
  return ok;
}

// L L^T h = g, in the original unknown order.
void solve(const Factor& L, const double* g, double* h) {
  const int F = L.F;
  std::vector<double> y((size_t)F * B);
  for (int j = 0; j < F; ++j)
    for (int c = 0; c < B; ++c) y[(size_t)j * B + c] = g[(size_t)L.perm[j] * B + c];
  // forward: L y = b, column-oriented
  for (int j = 0; j < F; ++j) {
    const double* W = L.L.data() + L.loff[j] * BB;
    double* yj = y.data() + (size_t)j * B;
    for (int r = 0; r < B; ++r) {
      double s = yj[r];
      for (int t = 0; t < r; ++t) s -= W[r * B + t] * yj[t];
      yj[r] = s / W[r * B + r];
    }
    for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) {
      const double* Lij = W + (size_t)(1 + t - L.sptr[j]) * BB;
      double* yi = y.data() + (size_t)L.sidx[t] * B;
      for (int r = 0; r < B; ++r) {
        double s = 0.0;
        for (int c = 0; c < B; ++c) s += Lij[r * B + c] * yj[c];
        yi[r] -= s;
      }
    }
  }
  // backward: L^T x = y
  for (int j = F - 1; j >= 0; --j) {
    const double* W = L.L.data() + L.loff[j] * BB;
    double* yj = y.data() + (size_t)j * B;
    for (int t = L.sptr[j]; t < L.sptr[j + 1]; ++t) {
      const double* Lij = W + (size_t)(1 + t - L.sptr[j]) * BB;
      const double* yi = y.data() + (size_t)L.sidx[t] * B;
      for (int c = 0; c < B; ++c) {
        double s = 0.0;
        for (int r = 0; r < B; ++r) s += Lij[r * B + c] * yi[r];
        yj[c] -= s;
      }
    }
    for (int r = B - 1; r >= 0; --r) {
      double s = yj[r];
      for (int t = r + 1; t < B; ++t) s -= W[t * B + r] * yj[t];
      yj[r] = s / W[r * B + r];
    }
  }
  for (int j = 0; j < F; ++j)
    for (int c = 0; c < B; ++c) h[(size_t)L.perm[j] * B + c] = y[(size_t)j * B + c];
}

// ------------------------------------------------------------ skinning ----

// predict_mesh (Deform.hpp:230-249): the float32 point-node difference, the
// blend term in float64, the sum rounded to float32 after every neighbour.
inline void ed_blend_one(const float* p, const int32_t* idx, const float* w32, const double* w64, int k,
                         const double* rot, const double* tr, const float* g, float out[3]) {
  float o[3] = {0.f, 0.f, 0.f};
  for (int j = 0; j < k; ++j) {
    const int n = idx[j];
    const double wj = w64 ? w64[j] : (double)w32[j];
    const double d[3] = {(double)(p[0] - g[3 * (size_t)n]), (double)(p[1] - g[3 * (size_t)n + 1]),
                         (double)(p[2] - g[3 * (size_t)n + 2])};
    const double* R = rot + 9 * (size_t)n;
    for (int q = 0; q < 3; ++q) {
      const double m = R[q] * d[0] + R[3 + q] * d[1] + R[6 + q] * d[2] + tr[3 * (size_t)n + q] +
                       (double)g[3 * (size_t)n + q];
      o[q] = (float)((double)o[q] + wj * m);
    }
  }
  out[0] = o[0];
  out[1] = o[1];
  out[2] = o[2];
}

void quat_to_matrix(const double q[4], double R[9]) {  // row-major
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  R[0] = 1 - 2 * (y * y + z * z);
  R[1] = 2 * (x * y - w * z);
  R[2] = 2 * (x * z + w * y);
  R[3] = 2 * (x * y + w * z);
  R[4] = 1 - 2 * (x * x + z * z);
  R[5] = 2 * (y * z - w * x);
  R[6] = 2 * (x * z - w * y);
  R[7] = 2 * (y * z + w * x);
  R[8] = 1 - 2 * (x * x + y * y);
}

void normalize4(double q[4]) {
  const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int i = 0; i < 4; ++i) q[i] /= n;
}

// Shoemake's trace / largest-diagonal method (Eigen's Quaternion(Matrix3)).
void quat_from_matrix(const double m[9], double q[4]) {
  const double tr = m[0] + m[4] + m[8];
  if (tr > 0) {
    const double t = std::sqrt(tr + 1.0), s = 0.5 / t;
    q[0] = 0.5 * t;
    q[1] = (m[7] - m[5]) * s;
    q[2] = (m[2] - m[6]) * s;
    q[3] = (m[3] - m[1]) * s;
    return;
  }
  int i = 0;
  if (m[4] > m[0]) i = 1;
  if (m[8] > m[i * 3 + i]) i = 2;
  const int j = (i + 1) % 3, k = (j + 1) % 3;
  const double t = std::sqrt(m[i * 3 + i] - m[j * 3 + j] - m[k * 3 + k] + 1.0), s = 0.5 / t;
  double v[3];
  v[i] = 0.5 * t;
  q[0] = (m[k * 3 + j] - m[j * 3 + k]) * s;
  v[j] = (m[j * 3 + i] + m[i * 3 + j]) * s;
  v[k] = (m[k * 3 + i] + m[i * 3 + k]) * s;
  q[1] = v[0];
  q[2] = v[1];
  q[3] = v[2];
}

void quat_mul(const double a[4], const double b[4], double o[4]) {
  o[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  o[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
  o[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
  o[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}

// Real-SH rotation of bands 1..3 (Ivanic-Ruedenberg recurrence), band 1 in
// the (y, z, x) order of helper.cpp:988-996; R row-major.
struct ShBands {
  double b1[3][3], b2[5][5], b3[7][7];
};

void sh_bands(const double R[9], ShBands& S) {
  const int perm[3] = {1, 2, 0};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) S.b1[a][b] = R[perm[a] * 3 + perm[b]];
  auto R1 = [&](int i, int j) { return S.b1[i + 1][j + 1]; };
  for (int l = 2; l <= 3; ++l) {
    const int lp = l - 1;
    auto Rp = [&](int a, int b) -> double { return l == 2 ? S.b1[a + lp][b + lp] : S.b2[a + lp][b + lp]; };
    auto P = [&](int i, int a, int b) -> double {
      if (b == l) return R1(i, 1) * Rp(a, l - 1) - R1(i, -1) * Rp(a, -l + 1);
      if (b == -l) return R1(i, 1) * Rp(a, -l + 1) + R1(i, -1) * Rp(a, l - 1);
      return R1(i, 0) * Rp(a, b);
    };
    for (int m = -l; m <= l; ++m)
      for (int n = -l; n <= l; ++n) {
        const double d = m == 0 ? 1.0 : 0.0;
        const double den = std::abs(n) < l ? (double)((l + n) * (l - n)) : (double)(2 * l * (2 * l - 1));
        const int am = std::abs(m);
        const double u = std::sqrt((double)((l + m) * (l - m)) / den);
        const double v = 0.5 * std::sqrt((1 + d) * (double)((l + am - 1) * (l + am)) / den) * (1 - 2 * d);
        const double w = -0.5 * std::sqrt((double)((l - am - 1) * (l - am)) / den) * (1 - d);
        double acc = 0.0;
        if (u != 0) acc += u * P(0, m, n);
        if (v != 0) {
          double V;
          if (m == 0)
            V = P(1, 1, n) + P(-1, -1, n);
          else if (m > 0)
            V = P(1, m - 1, n) * std::sqrt(1.0 + (m == 1)) - P(-1, -m + 1, n) * (1 - (m == 1));
          else
            V = P(1, m + 1, n) * (1 - (m == -1)) + P(-1, -m - 1, n) * std::sqrt(1.0 + (m == -1));
          acc += v * V;
        }
        if (w != 0) {
          double W;
          if (m > 0)
            W = P(1, m + 1, n) + P(-1, -m - 1, n);
          else
            W = P(1, m - 1, n) - P(-1, -m + 1, n);
          acc += w * W;
        }
        if (l == 2)
          S.b2[m + l][n + l] = acc;
        else
          S.b3[m + l][n + l] = acc;
      }
  }
}

// rotate_sh with the odd-coefficient flips (GaussianView.cpp:3138-3154),
// float32 in and out.
void rotate_sh(const float* in, const double R[9], float* out) {
  ShBands S;
  sh_bands(R, S);
  double s[16][3];
  for (int c = 0; c < 16; ++c)
    for (int ch = 0; ch < 3; ++ch) s[c][ch] = (double)in[3 * c + ch] * ((c & 1) ? -1.0 : 1.0);
  double o[16][3];
  for (int ch = 0; ch < 3; ++ch) {
    o[0][ch] = s[0][ch];
    for (int a = 0; a < 3; ++a) {
      double t = 0.0;
      for (int b = 0; b < 3; ++b) t += S.b1[a][b] * s[1 + b][ch];
      o[1 + a][ch] = t;
    }
    for (int a = 0; a < 5; ++a) {
      double t = 0.0;
      for (int b = 0; b < 5; ++b) t += S.b2[a][b] * s[4 + b][ch];
      o[4 + a][ch] = t;
    }
    for (int a = 0; a < 7; ++a) {
      double t = 0.0;
      for (int b = 0; b < 7; ++b) t += S.b3[a][b] * s[9 + b][ch];
      o[9 + a][ch] = t;
    }
  }
  for (int c = 0; c < 16; ++c)
    for (int ch = 0; ch < 3; ++ch) out[3 * c + ch] = (float)(o[c][ch] * ((c & 1) ? -1.0 : 1.0));
}

// One-sided Jacobi SVD of a 3x3 (row-major) M: R = U V^T, K = diag(V S V^T).
void polar_svd(const double M[9], double R[9], double K[3]) {
  double A[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) A[r][c] = M[r * 3 + c];
  for (int sweep = 0; sweep < 40; ++sweep) {
    double off = 0.0;
    const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (auto& pq : pairs) {
      const int p = pq[0], q = pq[1];
      double al = 0, be = 0, ga = 0;
      for (int r = 0; r < 3; ++r) {
        al += A[r][p] * A[r][p];
        be += A[r][q] * A[r][q];
        ga += A[r][p] * A[r][q];
      }
      const double nrm = std::sqrt(al * be);
      if (nrm == 0.0 || std::abs(ga) <= 1e-17 * nrm) continue;
      off = std::max(off, std::abs(ga) / nrm);
      const double zeta = (be - al) / (2.0 * ga);
      const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::abs(zeta) + std::sqrt(1.0 + zeta * zeta));
      const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
      for (int r = 0; r < 3; ++r) {
        const double ap = A[r][p], aq = A[r][q];
        A[r][p] = c * ap - s * aq;
        A[r][q] = s * ap + c * aq;
        const double vp = V[r][p], vq = V[r][q];
        V[r][p] = c * vp - s * vq;
        V[r][q] = s * vp + c * vq;
      }
    }
    if (off < 1e-16) break;
  }
  double sig[3], U[3][3];
  for (int c = 0; c < 3; ++c) {
    sig[c] = std::sqrt(A[0][c] * A[0][c] + A[1][c] * A[1][c] + A[2][c] * A[2][c]);
    for (int r = 0; r < 3; ++r) U[r][c] = sig[c] > 0 ? A[r][c] / sig[c] : 0.0;
  }
  // a zero singular value: complete U's column by the cross product
  for (int c = 0; c < 3; ++c)
    if (!(sig[c] > 0)) {
      const int a = (c + 1) % 3, b = (c + 2) % 3;
      U[0][c] = U[1][a] * U[2][b] - U[2][a] * U[1][b];
      U[1][c] = U[2][a] * U[0][b] - U[0][a] * U[2][b];
      U[2][c] = U[0][a] * U[1][b] - U[1][a] * U[0][b];
    }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[r * 3 + c] = U[r][0] * V[c][0] + U[r][1] * V[c][1] + U[r][2] * V[c][2];
  for (int i = 0; i < 3; ++i) K[i] = V[i][0] * sig[0] * V[i][0] + V[i][1] * sig[1] * V[i][1] + V[i][2] * sig[2] * V[i][2];
}

// UpdateAsSixPointsWithdrawBad (GaussianView.cpp:3081-3166) for one Gaussian
// from its six deformed endpoints.
void refit_one(const float* E, const float* q_old, const float* s0, const float* sh_in, float* pos, float* q_out,
               float* s_out, float* sh_out, float* cov6) {
  double c[3] = {0, 0, 0};
  for (int e = 0; e < 6; ++e)
    for (int d = 0; d < 3; ++d) c[d] += (double)E[3 * e + d];
  for (int d = 0; d < 3; ++d) pos[d] = (float)(c[d] / 6.0);
  double M[9];
  for (int a = 0; a < 3; ++a)
    for (int d = 0; d < 3; ++d)
      M[d * 3 + a] = (double)(float)(0.5 * ((double)E[3 * (2 * a) + d] - (double)E[3 * (2 * a + 1) + d]));
  double R[9], K[3];
  polar_svd(M, R, K);
  for (int i = 0; i < 9; ++i) R[i] = (double)(float)R[i];
  double q[4];
  quat_from_matrix(R, q);
  normalize4(q);
  float qf[4];
  for (int i = 0; i < 4; ++i) qf[i] = (float)q[i];
  for (int d = 0; d < 3; ++d) {
    const float kf = (float)K[d];
    s_out[d] = kf / ((s0[d] + 1e-3f) * 2.0f) * s0[d];
  }
  double qn[4] = {qf[0], qf[1], qf[2], qf[3]};
  double qo[4] = {q_old[0], q_old[1], q_old[2], q_old[3]};
  const double nn = qo[0] * qo[0] + qo[1] * qo[1] + qo[2] * qo[2] + qo[3] * qo[3];
  double qi[4] = {qo[0] / nn, -qo[1] / nn, -qo[2] / nn, -qo[3] / nn};
  double qr[4];
  quat_mul(qn, qi, qr);
  normalize4(qr);
  double Rr[9];
  quat_to_matrix(qr, Rr);
  rotate_sh(sh_in, Rr, sh_out);
  for (int i = 0; i < 4; ++i) q_out[i] = qf[i];
  if (cov6) {
    double Rq[9];
    normalize4(qn);
    quat_to_matrix(qn, Rq);
    double s2[3];
    for (int d = 0; d < 3; ++d) s2[d] = (double)s_out[d] * (double)s_out[d];
    int o = 0;
    for (int r = 0; r < 3; ++r)
      for (int cc = r; cc < 3; ++cc)
        cov6[o++] = (float)(Rq[r * 3] * s2[0] * Rq[cc * 3] + Rq[r * 3 + 1] * s2[1] * Rq[cc * 3 + 1] +
                            Rq[r * 3 + 2] * s2[2] * Rq[cc * 3 + 2]);
  }
}

// FastgetOthogonalMatrix (helper.cpp:506-517): Newton polar iteration
// M <- (M + M^-T)/2 until max|dM| < 1e-6, keeping the iterate before the
// final update; then the normalised quaternion (float32).
void node_quaternion(const double* rot_cm, float q_out[4]) {
  double M[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) M[r * 3 + c] = (double)(float)rot_cm[c * 3 + r];
  for (int it = 0; it < 200; ++it) {
    const double a = M[0], b = M[1], c = M[2], d = M[3], e = M[4], f = M[5], g = M[6], h = M[7], i = M[8];
    const double A = e * i - f * h, Bv = -(d * i - f * g), Cv = d * h - e * g;
    const double det = a * A + b * Bv + c * Cv;
    // M^-T = cofactor / det
    const double cof[9] = {A, Bv, Cv, -(b * i - c * h), a * i - c * g, -(a * h - b * g),
                           b * f - c * e, -(a * f - c * d), a * e - b * d};
    double nxt[9], md = 0.0;
    for (int t = 0; t < 9; ++t) {
      nxt[t] = 0.5 * (M[t] + cof[t] / det);
      md = std::max(md, std::abs(M[t] - nxt[t]));
    }
    if (md < 1e-6) break;
    std::memcpy(M, nxt, sizeof(M));
  }
  double q[4];
  quat_from_matrix(M, q);
  normalize4(q);
  for (int t = 0; t < 4; ++t) q_out[t] = (float)q[t];
}

// Q_SlerpCUDA blend (cudakdtree.cu:113-148, 208-217) with float32 decisions.
void slerp_blend(const int32_t* idx, const float* w, int k, const float* quats, double out[4]) {
  double cur[4] = {1, 0, 0, 0};
  float last = 0.f;
  for (int j = 0; j < k; ++j) {
    const float cw = w[j];
    const double t = (double)(cw / (cw + last));
    double e[4];
    for (int i = 0; i < 4; ++i) e[i] = (double)quats[4 * (size_t)idx[j] + i];
    float c32[4], e32[4];
    for (int i = 0; i < 4; ++i) {
      c32[i] = (float)cur[i];
      e32[i] = (float)e[i];
    }
    float cosf_ = ((c32[1] * e32[1] + c32[2] * e32[2]) + c32[3] * e32[3]) + c32[0] * e32[0];
    double cs = (double)cosf_;
    if (cs < 0) {
      for (int i = 0; i < 4; ++i) e[i] = -e[i];
      cs = -cs;
    }
    double ra, rb;
    if (cs > (double)0.99995f) {
      ra = 1.0 - t;
      rb = t;
    } else {
      const double sn = std::sqrt(std::max(1.0 - cs * cs, 0.0));
      const double ang = std::atan2(sn, cs);
      ra = std::sin((1.0 - t) * ang) / sn;
      rb = std::sin(t * ang) / sn;
    }
    double nq[4];
    for (int i = 0; i < 4; ++i) nq[i] = (double)(float)(ra * (double)c32[i] + rb * e[i]);
    normalize4(nq);
    for (int i = 0; i < 4; ++i) cur[i] = nq[i];
    last = last + cw;
  }
  for (int i = 0; i < 4; ++i) out[i] = cur[i];
}

}  // namespace

// ------------------------------------------------------------------ ABI ----
extern "C" {

struct ocpu_solve_stats {
  int gn_iterations;
  int halvings;
  int status;  // 0 ok, 2 non-positive pivot, 3 bad input
  int n_free;
  long long n_rows;
  long long nnz_j;
  long long nnz_l_blocks;
  double factor_gflop;   // block-update flops of one factorisation
  int top_columns;       // columns factorised in the serial top phase
  int subtrees;
  double initial_energy, final_energy;
  double t_setup, t_analyse, t_jacobian, t_normal, t_factor, t_solve, t_line, t_total;
  double t_phase1, t_phase2;  // factorisation: parallel subtrees, serial top
};

// Deform::optimize restated: x0 = identity, max_iters Gauss-Newton
// iterations (early exit as Deform.cpp:165 when early_exit), rot_out [n][9]
// column-major and trans_out [n][3] in float64 (resetRT for the static nodes).
int ocpu_solve(int n, int k, const float* node_pos, const int32_t* nbr, const int32_t* aidx, const double* aw,
               const float* aims, int n_blocks, const int32_t* block_ptr, const int32_t* block_ids,
               const int32_t* block_type, int cons_on_center, float weighting_factor, float w_rot, float w_reg,
               float w_con, int max_iters, int early_exit, int nthreads, int ordering, double* rot_out,
               double* trans_out, ocpu_solve_stats* st) {
  const auto T0 = Clock::now();
  if (nthreads < 1) nthreads = omp_get_max_threads();
  omp_set_num_threads(nthreads);
  std::memset(st, 0, sizeof(*st));
  Problem P;
  if (make_problem(P, n, k, node_pos, nbr, aidx, aw, aims, n_blocks, block_ptr, block_ids, block_type,
                   cons_on_center, weighting_factor, w_rot, w_reg, w_con)) {
    st->status = 3;
    return 3;
  }
  const int F = P.F;
  const size_t nc = 12 * (size_t)F;
  std::vector<double> x(nc, 0.0), f(P.n_rows), f1(P.n_rows), g(nc), h(nc), xt(nc);
  for (int i = 0; i < F; ++i) x[12 * (size_t)i] = x[12 * (size_t)i + 4] = x[12 * (size_t)i + 8] = 1.0;
  Csr J;
  Csc T;
  BlockMatrix A;
  Factor L;
  const auto T1 = Clock::now();
  st->t_setup = secs(T0, T1);
  st->n_free = F;
  st->n_rows = P.n_rows;
  bool analysed = false;
  residual(P, x.data(), f.data());
  st->initial_energy = dot(f.data(), f.data(), f.size());
  int it = 0;
  for (; it < max_iters; ++it) {
    auto a = Clock::now();
    jacobian(P, x.data(), J);
    if (!analysed) transpose_pattern(J, T);
    auto b = Clock::now();
    st->t_jacobian += secs(a, b);
    if (!analysed) {
      a_pattern(J, F, A);
      std::vector<float> fx(3 * (size_t)F);
      for (int i = 0; i < F; ++i)
        for (int d = 0; d < 3; ++d) fx[3 * (size_t)i + d] = node_pos[3 * (size_t)P.free_ids[i] + d];
      analyse(A, fx.data(), ordering, L, nthreads);
      analysed = true;
      st->nnz_j = J.ptr[J.rows];
      st->nnz_l_blocks = (long long)L.loff[F];
      double fl = 0.0;
      for (int j = 0; j < F; ++j) {
        const double m = L.sptr[j + 1] - L.sptr[j] + 1;
        fl += m * (m + 1) / 2 * 2.0 * BB * B;
      }
      st->factor_gflop = fl * 1e-9;
      st->top_columns = (int)L.top_cols.size();
      st->subtrees = (int)L.sub_roots.size();
      auto c = Clock::now();
      st->t_analyse += secs(b, c);
      b = c;
    }
    a_numeric(J, T, A);
    residual(P, x.data(), f.data());
    jt_mul(J, T, f.data(), g.data());
    for (size_t i = 0; i < nc; ++i) g[i] = -g[i];
    auto c = Clock::now();
    st->t_normal += secs(b, c);
    if (!factorize(A, L, nthreads)) {
      st->status = 2;
      break;
    }
    auto d = Clock::now();
    st->t_factor += secs(c, d);
    solve(L, g.data(), h.data());
    auto e = Clock::now();
    st->t_solve += secs(d, e);
    const double normv = std::sqrt(dot(x.data(), x.data(), nc));
    const double old = dot(f.data(), f.data(), f.size());
    for (double alpha = 1.0; alpha > 1e-15; alpha *= 0.5) {
      for (size_t i = 0; i < nc; ++i) xt[i] = x[i] + h[i];
      residual(P, xt.data(), f1.data());
      if (dot(f1.data(), f1.data(), f1.size()) > old) {
        for (size_t i = 0; i < nc; ++i) h[i] *= 0.5;
        st->halvings++;
      } else {
        x.swap(xt);
        break;
      }
    }
    st->t_line += secs(e, Clock::now());
    if (early_exit && std::sqrt(dot(h.data(), h.data(), nc)) < (normv + 1e-6) * 1e-6) {
      ++it;
      break;
    }
  }
  st->gn_iterations = std::min(it, max_iters);
  residual(P, x.data(), f.data());
  st->final_energy = dot(f.data(), f.data(), f.size());
  for (int v = 0; v < n; ++v) {
    for (int t = 0; t < 9; ++t) rot_out[9 * (size_t)v + t] = (t % 4 == 0) ? 1.0 : 0.0;
    for (int t = 0; t < 3; ++t) trans_out[3 * (size_t)v + t] = 0.0;
  }
  for (int i = 0; i < F; ++i) {
    const int v = P.free_ids[i];
    for (int t = 0; t < 9; ++t) rot_out[9 * (size_t)v + t] = x[12 * (size_t)i + t];
    for (int t = 0; t < 3; ++t) trans_out[3 * (size_t)v + t] = x[12 * (size_t)i + 9 + t];
  }
  st->t_total = secs(T0, Clock::now());
  st->t_phase1 = g_t_phase1;
  st->t_phase2 = g_t_phase2;
  g_t_phase1 = g_t_phase2 = 0.0;
  return st->status;
}

// ED blend of P points (Deform.hpp:230-249); idx/w point-major [P][k]; w is
// float64 when w64 is given, else float32.
void ocpu_ed_blend(long long P, int k, const float* pts, const int32_t* idx, const double* w64, const float* w32,
                   const double* rot, const double* trans, const float* node_pos, float* out, int nthreads) {
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long long i = 0; i < P; ++i)
    ed_blend_one(pts + 3 * i, idx + (size_t)i * k, w32 ? w32 + (size_t)i * k : nullptr,
                 w64 ? w64 + (size_t)i * k : nullptr, k, rot, trans, node_pos, out + 3 * i);
}

// UpdatePosition's endpoint blend + UpdateAsSixPointsWithdrawBad for N
// Gaussians: ends [N][6][3] (updated in place), idx/w [N][6][k] float32
// weights; outputs pos [N][3], q [N][4] (q holds the old quaternion on
// input), scale [N][3], shs [N][48] (in place), cov6 [N][6] optional.
void ocpu_skin_gaussians(long long N, int k, float* ends, const int32_t* idx, const float* w, const double* rot,
                         const double* trans, const float* node_pos, const float* scale0, float* pos, float* q,
                         float* scale, float* shs, float* cov6, int nthreads) {
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long long i = 0; i < N; ++i) {
    float E[18];
    for (int e = 0; e < 6; ++e)
      ed_blend_one(ends + 18 * i + 3 * e, idx + ((size_t)i * 6 + e) * k, w + ((size_t)i * 6 + e) * k, nullptr, k,
                   rot, trans, node_pos, E + 3 * e);
    std::memcpy(ends + 18 * i, E, sizeof(E));
    float qo[4], sh[48];
    std::memcpy(qo, q + 4 * i, sizeof(qo));
    std::memcpy(sh, shs + 48 * i, sizeof(sh));
    refit_one(E, qo, scale0 + 3 * i, sh, pos + 3 * i, q + 4 * i, scale + 3 * i, shs + 48 * i,
              cov6 ? cov6 + 6 * i : nullptr);
  }
}

// UpdatePositionforSamples + FastUpdateSamplesSH for S samples: positions
// blended in place, node quaternions by the Newton polar iteration, the
// slerp blend of the k node quaternions, the 48-float feature rotated in
// place; idx/w [S][k] float32.
void ocpu_skin_samples(long long S, int k, int n_nodes, float* sample_pos, const int32_t* idx, const float* w,
                       const double* rot, const double* trans, const float* node_pos, float* feature,
                       int nthreads) {
  if (nthreads < 1) nthreads = omp_get_max_threads();
  std::vector<float> nq(4 * (size_t)n_nodes);
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int v = 0; v < n_nodes; ++v) node_quaternion(rot + 9 * (size_t)v, nq.data() + 4 * (size_t)v);
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long long i = 0; i < S; ++i) {
    float p[3];
    ed_blend_one(sample_pos + 3 * i, idx + (size_t)i * k, w + (size_t)i * k, nullptr, k, rot, trans, node_pos, p);
    sample_pos[3 * i] = p[0];
    sample_pos[3 * i + 1] = p[1];
    sample_pos[3 * i + 2] = p[2];
    double qb[4];
    slerp_blend(idx + (size_t)i * k, w + (size_t)i * k, k, nq.data(), qb);
    normalize4(qb);
    double R[9];
    quat_to_matrix(qb, R);
    float f[48];
    std::memcpy(f, feature + 48 * i, sizeof(f));
    rotate_sh(f, R, feature + 48 * i);
  }
}

// kNN skinning weights (Deform.hpp:187-208) by brute force over the nodes:
// the k+1 nearest by (float32 distance, index), w_j = (1 - d_j/d_{k+1})^2
// normalised, in float64.  idx [P][k], w [P][k].
void ocpu_knn_weights(long long P, const float* pts, int n, const float* nodes, int k, int32_t* idx_out,
                      double* w_out, int nthreads) {
  if (nthreads < 1) nthreads = omp_get_max_threads();
  const int kk = k + 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
  for (long long i = 0; i < P; ++i) {
    float bd[16];
    int bi[16];
    int m = 0;
    const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
    for (int v = 0; v < n; ++v) {
      const float dx = px - nodes[3 * (size_t)v], dy = py - nodes[3 * (size_t)v + 1], dz = pz - nodes[3 * (size_t)v + 2];
      const float d = std::sqrt((dx * dx + dy * dy) + dz * dz);
      if (m == kk && !(d < bd[kk - 1])) continue;
      int p = m < kk ? m++ : kk - 1;
      while (p > 0 && bd[p - 1] > d) {
        bd[p] = bd[p - 1];
        bi[p] = bi[p - 1];
        --p;
      }
      bd[p] = d;
      bi[p] = v;
    }
    const double dmax = bd[k];
    double ws[16], sum = 0.0;
    for (int j = 0; j < k; ++j) {
      const double r = 1.0 - (double)bd[j] / dmax;
      ws[j] = k == 1 ? 1.0 : r * r;
      sum += ws[j];
    }
    for (int j = 0; j < k; ++j) {
      idx_out[(size_t)i * k + j] = bi[j];
      w_out[(size_t)i * k + j] = k == 1 ? 1.0 : ws[j] / sum;
    }
  }
}

int ocpu_max_threads() { return omp_get_max_threads(); }

}  // extern "C"
