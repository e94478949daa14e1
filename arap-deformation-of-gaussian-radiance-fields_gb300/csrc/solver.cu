// Host side of the Gauss-Newton solver: solve-plan construction (the
// bookkeeping of the Deform constructor, Deform.hpp:414-455 and
// Deform.cpp:6-75) and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <set>
#include <vector>

#include "solver_kernel.cuh"

using namespace arap;

struct arap_solver {
  int n = 0, k = 0, F = 0, S = 0, G = 0, U = 0, n_items = 0, n_rows = 0;
  arap_solve_config cfg{};
  int grid = 0;
  void* block = nullptr;  // one device allocation holding everything below
  SolveParams P{};
  // a configured spin limit: the solve runs on the instance-table kernel as
  // a batch of one (its barrier waits read the limit); its parameters and
  // CTA range live here
  bool checked = false;
  void* self = nullptr;  // SolveParams, then int cta_first[2]
  std::vector<int32_t> free_host;
  std::vector<int32_t> order_host;  // processing order (free ranks)
  std::vector<int32_t> stage_cost;  // shared-memory bytes of each free node's tables
  std::vector<int32_t> res_cost;    // the same in resident mode (two-level PCG only; empty otherwise)
};

namespace {

struct Carver {
  char* base;
  size_t off = 0;
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += sizeof(T) * (count ? count : 1);
    return p;
  }
};

int bits_of(float f) {
  int i;
  std::memcpy(&i, &f, sizeof(i));
  return i;
}

template <typename RT>
int occupancy_grid(int per_sm_cap) {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gn_solve_kernel<RT>, kSolveThreads, 0) !=
      cudaSuccess)
    return -1;
  if (per_sm < 1) return -1;
  return sms * std::min(per_sm, per_sm_cap);
}

// Largest dynamic shared memory a CTA of kernel fn may take for its resident
// node tables: the device's per-block opt-in limit less the kernel's static
// shared memory and a reserve, and at most kStageMaxBytes so that L1 keeps
// room for the kernel's local memory.  The kernel's attribute is raised to it.
constexpr int kStageMaxBytes = 160 * 1024;
int stage_limit(const void* fn) {
  int dev = 0, optin = 0;
  cudaFuncAttributes fa{};
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  const int lim = std::min(optin - (int)fa.sharedSizeBytes - 1024, kStageMaxBytes) & ~15;
  if (lim <= 0) return 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return lim;
}

// Shared memory the tables of a solve need when its free nodes are dealt
// round-robin over nbk CTAs (the largest CTA share), uncapped; with NC > 0
// each CTA also holds its rows of the coarse inverse.
long long stage_need(const std::vector<int32_t>& order, const std::vector<int32_t>& cost, int nbk, int NC) {
  if (nbk <= 0) return 0;
  std::vector<long long> per(nbk, 0);
  for (int b = 0; b < nbk && NC > 0; ++b) per[b] = 4ll * NC * stage_coarse_rows(NC, b, nbk);
  for (size_t p = 0; p < order.size(); ++p) per[p % nbk] += cost[order[p]];
  long long need = 0;
  for (long long v : per) need = std::max(need, v);
  return (need + 15) & ~15ll;
}

// Staging of a solve on nbk CTAs under limit bytes: resident mode when every
// CTA's nodes fit with their PCG vectors, else as many nodes as fit.
struct StagePlan {
  int bytes = 0;
  int resident = 0;
};
StagePlan plan_stage(const arap_solver* s, int nbk, int limit) {
  StagePlan p;
  if (limit <= 0 || nbk <= 0) return p;
  if (!s->res_cost.empty()) {
    const long long need = stage_need(s->order_host, s->res_cost, nbk, s->P.NC);
    if (need <= limit) {
      p.bytes = (int)need;
      p.resident = 1;
      return p;
    }
  }
  p.bytes = (int)std::min<long long>(stage_need(s->order_host, s->stage_cost, nbk, 0), limit);
  return p;
}

}  // namespace

extern "C" int arap_solver_create(arap_solver** out, int n, int k, const int32_t* neighbors,
                                  const int32_t* anchor_idx, const float* anchor_w,
                                  const int32_t* block_offsets_host, const int32_t* block_nodes_host,
                                  const int32_t* block_type_host, int n_blocks,
                                  const arap_solve_config* cfg_in, arap_stream_t stream) {
  if (!out) return ARAP_EBADINPUT;
  *out = nullptr;
  if (n < 2 || k < 1 || k > ARAP_KNN_MAX || !neighbors || !anchor_idx || !anchor_w || n_blocks < 0 ||
      (n_blocks > 0 && (!block_offsets_host || !block_nodes_host || !block_type_host)))
    return ARAP_EBADINPUT;
  arap_solve_config cfg;
  if (cfg_in)
    cfg = *cfg_in;
  else
    arap_solve_config_default(&cfg);
  if (cfg.max_iters < 0) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;

  // inputs to host
  std::vector<int32_t> nb((size_t)n * k), aidx((size_t)n * k);
  std::vector<float> aw((size_t)n * k);
  ARAP_CUDA_TRY(cudaMemcpyAsync(nb.data(), neighbors, nb.size() * 4, cudaMemcpyDeviceToHost, st));
  ARAP_CUDA_TRY(cudaMemcpyAsync(aidx.data(), anchor_idx, aidx.size() * 4, cudaMemcpyDeviceToHost, st));
  ARAP_CUDA_TRY(cudaMemcpyAsync(aw.data(), anchor_w, aw.size() * 4, cudaMemcpyDeviceToHost, st));
  ARAP_CUDA_TRY(cudaStreamSynchronize(st));
  for (size_t i = 0; i < nb.size(); ++i)
    if (nb[i] < 0 || nb[i] >= n || aidx[i] < 0 || aidx[i] >= n) return ARAP_EBADINPUT;
  std::vector<std::vector<int32_t>> blocks(n_blocks);
  for (int b = 0; b < n_blocks; ++b) {
    const int a0 = block_offsets_host[b], a1 = block_offsets_host[b + 1];
    if (a0 < 0 || a1 < a0) return ARAP_EBADINPUT;
    for (int a = a0; a < a1; ++a) {
      if (block_nodes_host[a] < 0 || block_nodes_host[a] >= n) return ARAP_EBADINPUT;
      blocks[b].push_back(block_nodes_host[a]);
    }
  }

  // free / static sets (UpdateIndicies, GaussianView.cpp:2010-2035)
  std::vector<char> is_static(n, 0);
  for (int b = 0; b < n_blocks; ++b)
    if (block_type_host[b] < 0)
      for (int v : blocks[b]) is_static[v] = 1;
  std::vector<int32_t> rank(n, -1), free_ids;
  for (int i = 0; i < n; ++i)
    if (!is_static[i]) {
      rank[i] = (int32_t)free_ids.size();
      free_ids.push_back(i);
    }
  const int F = (int)free_ids.size();
  const int S = n - F;
  if (F == 0) return ARAP_EBADINPUT;

  // block membership for BelongsToSameBlock (Deform.cpp:20-32)
  std::vector<std::vector<int>> node_blocks(n);
  for (int b = 0; b < n_blocks; ++b)
    if (block_type_host[b] != -1)
      for (int v : blocks[b])
        if (node_blocks[v].empty() || node_blocks[v].back() != b) node_blocks[v].push_back(b);
  auto same_block = [&](int i, int j) {
    for (int a : node_blocks[i])
      for (int b : node_blocks[j])
        if (a == b) return true;
    return false;
  };
  const float wf = cfg.weighting_factor;

  // constraint groups (Deform.cpp:299-371 / 484-580)
  std::vector<int32_t> grp_off{0}, grp_member, tsrc_off{0}, tsrc;
  std::vector<float> grp_mult;
  for (int b = 0; b < n_blocks; ++b) {
    if (block_type_host[b] == -1) continue;
    if (!cfg.cons_on_center) {
      for (int c : blocks[b]) {
        grp_member.push_back(c);
        grp_off.push_back((int32_t)grp_member.size());
        tsrc.push_back(c);
        tsrc_off.push_back((int32_t)tsrc.size());
        grp_mult.push_back(1.f);
      }
    } else {
      // SelectKeyControls (Deform.cpp:34-75): the first min(20,|block|) ids,
      // as a set; the target is the mean of their aims
      const int m = std::min<int>(20, (int)blocks[b].size());
      if (m == 0) continue;
      std::set<int32_t> sel(blocks[b].begin(), blocks[b].begin() + m);
      for (int c : sel) grp_member.push_back(c);
      grp_off.push_back((int32_t)grp_member.size());
      for (int a = 0; a < m; ++a) tsrc.push_back(blocks[b][a]);
      tsrc_off.push_back((int32_t)tsrc.size());
      grp_mult.push_back((float)sel.size());
    }
  }
  const int G = (int)grp_mult.size();
  const int U = (int)grp_member.size();
  std::vector<int32_t> mem_rank((size_t)U * k), mem_node((size_t)U * k);
  std::vector<float> mem_w((size_t)U * k);
  for (int u = 0; u < U; ++u)
    for (int t = 0; t < k; ++t) {
      const int c = grp_member[u];
      const int l = aidx[(size_t)t * n + c];
      mem_node[(size_t)u * k + t] = l;
      mem_rank[(size_t)u * k + t] = rank[l];
      mem_w[(size_t)u * k + t] = aw[(size_t)t * n + c];
    }

  // coupling items per free node
  std::vector<std::vector<int4>> items(F);
  for (int r = 0; r < F; ++r) {
    const int j = free_ids[r];
    for (int t = 0; t < k; ++t) {
      const int kn = nb[(size_t)j * k + t];
      items[r].push_back(make_int4(ITEM_OUT, rank[kn], kn, bits_of(same_block(j, kn) ? wf : 1.f)));
    }
  }
  for (int i = 0; i < n; ++i)
    for (int t = 0; t < k; ++t) {
      const int j = nb[(size_t)i * k + t];
      if (rank[j] < 0) continue;
      if (rank[i] >= 0)
        items[rank[j]].push_back(make_int4(ITEM_IN, rank[i], i, bits_of(same_block(i, j) ? wf : 1.f)));
      else
        items[rank[j]].push_back(make_int4(ITEM_STATIC, -1, i, 0));
    }
  for (int g = 0; g < G; ++g)
    for (int u = grp_off[g]; u < grp_off[g + 1]; ++u)
      for (int t = 0; t < k; ++t) {
        const int l = mem_node[(size_t)u * k + t];
        if (rank[l] >= 0) items[rank[l]].push_back(make_int4(ITEM_CON, u * k + t, g, 0));
      }
  std::vector<int32_t> item_off(F + 1, 0);
  std::vector<int4> item_flat;
  for (int r = 0; r < F; ++r) {
    auto& v = items[r];
    std::stable_sort(v.begin(), v.end(), [](const int4& a, const int4& b) {
      if (a.x != b.x) return a.x < b.x;
      if (a.x == ITEM_CON) return a.z < b.z;
      return false;
    });
    item_flat.insert(item_flat.end(), v.begin(), v.end());
    item_off[r + 1] = (int32_t)item_flat.size();
  }

  // aggregates of the coarse space: breadth-first growth over the node graph
  // (both edge directions, free nodes only) up to coarse_nodes members; small
  // leftovers join their neighbouring aggregate
  std::vector<int32_t> agg(F, -1), pivot, agg_count;
  auto aggregate = [&](int target) {
    std::fill(agg.begin(), agg.end(), -1);
    pivot.clear();
    agg_count.clear();
    std::vector<std::vector<int32_t>> adj(F);
    for (int i = 0; i < n; ++i) {
      if (rank[i] < 0) continue;
      for (int t = 0; t < k; ++t) {
        const int j = nb[(size_t)i * k + t];
        if (rank[j] < 0) continue;
        adj[rank[i]].push_back(rank[j]);
        adj[rank[j]].push_back(rank[i]);
      }
    }
    std::vector<int32_t> queue;
    for (int seed = 0; seed < F; ++seed) {
      if (agg[seed] >= 0) continue;
      const int a = (int)pivot.size();
      pivot.push_back(free_ids[seed]);
      agg_count.push_back(0);
      queue.assign(1, seed);
      agg[seed] = a;
      agg_count[a] = 1;
      for (size_t q = 0; q < queue.size() && agg_count[a] < target; ++q)
        for (int v : adj[queue[q]]) {
          if (agg[v] >= 0) continue;
          agg[v] = a;
          queue.push_back(v);
          if (++agg_count[a] >= target) break;
        }
    }
    // merge aggregates below a quarter of the target into a neighbour
    const int NA0 = (int)pivot.size();
    std::vector<int32_t> remap(NA0);
    for (int a = 0; a < NA0; ++a) remap[a] = a;
    for (int r = 0; r < F; ++r) {
      const int a = agg[r];
      if (agg_count[a] >= target / 4 || remap[a] != a) continue;
      for (int v : adj[r]) {
        const int b = remap[agg[v]];
        if (b != a && agg_count[b] >= target / 4) {
          remap[a] = b;
          agg_count[b] += agg_count[a];
          agg_count[a] = 0;
          break;
        }
      }
    }
    std::vector<int32_t> newid(NA0, -1), piv2, cnt2;
    for (int a = 0; a < NA0; ++a) {
      int b = a;
      while (remap[b] != b) b = remap[b];
      if (newid[b] < 0) {
        newid[b] = (int32_t)piv2.size();
        piv2.push_back(pivot[b]);
        cnt2.push_back(0);
      }
      newid[a] = newid[b];
    }
    for (int r = 0; r < F; ++r) {
      agg[r] = newid[agg[r]];
      cnt2[agg[r]] += 1;
    }
    pivot.swap(piv2);
    agg_count.swap(cnt2);
  };
  if (cfg.coarse_nodes > 0 && F > cfg.coarse_nodes) {
    int target = cfg.coarse_nodes;
    aggregate(target);
    while ((int)pivot.size() > kMaxCoarseAggs) {
      target += (target + 3) / 4;
      aggregate(target);
    }
  }
  const int NA = (int)pivot.size();
  const int NC = 12 * NA;
  // cost of each node for the processing order, from the unpatched kinds
  std::vector<long long> node_cost(F, 16);
  for (int r = 0; r < F; ++r)
    for (int t = item_off[r]; t < item_off[r + 1]; ++t)
      node_cost[r] += item_flat[t].x == ITEM_CON ? 1 + (grp_off[item_flat[t].z + 1] - grp_off[item_flat[t].z]) * k : 2;
  // aggregate of the other node in each coupling item, and of each anchor
  std::vector<int32_t> mem_agg((size_t)U * k, -1);
  if (NA > 0) {
    for (size_t q = 0; q < mem_agg.size(); ++q)
      if (mem_rank[q] >= 0) mem_agg[q] = agg[mem_rank[q]];
    for (auto& it4 : item_flat)
      if ((it4.x == ITEM_OUT || it4.x == ITEM_IN) && it4.y >= 0) it4.x |= agg[it4.y] << 4;
  }
  // per group: the distinct aggregates of its free anchors
  std::vector<int32_t> gca_off{0}, gca;
  if (NA > 0) {
    for (int g = 0; g < G; ++g) {
      const size_t first = gca.size();
      for (int u = grp_off[g]; u < grp_off[g + 1]; ++u)
        for (int t = 0; t < k; ++t) {
          const int rk = mem_rank[(size_t)u * k + t];
          if (rk < 0) continue;
          if (std::find(gca.begin() + first, gca.end(), agg[rk]) == gca.end()) gca.push_back(agg[rk]);
        }
      gca_off.push_back((int32_t)gca.size());
    }
  }
  // coarse-list entries and constraint items of each node, and the shared
  // memory of its tables
  // and, with a coarse level, the distinct aggregates coupled to it (its own,
  // its regularisation neighbours', its constraint groups')
  std::vector<int4> con_info(F, make_int4(0, 0, 0, 0));
  std::vector<int32_t> stage_cost(F, 0), res_cost;
  if (NA > 0) res_cost.assign(F, 0);
  std::vector<int32_t> coupled;
  for (int r = 0; r < F; ++r) {
    const int items_r = item_off[r + 1] - item_off[r];
    coupled.clear();
    if (NA > 0) coupled.push_back(agg[r]);
    for (int t = item_off[r]; t < item_off[r + 1]; ++t) {
      if (NA == 0) continue;
      const int4 m = item_flat[t];
      const int kind = m.x & 15;
      if ((kind == ITEM_OUT || kind == ITEM_IN) && m.y >= 0) coupled.push_back(agg[m.y]);
      if (kind == ITEM_CON) {
        con_info[r].x += gca_off[m.z + 1] - gca_off[m.z];
        con_info[r].y += 1;
        con_info[r].w += (grp_off[m.z + 1] - grp_off[m.z]) * k;
        for (int f = gca_off[m.z]; f < gca_off[m.z + 1]; ++f) coupled.push_back(gca[f]);
      }
    }
    std::sort(coupled.begin(), coupled.end());
    con_info[r].z = (int)(std::unique(coupled.begin(), coupled.end()) - coupled.begin());
    stage_cost[r] = stage_node_bytes(items_r, con_info[r].x, con_info[r].y, con_info[r].z, con_info[r].w, false);
    if (NA > 0)
      res_cost[r] = stage_node_bytes(items_r, con_info[r].x, con_info[r].y, con_info[r].z, con_info[r].w, true);
  }

  auto* s = new (std::nothrow) arap_solver();
  if (!s) return ARAP_ENOMEM;
  s->n = n;
  s->k = k;
  s->F = F;
  s->S = S;
  s->G = G;
  s->U = U;
  s->n_items = (int)item_flat.size();
  s->n_rows = F * (6 + 3 * k) + S * 3 * k + 3 * G;
  s->cfg = cfg;
  s->free_host = free_ids;
  if (s->cfg.pcg_tol <= 0.f) s->cfg.pcg_tol = cfg.precision == ARAP_PRECISION_MIXED ? 1e-6f : 1e-6f;
  if (s->cfg.pcg_max_iters <= 0) s->cfg.pcg_max_iters = 2000;
  if (s->cfg.coarse_reuse == 0.f) s->cfg.coarse_reuse = 0.05f;
  const int grid = cfg.precision == ARAP_PRECISION_MIXED ? occupancy_grid<ff>(2) : occupancy_grid<float>(2);
  if (grid <= 0) {
    delete s;
    return ARAP_ECUDA;
  }
  s->grid = std::min(grid, kMaxGridCtas);
  s->checked = cfg.spin_limit > 0;

  // device layout
  auto carve = [&](Carver& cv, SolveParams& P) {
    P.free_ids = cv.take<int32_t>(F);
    P.rank = cv.take<int32_t>(n);
    P.item_off = cv.take<int32_t>(F + 1);
    P.items = cv.take<int4>(item_flat.size());
    P.grp_off = cv.take<int32_t>(G + 1);
    P.grp_member = cv.take<int32_t>(U);
    P.grp_mult = cv.take<float>(G);
    P.tsrc_off = cv.take<int32_t>(G + 1);
    P.tsrc = cv.take<int32_t>(tsrc.size());
    P.mem_rank = cv.take<int32_t>((size_t)U * k);
    P.mem_node = cv.take<int32_t>((size_t)U * k);
    P.mem_w = cv.take<float>((size_t)U * k);
    P.mem_geo = cv.take<float4>((size_t)U * k);
    P.grp_target = cv.take<float4>(G);
    P.grp_f = cv.take<double>((size_t)3 * G);
    P.item_cq = cv.take<float4>(item_flat.size());
    P.x = cv.take<double>((size_t)F * 12);
    P.xf = cv.take<float>((size_t)F * 12);
    P.xo = cv.take<float2>((size_t)F * 12);
    P.h = cv.take<float>((size_t)F * 12);
    P.r = cv.take<float>((size_t)F * 12);
    P.z = cv.take<float>((size_t)F * 12);
    P.p0 = cv.take<float>((size_t)F * 12);
    P.p1 = cv.take<float>((size_t)F * 12);
    P.q = cv.take<float>((size_t)F * 12);
    P.u = cv.take<float>((size_t)F * 12);
    P.dinv = cv.take<float>((size_t)F * 144);
    P.order = cv.take<int32_t>(F);
    P.agg = cv.take<int32_t>(F);
    P.pivot = cv.take<int32_t>(NA);
    P.agg_count = cv.take<int32_t>(NA);
    P.Qd = cv.take<double>((size_t)NA * NA * 16);
    P.Cw = cv.take<float>((size_t)2 * NC * NC);
    P.rotagg = cv.take<double>((size_t)2 * NA * 81);
    P.Cinv = cv.take<float>((size_t)NC * NC);
    P.rc = cv.take<double>((size_t)2 * NC);
    P.zc = cv.take<float>(NC);
    P.mem_agg = cv.take<int32_t>((size_t)U * k);
    P.dpiv = cv.take<float4>(NA ? F : 0);
    P.gca_off = cv.take<int32_t>(NA ? G + 1 : 0);
    P.gca = cv.take<int32_t>(gca.size());
    P.gcv = cv.take<float4>(gca.size());
    P.uzg = cv.take<float4>(NA ? G : 0);
    P.con_info = cv.take<int4>(F);
    P.partials = cv.take<double>((size_t)2 * kReduceSlots * grid);
    P.stats = cv.take<double>(kStatSlots);
    P.bar = cv.take<GridBarrier>(1);
  };
  Carver sizing{nullptr};
  SolveParams dummy{};
  carve(sizing, dummy);
  if (cudaMalloc(&s->block, sizing.off + 256) != cudaSuccess) {
    (void)cudaGetLastError();
    delete s;
    return ARAP_ENOMEM;
  }
  Carver cv{static_cast<char*>(s->block)};
  SolveParams& P = s->P;
  carve(cv, P);
  auto up = [&](const void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice, st) : cudaSuccess;
  };
  cudaError_t e = cudaSuccess;
  e = e ? e : up(P.free_ids, free_ids.data(), free_ids.size() * 4);
  e = e ? e : up(P.rank, rank.data(), rank.size() * 4);
  e = e ? e : up(P.item_off, item_off.data(), item_off.size() * 4);
  e = e ? e : up(P.items, item_flat.data(), item_flat.size() * sizeof(int4));
  e = e ? e : up(P.grp_off, grp_off.data(), grp_off.size() * 4);
  e = e ? e : up(P.grp_member, grp_member.data(), grp_member.size() * 4);
  e = e ? e : up(P.grp_mult, grp_mult.data(), grp_mult.size() * 4);
  e = e ? e : up(P.tsrc_off, tsrc_off.data(), tsrc_off.size() * 4);
  e = e ? e : up(P.tsrc, tsrc.data(), tsrc.size() * 4);
  e = e ? e : up(P.mem_rank, mem_rank.data(), mem_rank.size() * 4);
  e = e ? e : up(P.mem_node, mem_node.data(), mem_node.size() * 4);
  e = e ? e : up(P.mem_w, mem_w.data(), mem_w.size() * 4);
  // processing order: costliest nodes first; the kernel deals order position
  // p to CTA p % grid, so every SM gets its share of the expensive nodes
  std::vector<int32_t> order(F);
  {
    std::vector<std::pair<long long, int>> cost(F);
    for (int r = 0; r < F; ++r) cost[r] = {-node_cost[r], r};
    std::sort(cost.begin(), cost.end());
    for (int i = 0; i < F; ++i) order[i] = cost[i].second;
  }
  e = e ? e : up(P.order, order.data(), order.size() * 4);
  e = e ? e : up(P.con_info, con_info.data(), con_info.size() * sizeof(int4));
  if (NA > 0) {
    e = e ? e : up(P.mem_agg, mem_agg.data(), mem_agg.size() * 4);
    e = e ? e : up(P.agg, agg.data(), agg.size() * 4);
    e = e ? e : up(P.pivot, pivot.data(), pivot.size() * 4);
    e = e ? e : up(P.agg_count, agg_count.data(), agg_count.size() * 4);
    e = e ? e : up(P.gca_off, gca_off.data(), gca_off.size() * 4);
    e = e ? e : up(P.gca, gca.data(), gca.size() * 4);
  }
  // the barrier record: count, failed and status zeroed, the configured spin limit
  const GridBarrier bar0{0u, 0, (unsigned int)(cfg.spin_limit > 0 ? cfg.spin_limit : kSpinLimit), 0};
  e = e ? e : cudaMemcpyAsync(P.bar, &bar0, sizeof(bar0), cudaMemcpyHostToDevice, st);
  const int cta_range[2] = {0, s->grid};
  if (s->checked && e == cudaSuccess) {
    e = cudaMalloc(&s->self, sizeof(SolveParams) + sizeof(cta_range));
    e = e ? e
          : cudaMemcpyAsync(static_cast<char*>(s->self) + sizeof(SolveParams), cta_range, sizeof(cta_range),
                            cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    cudaFree(s->block);
    if (s->self) cudaFree(s->self);
    delete s;
    return ARAP_ECUDA;
  }
  P.n = n;
  P.k = k;
  P.F = F;
  P.G = G;
  P.U = U;
  P.n_items = (int)item_flat.size();
  P.wr = std::sqrt((double)cfg.w_rot);
  P.wg = std::sqrt((double)cfg.w_reg);
  P.wc = std::sqrt((double)cfg.w_con);
  P.wrf = (float)P.wr;
  P.wgf = (float)P.wg;
  P.wcf = (float)P.wc;
  P.wr_lo = (float)(P.wr - (double)P.wrf);
  P.wg_lo = (float)(P.wg - (double)P.wgf);
  P.wc_lo = (float)(P.wc - (double)P.wcf);
  P.wf = wf;
  P.max_iters = cfg.max_iters;
  P.early_exit = cfg.early_exit;
  P.pcg_max = s->cfg.pcg_max_iters;
  P.pcg_tol = s->cfg.pcg_tol;
  P.coarse_reuse = s->cfg.coarse_reuse > 0.f ? s->cfg.coarse_reuse : 0.f;
  P.mode = 0;
  P.refine = 0;
  P.NA = NA;
  P.NC = NC;
  s->order_host = order;
  s->stage_cost = stage_cost;
  s->res_cost = res_cost;
  {
    const bool mixed = cfg.precision == ARAP_PRECISION_MIXED;
    const void* fn = s->checked ? (mixed ? (const void*)gn_solve_batch_kernel<ff>
                                         : (const void*)gn_solve_batch_kernel<float>)
                                : (mixed ? (const void*)gn_solve_kernel<ff> : (const void*)gn_solve_kernel<float>);
    const StagePlan sp = plan_stage(s, s->grid, stage_limit(fn));
    P.stage_cap = sp.bytes;
    P.resident = sp.resident;
  }
  *out = s;
  return ARAP_OK;
}

// Read and clear the status word and the timeout flag of a solve's barrier
// record (synchronises): the status word's code, else ARAP_ETIMEOUT when a
// barrier wait gave up.
static int read_solver_status(GridBarrier* bar, cudaStream_t st) {
  int failed = 0;
  if (cudaMemcpyAsync(&failed, &bar->failed, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemsetAsync(&bar->failed, 0, sizeof(int), st) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  const int code = status_read_clear(&bar->status, st);  // synchronises
  if (code != ARAP_OK) return code;
  return failed ? ARAP_ETIMEOUT : ARAP_OK;
}

// Host stats of one solve from its device slots; returns the call's status
// (ARAP_NOT_CONVERGED is reported in the stats only).
static int fill_stats(const arap_solver* s, const double* st8, int dev_status, arap_solve_stats* stats_host) {
  std::memset(stats_host, 0, sizeof(*stats_host));
  stats_host->gn_iterations = (int)st8[ST_ITERS];
  stats_host->pcg_iterations = (int)st8[ST_PCG];
  stats_host->halvings = (int)st8[ST_HALV];
  stats_host->initial_energy = st8[ST_E0];
  stats_host->final_energy = st8[ST_E];
  stats_host->n_free = s->F;
  stats_host->n_static = s->S;
  stats_host->n_rows = s->n_rows;
  for (int q = 0; q < 9; ++q) stats_host->phase_ms[q] = st8[ST_T_PREP + q] * 1e-6;
  stats_host->n_coarse = s->P.NC;
  stats_host->resident = s->P.resident ? 1 : 0;
  stats_host->coarse_fallbacks = (int)st8[ST_CFALL];
  stats_host->coarse_inversions = (int)st8[ST_CINV_N];
  {
    const int n_it = std::min((int)st8[ST_ITERS], kHalvIters);
    for (int it = 0; it < n_it; ++it)
      stats_host->iteration_halvings[it] = (int)(st8[ST_HALV_IT + it] - (it ? st8[ST_HALV_IT + it - 1] : 0.0));
  }
  int status = dev_status;
  if (status == ARAP_OK && s->cfg.early_exit && st8[ST_CONV] == 0.0 && s->cfg.max_iters > 0)
    status = ARAP_NOT_CONVERGED;
  stats_host->status = status;
  return status == ARAP_NOT_CONVERGED ? ARAP_OK : status;
}

// The parameters of a checked solve into its device copy, in stream order
// (a kernel argument, so that a captured graph replays the values of its
// capture).
__global__ void put_params_kernel(SolveParams P, SolveParams* dst) {
  if (threadIdx.x == 0) *dst = P;
}

static int launch_solver(arap_solver* s, cudaStream_t st) {
  // count and failed (the first 8 bytes); the spin limit stays
  if (cudaMemsetAsync(s->P.bar, 0, 2 * sizeof(int), st) != cudaSuccess) return ARAP_ECUDA;
  cudaError_t e;
  if (s->checked) {
    SolveParams* dp = static_cast<SolveParams*>(s->self);
    int* cta = reinterpret_cast<int*>(static_cast<char*>(s->self) + sizeof(SolveParams));
    int one = 1;
    put_params_kernel<<<1, 32, 0, st>>>(s->P, dp);
    void* bargs[] = {&dp, &cta, &one};
    const void* fn = s->cfg.precision == ARAP_PRECISION_MIXED ? (const void*)gn_solve_batch_kernel<ff>
                                                              : (const void*)gn_solve_batch_kernel<float>;
    e = cudaLaunchCooperativeKernel(fn, s->grid, kSolveThreads, bargs, (size_t)s->P.stage_cap, st);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return ARAP_ECUDA;
    }
    return ARAP_OK;
  }
  void* args[] = {&s->P};
  if (s->cfg.precision == ARAP_PRECISION_MIXED)
    e = cudaLaunchCooperativeKernel((const void*)gn_solve_kernel<ff>, s->grid, kSolveThreads, args,
                                    (size_t)s->P.stage_cap, st);
  else
    e = cudaLaunchCooperativeKernel((const void*)gn_solve_kernel<float>, s->grid, kSolveThreads, args,
                                    (size_t)s->P.stage_cap, st);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  return ARAP_OK;
}

extern "C" int arap_solver_solve(arap_solver* s, const float* node_pos, const float* aims, float* rot_out,
                                 float* trans_out, arap_solve_stats* stats_host, arap_stream_t stream) {
  if (!s || !node_pos || !aims || !rot_out || !trans_out) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  s->P.node_pos = node_pos;
  s->P.aims = aims;
  s->P.rot_out = rot_out;
  s->P.trans_out = trans_out;
  s->P.mode = 0;
  s->P.x_in = nullptr;
  s->P.grad_out = nullptr;
  int rc = launch_solver(s, st);
  if (rc != ARAP_OK) return rc;
  if (!stats_host) return ARAP_OK;
  double st8[kStatSlots];
  ARAP_CUDA_TRY(cudaMemcpyAsync(st8, s->P.stats, sizeof(st8), cudaMemcpyDeviceToHost, st));
  const int dev_status = read_solver_status(s->P.bar, st);  // synchronises
  return fill_stats(s, st8, dev_status, stats_host);
}

extern "C" int arap_solver_energy_grad(arap_solver* s, const float* node_pos, const float* aims, const double* x,
                                       double* grad_out, double* energy_host, arap_stream_t stream) {
  if (!s || !node_pos || !aims || !x || !grad_out) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  SolveParams saved = s->P;
  s->P.node_pos = node_pos;
  s->P.aims = aims;
  s->P.mode = 1;
  s->P.x_in = x;
  s->P.grad_out = grad_out;
  s->P.max_iters = 1;
  int rc = launch_solver(s, st);
  const SolveParams used = s->P;
  s->P = saved;
  s->P.node_pos = used.node_pos;
  s->P.aims = used.aims;
  if (rc != ARAP_OK) return rc;
  if (energy_host) {
    double st8[kStatSlots];
    ARAP_CUDA_TRY(cudaMemcpyAsync(st8, used.stats, sizeof(st8), cudaMemcpyDeviceToHost, st));
    const int dev_status = read_solver_status(used.bar, st);
    *energy_host = st8[ST_E];
    return dev_status;
  }
  return ARAP_OK;
}

extern "C" int arap_solver_status(arap_solver* s, arap_stream_t stream) {
  if (!s) return ARAP_EBADINPUT;
  return read_solver_status(s->P.bar, (cudaStream_t)stream);
}

extern "C" int arap_solver_free_count(const arap_solver* s) { return s ? s->F : -1; }

extern "C" int arap_solver_free_ids(const arap_solver* s, int32_t* free_ids_host) {
  if (!s || !free_ids_host) return ARAP_EBADINPUT;
  std::memcpy(free_ids_host, s->free_host.data(), s->free_host.size() * 4);
  return ARAP_OK;
}

extern "C" void arap_solver_destroy(arap_solver* s) {
  if (!s) return;
  if (s->block) cudaFree(s->block);
  if (s->self) cudaFree(s->self);
  delete s;
}

// ------------------------------------------------------------ batches ----
struct arap_solver_batch {
  std::vector<arap_solver*> solvers;
  int precision = 0;
  int grid = 0;                 // co-resident CTAs of the batched kernel
  float exponent = 1.f;         // CTA share ~ (coupling items + free nodes)^exponent
  // Waves: launches that each run a group of instances on the whole grid.
  // Instances whose nodes fit in shared memory on some number of CTAs (the
  // resident two-level PCG) are packed into waves by that minimum, largest
  // first; the others share one wave.  Position p of the parameter array is
  // instance order[p]; wave w covers positions wave_first[w] ..
  // wave_first[w+1]-1, and its CTA ranges are cta_local[wave_first[w] + w ..]
  // (n_w + 1 entries).
  std::vector<int> order, wave_first, cta_local, wave_cap;
  std::vector<int> ctas;        // per instance: its CTAs
  std::vector<size_t> part_off; // per instance: offset of its barrier partials
  int stage_limit = 0;          // shared-memory limit of the batched kernel's resident tables
  std::vector<int> resident;    // per instance: resident mode (see plan_stage)
  void* block = nullptr;        // device: params, cta_first, barriers, partials
  SolveParams* d_params = nullptr;
  int* d_cta_first = nullptr;
  GridBarrier* d_bars = nullptr;
  double* d_partials = nullptr;
  SolveParams* h_params = nullptr;  // pinned staging of the parameter array
  cudaEvent_t staged{};             // the last upload of h_params has been read
  bool staged_valid = false;
};

namespace {

// Fewest CTAs on which solver s runs resident (all its nodes, with their PCG
// vectors, in shared memory), or -1 when no share of the grid suffices.
int resident_min_ctas(const arap_solver* s, int grid, int limit) {
  if (s->res_cost.empty() || !plan_stage(s, grid, limit).resident) return -1;
  int lo = 1, hi = grid;  // resident at hi; more CTAs never hurt
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (plan_stage(s, mid, limit).resident)
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

// Adds the grid's spare CTAs to the instances of one wave in proportion to
// their work estimate raised to the exponent (largest remainders).
void share_spare(const arap_solver_batch* b, const std::vector<int>& inst, std::vector<int>& n, int spare) {
  const int m = (int)inst.size();
  if (m == 0 || spare <= 0) return;
  std::vector<double> w(m);
  double sum = 0.0;
  for (int q = 0; q < m; ++q) {
    const arap_solver* s = b->solvers[inst[q]];
    w[q] = std::pow((double)(s->n_items + s->F) + 1.0, (double)b->exponent);
    sum += w[q];
  }
  std::vector<std::pair<double, int>> rem(m);
  int given = 0;
  for (int q = 0; q < m; ++q) {
    const double share = spare * w[q] / sum;
    const int whole = (int)std::floor(share);
    n[q] += whole;
    given += whole;
    rem[q] = {-(share - whole), q};
  }
  std::sort(rem.begin(), rem.end());
  for (int q = 0; q < spare - given; ++q) n[rem[q % m].second] += 1;
}

// Waves and CTA ranges of a batch (see arap_solver_batch).
void split_ctas(arap_solver_batch* b) {
  const int count = (int)b->solvers.size();
  std::vector<int> need(count);
  std::vector<int> res_inst, other;
  for (int i = 0; i < count; ++i) {
    need[i] = resident_min_ctas(b->solvers[i], b->grid, b->stage_limit);
    (need[i] > 0 ? res_inst : other).push_back(i);
  }
  std::stable_sort(res_inst.begin(), res_inst.end(), [&](int x, int y) { return need[x] > need[y]; });
  // first fit, largest first
  std::vector<std::vector<int>> waves;
  std::vector<int> used;
  for (int i : res_inst) {
    size_t w = 0;
    while (w < waves.size() && used[w] + need[i] > b->grid) ++w;
    if (w == waves.size()) {
      waves.emplace_back();
      used.push_back(0);
    }
    waves[w].push_back(i);
    used[w] += need[i];
  }
  if (!other.empty()) {
    waves.push_back(other);
    used.push_back(0);
  }
  b->order.clear();
  b->wave_first.assign(1, 0);
  b->cta_local.clear();
  b->wave_cap.clear();
  b->ctas.assign(count, 0);
  b->resident.assign(count, 0);
  b->part_off.assign(count, 0);
  size_t poff = 0;
  for (auto& wv : waves) {
    std::vector<int> n(wv.size());
    int base = 0;
    for (size_t q = 0; q < wv.size(); ++q) {
      n[q] = need[wv[q]] > 0 ? need[wv[q]] : 1;
      base += n[q];
    }
    share_spare(b, wv, n, b->grid - base);
    int cap = 0, first = 0;
    b->cta_local.push_back(0);
    for (size_t q = 0; q < wv.size(); ++q) {
      const int i = wv[q];
      const StagePlan sp = plan_stage(b->solvers[i], n[q], b->stage_limit);
      cap = std::max(cap, sp.bytes);
      b->resident[i] = sp.resident;
      b->ctas[i] = n[q];
      b->part_off[i] = poff;
      poff += (size_t)2 * kReduceSlots * n[q];
      b->order.push_back(i);
      first += n[q];
      b->cta_local.push_back(first);
    }
    b->wave_cap.push_back(cap);
    b->wave_first.push_back((int)b->order.size());
  }
}

// The CTA ranges go to the device when they change (creation, autotuning),
// never inside a solve, so a solve can be captured in a CUDA graph.
int upload_ctas(arap_solver_batch* b) {
  if (cudaMemcpy(b->d_cta_first, b->cta_local.data(), sizeof(int) * b->cta_local.size(), cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  return ARAP_OK;
}

template <typename RT>
int batch_grid() {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gn_solve_batch_kernel<RT>, kSolveThreads, 0) !=
      cudaSuccess || per_sm < 1)
    return -1;
  return std::min(sms * std::min(per_sm, 2), kMaxGridCtas);
}

}  // namespace

extern "C" int arap_solver_batch_create(arap_solver_batch** out, arap_solver* const* solvers, int count,
                                        float balance_exponent, arap_stream_t stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (!out || !solvers || count < 1) return ARAP_EBADINPUT;
  *out = nullptr;
  for (int i = 0; i < count; ++i)
    if (!solvers[i] || solvers[i]->cfg.precision != solvers[0]->cfg.precision) return ARAP_EBADINPUT;
  auto* b = new (std::nothrow) arap_solver_batch();
  if (!b) return ARAP_ENOMEM;
  b->solvers.assign(solvers, solvers + count);
  b->precision = solvers[0]->cfg.precision;
  b->grid = b->precision == ARAP_PRECISION_MIXED ? batch_grid<ff>() : batch_grid<float>();
  if (b->grid <= 0) {
    delete b;
    return ARAP_ECUDA;
  }
  if (count > b->grid) {
    delete b;
    return ARAP_EUNSUPPORTED;
  }
  b->exponent = balance_exponent > 0.f ? balance_exponent : 1.f;
  b->stage_limit = stage_limit(b->precision == ARAP_PRECISION_MIXED ? (const void*)gn_solve_batch_kernel<ff>
                                                                    : (const void*)gn_solve_batch_kernel<float>);
  split_ctas(b);
  Carver sizing{nullptr};
  auto carve = [&](Carver& cv) {
    b->d_params = cv.take<SolveParams>(count);
    b->d_cta_first = cv.take<int>(2 * count);
    b->d_bars = cv.take<GridBarrier>(count);
    b->d_partials = cv.take<double>((size_t)2 * kReduceSlots * b->grid * count);
  };
  carve(sizing);
  if (cudaMalloc(&b->block, sizing.off + 256) != cudaSuccess ||
      cudaMallocHost(reinterpret_cast<void**>(&b->h_params), sizeof(SolveParams) * count) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming) != cudaSuccess) {
    (void)cudaGetLastError();
    arap_solver_batch_destroy(b);
    return ARAP_ENOMEM;
  }
  Carver cv{static_cast<char*>(b->block)};
  carve(cv);
  {
    std::vector<GridBarrier> bars(count);
    for (int i = 0; i < count; ++i) {
      const int lim = solvers[i]->cfg.spin_limit;
      bars[i] = GridBarrier{0u, 0, (unsigned int)(lim > 0 ? lim : kSpinLimit), 0};
    }
    if (cudaMemcpyAsync(b->d_bars, bars.data(), sizeof(GridBarrier) * count, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      (void)cudaGetLastError();
      arap_solver_batch_destroy(b);
      return ARAP_ECUDA;
    }
  }
  if (upload_ctas(b) != ARAP_OK) {
    arap_solver_batch_destroy(b);
    return ARAP_ECUDA;
  }
  *out = b;
  return ARAP_OK;
}

extern "C" int arap_solver_batch_solve(arap_solver_batch* b, const float* const* node_pos, const float* const* aims,
                                       float* const* rot_out, float* const* trans_out, arap_solve_stats* stats_host,
                                       arap_stream_t stream) {
  if (!b || !node_pos || !aims || !rot_out || !trans_out) return ARAP_EBADINPUT;
  const int count = (int)b->solvers.size();
  for (int i = 0; i < count; ++i)
    if (!node_pos[i] || !aims[i] || !rot_out[i] || !trans_out[i]) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  ARAP_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
  // the previous upload of the staging array must have been read before it is rewritten
  if (b->staged_valid && cap == cudaStreamCaptureStatusNone) ARAP_CUDA_TRY(cudaEventSynchronize(b->staged));
  std::vector<int> wave_of(count, 0);
  for (size_t w = 0; w + 1 < b->wave_first.size(); ++w)
    for (int p = b->wave_first[w]; p < b->wave_first[w + 1]; ++p) wave_of[b->order[p]] = (int)w;
  for (int p = 0; p < count; ++p) {
    const int i = b->order[p];
    SolveParams P = b->solvers[i]->P;
    P.node_pos = node_pos[i];
    P.aims = aims[i];
    P.rot_out = rot_out[i];
    P.trans_out = trans_out[i];
    P.mode = 0;
    P.x_in = nullptr;
    P.grad_out = nullptr;
    P.bar = b->d_bars + i;
    P.partials = b->d_partials + b->part_off[i];
    P.stage_cap = b->wave_cap[wave_of[i]];
    P.resident = b->resident[i];
    b->h_params[p] = P;
  }
  ARAP_CUDA_TRY(cudaMemcpyAsync(b->d_params, b->h_params, sizeof(SolveParams) * count, cudaMemcpyHostToDevice, st));
  if (cap == cudaStreamCaptureStatusNone) {
    ARAP_CUDA_TRY(cudaEventRecord(b->staged, st));
    b->staged_valid = true;
  }
  // count and failed of every instance's barrier (the first 8 bytes of each)
  ARAP_CUDA_TRY(cudaMemset2DAsync(b->d_bars, sizeof(GridBarrier), 0, 2 * sizeof(int), count, st));
  const void* fn = b->precision == ARAP_PRECISION_MIXED ? (const void*)gn_solve_batch_kernel<ff>
                                                        : (const void*)gn_solve_batch_kernel<float>;
  for (size_t w = 0; w + 1 < b->wave_first.size(); ++w) {
    const int p0 = b->wave_first[w];
    int nw = b->wave_first[w + 1] - p0;
    const SolveParams* prm = b->d_params + p0;
    const int* cf = b->d_cta_first + p0 + (int)w;
    const int grid = b->cta_local[p0 + (int)w + nw];
    void* args[] = {&prm, &cf, &nw};
    if (cudaLaunchCooperativeKernel(fn, grid, kSolveThreads, args, (size_t)b->wave_cap[w], st) != cudaSuccess) {
      (void)cudaGetLastError();
      return ARAP_ECUDA;
    }
  }
  if (!stats_host) return ARAP_OK;
  std::vector<double> st8((size_t)kStatSlots * count);
  for (int i = 0; i < count; ++i)
    ARAP_CUDA_TRY(cudaMemcpyAsync(st8.data() + (size_t)kStatSlots * i, b->solvers[i]->P.stats,
                                  sizeof(double) * kStatSlots, cudaMemcpyDeviceToHost, st));
  int status = ARAP_OK;
  for (int i = 0; i < count; ++i) {
    const int dev_status = read_solver_status(b->d_bars + i, st);  // synchronises
    const int si = fill_stats(b->solvers[i], st8.data() + (size_t)kStatSlots * i, dev_status, stats_host + i);
    if (status == ARAP_OK) status = si;
  }
  return status;
}

extern "C" int arap_solver_batch_autotune(arap_solver_batch* b, const float* const* node_pos,
                                          const float* const* aims, float* const* rot_out, float* const* trans_out,
                                          float* best_exponent, arap_stream_t stream) {
  if (!b) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  const float candidates[] = {0.75f, 1.0f, 1.25f, 1.5f, 2.0f};
  float best = b->exponent, best_ms = 1e30f;
  cudaEvent_t e0, e1;
  ARAP_CUDA_TRY(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return ARAP_ECUDA;
  }
  int rc = ARAP_OK;
  for (float c : candidates) {
    b->exponent = c;
    split_ctas(b);
    if ((rc = upload_ctas(b)) != ARAP_OK) break;
    // one untimed solve, then the timed one
    rc = arap_solver_batch_solve(b, node_pos, aims, rot_out, trans_out, nullptr, stream);
    if (rc != ARAP_OK) break;
    if (cudaEventRecord(e0, st) != cudaSuccess) {
      rc = ARAP_ECUDA;
      break;
    }
    rc = arap_solver_batch_solve(b, node_pos, aims, rot_out, trans_out, nullptr, stream);
    if (rc != ARAP_OK) break;
    float ms = 0.f;
    if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      rc = ARAP_ECUDA;
      break;
    }
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->exponent = best;
  split_ctas(b);
  if (rc == ARAP_OK) rc = upload_ctas(b);
  if (best_exponent) *best_exponent = best;
  if (rc != ARAP_OK) return rc;
  for (size_t i = 0; i < b->solvers.size(); ++i)
    if (const int ds = read_solver_status(b->d_bars + i, st)) return ds;
  return ARAP_OK;
}

extern "C" int arap_solver_batch_ctas(const arap_solver_batch* b, int32_t* cta_first_host) {
  if (!b || !cta_first_host) return ARAP_EBADINPUT;
  // prefix sums of the CTAs each instance gets in its wave
  cta_first_host[0] = 0;
  for (size_t i = 0; i < b->ctas.size(); ++i) cta_first_host[i + 1] = cta_first_host[i] + b->ctas[i];
  return ARAP_OK;
}

extern "C" void arap_solver_batch_destroy(arap_solver_batch* b) {
  if (!b) return;
  if (b->staged_valid) cudaEventSynchronize(b->staged);
  if (b->staged) cudaEventDestroy(b->staged);
  if (b->h_params) cudaFreeHost(b->h_params);
  if (b->block) cudaFree(b->block);
  delete b;
}
