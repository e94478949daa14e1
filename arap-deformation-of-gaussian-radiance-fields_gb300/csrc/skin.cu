// Per-frame skinning kernels (sm_103a): node transform table, endpoint
// creation, fused Gaussian skinning + refit + SH rotation, node quaternions,
// fused sample skinning + slerp blend + SH rotation, node update, static masks
// and control-target generators.
//
// Layouts: per-item state the library owns (endpoints, kNN) is in planes
// [C][P] so that every warp load is one 128-byte line; per-item outputs that
// the rasteriser consumes keep the reference's AoS records (pos float3,
// rot float4 (w,x,y,z), scale float3, SH 48 floats [coef*3 + rgb]).
#include <algorithm>
#include <new>
#include <vector>

#include "arap_common.cuh"

namespace arap {

constexpr int kSkinThreads = 128;

// Node table entry: [R - I row-major 9 | g 3 | t 3 | 0] as four float4.
struct NodeXf {
  float4 a, b, c, d;
};

__device__ __forceinline__ NodeXf load_node(const float* __restrict__ table, int j) {
  const float4* t = reinterpret_cast<const float4*>(table) + 4 * (size_t)j;
  NodeXf x;
  x.a = __ldg(t);
  x.b = __ldg(t + 1);
  x.c = __ldg(t + 2);
  x.d = __ldg(t + 3);
  return x;
}

// w * ((R - I)(p - g) + t): the summand of DeformGraph::predict_mesh
// (Deform.hpp:238-246) minus w p.  A blend is accumulated from these small
// terms and added to (sum w) p once at the end (ed_finish), so the stored
// position is rounded once instead of once per neighbour.
__device__ __forceinline__ void ed_term(const NodeXf& x, float w, float px, float py, float pz,
                                        float& ox, float& oy, float& oz) {
  const float dx = px - x.c.y, dy = py - x.c.z, dz = pz - x.c.w;
  const float mx = fmaf(x.a.x, dx, fmaf(x.a.y, dy, fmaf(x.a.z, dz, x.d.x)));
  const float my = fmaf(x.a.w, dx, fmaf(x.b.x, dy, fmaf(x.b.y, dz, x.d.y)));
  const float mz = fmaf(x.b.z, dx, fmaf(x.b.w, dy, fmaf(x.c.x, dz, x.d.z)));
  ox = fmaf(w, mx, ox);
  oy = fmaf(w, my, oy);
  oz = fmaf(w, mz, oz);
}

// p' = (sum w) p + sum w ((R - I)(p - g) + t) = p + [(sum w - 1) p + acc].
__device__ __forceinline__ float ed_finish(float p, float wsum, float acc) {
  return p + fmaf(wsum - 1.0f, p, acc);
}

// A node's blend term in tile-local affine form for the Gaussian skinning:
// (R - I)(p - g) + t = A (p - o) + b_o with A = R - I and b_o = t - A (g - o),
// o a point of the tile (its first Gaussian's first endpoint), so that p - o
// and g - o stay small and no large terms cancel.  12 floats:
// a = (A00 A01 A02 A10), b = (A11 A12 A20 A21), c = (A22, b_o).
struct NodeAf {
  float4 a, b, c;
};

__device__ __forceinline__ NodeAf node_affine(const NodeXf& x, float ox, float oy, float oz) {
  const float gx = x.c.y - ox, gy = x.c.z - oy, gz = x.c.w - oz;
  NodeAf r;
  r.a = x.a;
  r.b = x.b;
  r.c = make_float4(x.c.x, x.d.x - fmaf(x.a.x, gx, fmaf(x.a.y, gy, x.a.z * gz)),
                    x.d.y - fmaf(x.a.w, gx, fmaf(x.b.x, gy, x.b.y * gz)),
                    x.d.z - fmaf(x.b.z, gx, fmaf(x.b.w, gy, x.c.x * gz)));
  return r;
}

// w * (A d + b_o), d = p - o, accumulated into (ox, oy, oz).
__device__ __forceinline__ void ed_term_af(const NodeAf& x, float w, float dx, float dy, float dz, float& ox,
                                           float& oy, float& oz) {
  const float mx = fmaf(x.a.x, dx, fmaf(x.a.y, dy, fmaf(x.a.z, dz, x.c.y)));
  const float my = fmaf(x.a.w, dx, fmaf(x.b.x, dy, fmaf(x.b.y, dz, x.c.z)));
  const float mz = fmaf(x.b.z, dx, fmaf(x.b.w, dy, fmaf(x.c.x, dz, x.c.w)));
  ox = fmaf(w, mx, ox);
  oy = fmaf(w, my, oy);
  oz = fmaf(w, mz, oz);
}

__global__ void node_table_kernel(int n, const float* __restrict__ rot,
                                  const float* __restrict__ trans,
                                  const float* __restrict__ pos, float* __restrict__ table) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float* r = rot + 9 * (size_t)j;  // column-major
  float4* t = reinterpret_cast<float4*>(table) + 4 * (size_t)j;
  const float gx = pos[3 * (size_t)j], gy = pos[3 * (size_t)j + 1], gz = pos[3 * (size_t)j + 2];
  t[0] = make_float4(r[0] - 1.0f, r[3], r[6], r[1]);
  t[1] = make_float4(r[4] - 1.0f, r[7], r[2], r[5]);
  t[2] = make_float4(r[8] - 1.0f, gx, gy, gz);
  t[3] = make_float4(trans[3 * (size_t)j], trans[3 * (size_t)j + 1], trans[3 * (size_t)j + 2], 0.f);
}

// GetEndPoints (GaussianView.cpp:4643-4668).
__global__ void end_points_kernel(int N, const float* __restrict__ pos,
                                  const float* __restrict__ rot, const float* __restrict__ scale,
                                  float* __restrict__ ends, float* __restrict__ ends_xyz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float4 q = quat_normalize(__ldg(reinterpret_cast<const float4*>(rot) + i));
  float R[9];
  quat_to_rowmajor(q, R);
  const float mu[3] = {pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2]};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float h = (scale[3 * (size_t)i + a] + 1e-3f) * 2.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float e = R[c * 3 + a] * h;
      const float plus = mu[c] + e, minus = mu[c] - e;
      ends[(size_t)(3 * (2 * a) + c) * N + i] = plus;
      ends[(size_t)(3 * (2 * a + 1) + c) * N + i] = minus;
      if (ends_xyz) {
        ends_xyz[((size_t)(2 * a) * N + i) * 3 + c] = plus;
        ends_xyz[((size_t)(2 * a + 1) * N + i) * 3 + c] = minus;
      }
    }
  }
}

// Fused UpdatePosition (endpoint part, GaussianView.cpp:3022-3040) and
// UpdateAsSixPointsWithdrawBad (GaussianView.cpp:3081-3166): one thread per
// Gaussian, kSkinTile per CTA.  The tile's 48-float SH records go through
// shared memory (16-byte cp.async copies of the contiguous records in, the
// rotation in place, coalesced 16-byte stores out) so that every global
// access of the kernel is coalesced.
constexpr int kSkinTile = kSkinThreads;  // Gaussians per CTA
constexpr int kShStride = 52;            // floats per staged SH record (13 float4: conflict-free)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(smem)), "l"(gmem) : "memory");
}

// The tile's SH records [cnt][48] into s_sh [T][kShStride] (all threads).
__device__ __forceinline__ void stage_sh(float* s_sh, const float* shs, int tile0, int cnt) {
  const float* src = shs + 48 * (size_t)tile0;
  for (int q = threadIdx.x; q < 12 * cnt; q += kSkinThreads)
    cp_async16(s_sh + (q / 12) * kShStride + (q % 12) * 4, src + 4 * (size_t)q);
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// s_sh back to the tile's SH records (all threads; after a __syncthreads).
__device__ __forceinline__ void store_sh(float* shs, const float* s_sh, int tile0, int cnt) {
  float4* dst = reinterpret_cast<float4*>(shs + 48 * (size_t)tile0);
  for (int q = threadIdx.x; q < 12 * cnt; q += kSkinThreads)
    __stcs(dst + q, *reinterpret_cast<const float4*>(s_sh + (q / 12) * kShStride + (q % 12) * 4));
}

// ---- bulk copies (TMA) and their mbarrier
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// global -> shared bulk copy completing on bar; both addresses 16-byte
// aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Bounded wait for phase `parity` of bar: false after max_polls polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int max_polls) {
  for (int it = 0; it < max_polls; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
constexpr int kMbarPolls = 1 << 18;

// The refit of one Gaussian from its six blended endpoints e (UpdateAsSix-
// PointsWithdrawBad, GaussianView.cpp:3081-3166): centre, polar factor R of
// the endpoint matrix, quaternion, scale, Sigma; writes mu, q, scale and
// Sigma of Gaussian i and returns in qr the rotation q q_old^-1 (a unit
// quaternion) that rotates its SH.
template <bool MIXED>
__device__ __forceinline__ void refit_gaussian(int i, const float (&e)[18], const float (&s0v)[3], float4 q_old,
                                               float* __restrict__ pos_out, float* __restrict__ rot_out,
                                               float* __restrict__ scale_out, float* __restrict__ cov_out,
                                               int* __restrict__ status, float4& qr) {
  float cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll
  for (int ep = 0; ep < 6; ++ep) {
    cx += e[3 * ep];
    cy += e[3 * ep + 1];
    cz += e[3 * ep + 2];
  }
  cx *= (1.0f / 6.0f);
  cy *= (1.0f / 6.0f);
  cz *= (1.0f / 6.0f);
  // M = (P - c) Q^+ with Q = [e0 -e0 e1 -e1 e2 -e2], Q^+ = Q^T / 2:
  // column a of M is (P_{2a} - P_{2a+1}) / 2.
  float M[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int r = 0; r < 3; ++r) M[r * 3 + a] = 0.5f * (e[3 * (2 * a) + r] - e[3 * (2 * a + 1) + r]);
  float R[9];
  bool ok;
  if (MIXED) {
    // FP64 polar factor when M is ill-conditioned (sigma_min/sigma_max < 1e-3)
    float nx = 0.f, ny = 0.f, Y[9];
    ok = inv_transpose3(M, Y);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      nx += M[q] * M[q];
      ny += Y[q] * Y[q];
    }
    if (!ok || nx * ny > 1e6f) {
      double Md[9], Rd[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) Md[q] = M[q];
      ok = polar_factor<double>(Md, Rd, 40, 1e-15);
#pragma unroll
      for (int q = 0; q < 9; ++q) R[q] = (float)Rd[q];
    } else {
      ok = polar_factor<float>(M, R, 20, 2e-7f);
    }
  } else {
    ok = polar_factor<float>(M, R, 20, 2e-7f);
  }
  if (!ok) raise_status(status, ARAP_ENONFINITE);
  // K = diag(R^T M) = diag(V S V^T)
  float Kd[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) Kd[a] = R[a] * M[a] + R[3 + a] * M[3 + a] + R[6 + a] * M[6 + a];
  const float4 q = quat_normalize(quat_from_rowmajor(R));
  float sc[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float s0 = s0v[a];
    sc[a] = Kd[a] / ((s0 + 1e-3f) * 2.0f) * s0;
  }
  pos_out[3 * (size_t)i] = cx;
  pos_out[3 * (size_t)i + 1] = cy;
  pos_out[3 * (size_t)i + 2] = cz;
  scale_out[3 * (size_t)i] = sc[0];
  scale_out[3 * (size_t)i + 1] = sc[1];
  scale_out[3 * (size_t)i + 2] = sc[2];
  reinterpret_cast<float4*>(rot_out)[i] = q;
  if (cov_out) {
    float Rq[9];
    quat_to_rowmajor(q, Rq);
    const float s2[3] = {sc[0] * sc[0], sc[1] * sc[1], sc[2] * sc[2]};
    float S[6];
    int o = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = r; c < 3; ++c)
        S[o++] = Rq[r * 3] * s2[0] * Rq[c * 3] + Rq[r * 3 + 1] * s2[1] * Rq[c * 3 + 1] +
                 Rq[r * 3 + 2] * s2[2] * Rq[c * 3 + 2];
#pragma unroll
    for (int q6 = 0; q6 < 6; ++q6) cov_out[6 * (size_t)i + q6] = S[q6];
  }
  qr = quat_normalize(quat_mul(q, quat_inverse(q_old)));
}

// Rotates the staged 48-float SH record rec (kShStride floats) by the unit
// quaternion qr.
__device__ __forceinline__ void rotate_sh_record(float* rec_f, float4 qr) {
  float4* rec = reinterpret_cast<float4*>(rec_f);
  float v[48];
#pragma unroll
  for (int q4 = 0; q4 < 12; ++q4) {
    const float4 u = rec[q4];
    v[4 * q4] = u.x;
    v[4 * q4 + 1] = u.y;
    v[4 * q4 + 2] = u.z;
    v[4 * q4 + 3] = u.w;
  }
  rotate_sh48<true>(qr, v);
#pragma unroll
  for (int q4 = 0; q4 < 12; ++q4) rec[q4] = make_float4(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3]);
}

constexpr size_t skin_smem_bytes() { return sizeof(float) * (size_t)kSkinTile * (4 + kShStride); }

// Without a plan: each endpoint's K node records are gathered from the node
// table (L1/L2) and put into tile-local affine form on the fly; indices and
// weights come from the planes [K*6][N].
template <int K, bool MIXED>
__global__ void __launch_bounds__(kSkinThreads, 4)
    skin_gaussians_kernel(int N, float* __restrict__ ends, const int32_t* __restrict__ eidx,
                          const float* __restrict__ ew, const float* __restrict__ table,
                          const float* __restrict__ scale0, const uint8_t* __restrict__ static_mask,
                          float* __restrict__ pos_out, float* __restrict__ rot_inout,
                          float* __restrict__ scale_out, float* __restrict__ shs,
                          float* __restrict__ cov_out, int* __restrict__ status) {
  extern __shared__ float4 s_raw4[];
  float* s_sh = reinterpret_cast<float*>(s_raw4);                         // [T][52]
  float4* s_q = reinterpret_cast<float4*>(s_sh + kSkinTile * kShStride);  // [T]
  const int t = threadIdx.x;
  const int tile0 = blockIdx.x * kSkinTile;
  const int cnt = min(kSkinTile, N - tile0);
  const int i = tile0 + t;
  const bool active = t < cnt;
  // the tile's origin: its first Gaussian's first endpoint before this frame
  // (read by every thread before any thread writes its endpoints)
  const float o_x = __ldg(ends + tile0), o_y = __ldg(ends + (size_t)N + tile0),
              o_z = __ldg(ends + 2 * (size_t)N + tile0);
  if (active) cp_async16(s_q + t, reinterpret_cast<const float4*>(rot_inout) + i);
  if (shs)
    stage_sh(s_sh, shs, tile0, cnt);
  else
    asm volatile("cp.async.commit_group;" ::: "memory");
  __syncthreads();

  float e[18];
  const bool is_static = active && static_mask && __ldg(static_mask + i);
  float s0v[3] = {0.f, 0.f, 0.f};
  if (active) {
#pragma unroll
    for (int a = 0; a < 3; ++a) s0v[a] = __ldg(scale0 + 3 * (size_t)i + a);
#pragma unroll
    for (int c = 0; c < 18; ++c) e[c] = __ldcs(ends + (size_t)c * N + i);
#pragma unroll
    for (int ep = 0; ep < 6; ++ep) {
      float ox = 0.f, oy = 0.f, oz = 0.f, ws = 0.f;
      const float dx = e[3 * ep] - o_x, dy = e[3 * ep + 1] - o_y, dz = e[3 * ep + 2] - o_z;
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const int id = __ldcs(eidx + (size_t)(j * 6 + ep) * N + i);
        const float w = __ldcs(ew + (size_t)(j * 6 + ep) * N + i);
        const NodeAf x = node_affine(load_node(table, id), o_x, o_y, o_z);
        ws += w;
        ed_term_af(x, w, dx, dy, dz, ox, oy, oz);
      }
      e[3 * ep] = ed_finish(e[3 * ep], ws, ox);
      e[3 * ep + 1] = ed_finish(e[3 * ep + 1], ws, oy);
      e[3 * ep + 2] = ed_finish(e[3 * ep + 2], ws, oz);
    }
#pragma unroll
    for (int c = 0; c < 18; ++c) __stcs(ends + (size_t)c * N + i, e[c]);
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  if (active && !is_static) {
    float4 qr;
    refit_gaussian<MIXED>(i, e, s0v, s_q[t], pos_out, rot_inout, scale_out, cov_out, status, qr);
    if (shs) rotate_sh_record(s_sh + t * kShStride, qr);
  }
  if (shs) {
    __syncthreads();
    store_sh(shs, s_sh, tile0, cnt);
  }
}

// ---- planned skinning
// Skinning plan (set-up time, arap_skin_plan_create): per tile of kSkinTile
// Gaussians the distinct nodes its endpoints blend (at most kPlanNodes), and
// one contiguous block of the tile's weights and 8-bit local node indices in
// the order the frame kernel reads them: weights as float4 [6][KQ][T]
// (neighbours 4q..4q+3 of endpoint ep of Gaussian t), local indices as
// 32-bit words [6][KQ][T] (four per word), KQ = ceil(K/4).  A frame copies the
// block into shared memory with one bulk copy (TMA) and its node records
// once; thread t then reads its weights and indices conflict-free and gathers
// the node records from shared memory.
constexpr int kPlanNodes = 256;
constexpr int kPlanRec = 12;  // floats per staged node record (NodeAf; the 48-byte stride spreads banks)
struct SkinPlanDev {
  const int32_t* tile_count;  // [tiles] distinct nodes of the tile (> kPlanNodes: no local list)
  const int32_t* tile_nodes;  // [tiles][kPlanNodes]
  const unsigned char* blk;   // [tiles][tile_bytes]: weights then local indices
  // for the adjoint: per tile, the references of each slot u (ref = (g * 6 +
  // ep) * K + j, ascending) at inv_ref[inv_off[u] .. inv_off[u + 1])
  const uint16_t* inv_off;    // [tiles][kPlanNodes + 1]
  const uint16_t* inv_ref;    // [tiles][6 * K * kSkinTile]
};
template <int K>
struct PlanTile {
  static constexpr int KQ = (K + 3) / 4;
  static constexpr int kWBytes = 6 * KQ * kSkinTile * 16;
  static constexpr int kLBytes = 6 * KQ * kSkinTile * 4;
  static constexpr int kBytes = kWBytes + kLBytes;
  static constexpr int kShBytes = kSkinTile * kShStride * 4;
  // region A holds the plan block during the blend, the SH records after it
  static constexpr int kRegionA = kBytes > kShBytes ? kBytes : kShBytes;
  static constexpr int kQOff = kRegionA;
  static constexpr int kNodeOff = kQOff + kSkinTile * 16;
  static constexpr int kBarOff = kNodeOff + kPlanNodes * kPlanRec * 4;
  static constexpr int kSmem = kBarOff + 16;
};
inline int plan_tile_bytes(int k) { return 6 * ((k + 3) / 4) * kSkinTile * 20; }

// The planned frame kernel.  Per tile: one thread starts two bulk copies (the
// tile's plan block and its previous quaternions) on an mbarrier; meanwhile
// every thread requests its endpoints and the tile's node records are put
// into tile-local affine form in shared memory.  The blend reads everything
// from shared memory; its region then takes the tile's SH records
// (cp.async), which arrive while the refit runs.  A tile with more than
// kPlanNodes nodes gathers from the table as the unplanned kernel does.
template <int K, bool MIXED>
__global__ void __launch_bounds__(kSkinThreads, 4)
    skin_gaussians_planned_kernel(int N, float* __restrict__ ends, const int32_t* __restrict__ eidx,
                                  const float* __restrict__ ew, const float* __restrict__ table,
                                  const float* __restrict__ scale0, const uint8_t* __restrict__ static_mask,
                                  float* __restrict__ pos_out, float* __restrict__ rot_inout,
                                  float* __restrict__ scale_out, float* __restrict__ shs,
                                  float* __restrict__ cov_out, SkinPlanDev plan, int* __restrict__ status) {
  using PT = PlanTile<K>;
  constexpr int KQ = PT::KQ;
  extern __shared__ __align__(128) unsigned char s_buf[];
  const float4* s_w = reinterpret_cast<const float4*>(s_buf);                       // [6][KQ][T]
  const uint32_t* s_l = reinterpret_cast<const uint32_t*>(s_buf + PT::kWBytes);    // [6][KQ][T]
  float* s_sh = reinterpret_cast<float*>(s_buf);                                    // [T][52], after the blend
  const float4* s_q = reinterpret_cast<const float4*>(s_buf + PT::kQOff);          // [T]
  float* s_nodes = reinterpret_cast<float*>(s_buf + PT::kNodeOff);                  // [kPlanNodes][12]
  const uint32_t bar = smem_addr(s_buf + PT::kBarOff);
  const int t = threadIdx.x;
  const int tile0 = blockIdx.x * kSkinTile;
  const int cnt = min(kSkinTile, N - tile0);
  const int i = tile0 + t;
  const bool active = t < cnt;
  const int n_local = __ldg(plan.tile_count + blockIdx.x);
  const bool local = n_local <= kPlanNodes;
  if (t == 0) mbar_init(bar, 1);
  __syncthreads();
  if (t == 0) {
    const uint32_t qb = 16u * (uint32_t)cnt;
    mbar_arrive_expect_tx(bar, qb + (local ? (uint32_t)PT::kBytes : 0u));
    bulk_g2s(smem_addr(s_buf + PT::kQOff), rot_inout + 4 * (size_t)tile0, qb, bar);
    if (local) bulk_g2s(smem_addr(s_buf), plan.blk + (size_t)blockIdx.x * PT::kBytes, PT::kBytes, bar);
  }
  const float o_x = __ldg(ends + tile0), o_y = __ldg(ends + (size_t)N + tile0),
              o_z = __ldg(ends + 2 * (size_t)N + tile0);
  float e[18];
  float s0v[3] = {0.f, 0.f, 0.f};
  const bool is_static = active && static_mask && __ldg(static_mask + i);
  if (active) {
#pragma unroll
    for (int c = 0; c < 18; ++c) e[c] = __ldcs(ends + (size_t)c * N + i);
#pragma unroll
    for (int a = 0; a < 3; ++a) s0v[a] = __ldg(scale0 + 3 * (size_t)i + a);
  }
  {
    // every slot of the tile's node list holds a valid node id (the plan
    // fills the slots past the tile's count), so the records are requested
    // without waiting for the count: two list loads, then the two records
    static_assert(kPlanNodes == 2 * kSkinThreads, "two list slots per thread");
    const int32_t* list = plan.tile_nodes + (size_t)blockIdx.x * kPlanNodes;
    const int id0 = __ldg(list + t), id1 = __ldg(list + kSkinThreads + t);
    const NodeXf x0 = load_node(table, id0), x1 = load_node(table, id1);
    const NodeAf r0 = node_affine(x0, o_x, o_y, o_z), r1 = node_affine(x1, o_x, o_y, o_z);
    float4* d0 = reinterpret_cast<float4*>(s_nodes + t * kPlanRec);
    float4* d1 = reinterpret_cast<float4*>(s_nodes + (kSkinThreads + t) * kPlanRec);
    d0[0] = r0.a;
    d0[1] = r0.b;
    d0[2] = r0.c;
    d1[0] = r1.a;
    d1[1] = r1.b;
    d1[2] = r1.c;
  }
  // node records written; every thread waits for the bulk copies itself
  __syncthreads();
  const bool arrived = mbar_wait(bar, 0u, kMbarPolls);
  if (__syncthreads_or(!arrived)) {
    if (t == 0) raise_status(status, ARAP_ETIMEOUT);
    return;
  }
  if (active) {
#pragma unroll
    for (int ep = 0; ep < 6; ++ep) {
      float ox = 0.f, oy = 0.f, oz = 0.f, ws = 0.f;
      const float dx = e[3 * ep] - o_x, dy = e[3 * ep + 1] - o_y, dz = e[3 * ep + 2] - o_z;
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        float4 w4 = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t lw = 0u;
        if (local) {
          w4 = s_w[(ep * KQ + q) * kSkinTile + t];
          lw = s_l[(ep * KQ + q) * kSkinTile + t];
        }
        const float wq[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int j = 4 * q + r;
          if (j < K) {
            NodeAf x;
            float w;
            if (local) {
              const float4* r4 = reinterpret_cast<const float4*>(s_nodes + ((lw >> (8 * r)) & 0xffu) * kPlanRec);
              x.a = r4[0];
              x.b = r4[1];
              x.c = r4[2];
              w = wq[r];
            } else {
              x = node_affine(load_node(table, __ldcs(eidx + (size_t)(j * 6 + ep) * N + i)), o_x, o_y, o_z);
              w = __ldcs(ew + (size_t)(j * 6 + ep) * N + i);
            }
            ws += w;
            ed_term_af(x, w, dx, dy, dz, ox, oy, oz);
          }
        }
      }
      e[3 * ep] = ed_finish(e[3 * ep], ws, ox);
      e[3 * ep + 1] = ed_finish(e[3 * ep + 1], ws, oy);
      e[3 * ep + 2] = ed_finish(e[3 * ep + 2], ws, oz);
    }
#pragma unroll
    for (int c = 0; c < 18; ++c) __stcs(ends + (size_t)c * N + i, e[c]);
  }
  // region A: plan block read by every thread; the SH records go there and
  // arrive while the refit runs
  __syncthreads();
  if (shs) stage_sh(s_sh, shs, tile0, cnt);
  float4 qr;
  const bool refit = active && !is_static;
  if (refit) refit_gaussian<MIXED>(i, e, s0v, s_q[t], pos_out, rot_inout, scale_out, cov_out, status, qr);
  if (shs) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    if (refit) rotate_sh_record(s_sh + t * kShStride, qr);
    __syncthreads();
    store_sh(shs, s_sh, tile0, cnt);
  }
}

// Adjoint of the Gaussian skinning map: given dL/dmu [N*3] and dL/dSigma
// [N*6] (packed xx,xy,xz,yy,yz,zz; dL = sum_p g_p dSigma_p), accumulate dL/d
// (R_j, t_j) into grad_node [n*12] ([dR column-major 9 | dt 3]).  Each thread
// recomputes its Gaussian's blended endpoints and polar factor from the
// pre-frame endpoints (nothing is stored by the forward), then
//   Sigma = R D R^T, D_a = (c_a K_a)^2, K_a = (R^T M)_aa, c_a = s0_a/((s0_a+1e-3)*2)
//   dL/dR += 2 G R D,  dL/dK_a = (R^T G R)_aa 2 c_a^2 K_a,
//   dL/dM += R diag(dL/dK) ; dL/dR += M diag(dL/dK),
//   polar: A = R^T dL/dR, w = (tr S I - S)^-1 skew(A), dL/dM += 2 R [w]x,
//   M_a = (P_2a - P_2a+1)/2, mu = mean P, P_e = sum_j w_ej (R_j (p_e - g_j) + g_j + t_j).
// Node gradients are summed per CTA in a shared-memory hash table of node ids
// and flushed with one global atomic per (node, component).
constexpr int kHashSlots = 512;

__device__ __forceinline__ void hash_add(int* keys, float (*vals)[12], int nid, const float (&v)[12],
                                         float* __restrict__ grad_node) {
  unsigned h = ((unsigned)nid * 2654435761u) & (kHashSlots - 1);
  for (int probe = 0; probe < kHashSlots; ++probe) {
    const int k = atomicCAS(keys + h, -1, nid);
    if (k == -1 || k == nid) {
#pragma unroll
      for (int c = 0; c < 12; ++c) atomicAdd(&vals[h][c], v[c]);
      return;
    }
    h = (h + 1) & (kHashSlots - 1);
  }
#pragma unroll
  for (int c = 0; c < 12; ++c) atomicAdd(grad_node + 12 * (size_t)nid + c, v[c]);
}

// The adjoint chain of one Gaussian from its endpoint matrix M and polar
// factor R to the gradients gP [18] of its six blended endpoints (the
// formulas above).
__device__ __forceinline__ void skin_adjoint_gP(int i, const float (&M)[9], const float (&R)[9],
                                                const float* __restrict__ scale0,
                                                const float* __restrict__ grad_pos,
                                                const float* __restrict__ grad_cov, float (&gP)[18]) {
  float S[9];  // R^T M, symmetrised
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) S[a * 3 + b] = R[a] * M[b] + R[3 + a] * M[3 + b] + R[6 + a] * M[6 + b];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a + 1; b < 3; ++b) S[a * 3 + b] = S[b * 3 + a] = 0.5f * (S[a * 3 + b] + S[b * 3 + a]);
  float cK[3], D[3], Kd[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float s0 = scale0[3 * (size_t)i + a];
    cK[a] = s0 / ((s0 + 1e-3f) * 2.0f);
    Kd[a] = R[a] * M[a] + R[3 + a] * M[3 + a] + R[6 + a] * M[6 + a];
    D[a] = (cK[a] * Kd[a]) * (cK[a] * Kd[a]);
  }
  const float* gc = grad_cov + 6 * (size_t)i;
  const float G[9] = {gc[0], 0.5f * gc[1], 0.5f * gc[2], 0.5f * gc[1], gc[3], 0.5f * gc[4],
                      0.5f * gc[2], 0.5f * gc[4], gc[5]};
  float GR[9];  // G R
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a) GR[r * 3 + a] = G[r * 3] * R[a] + G[r * 3 + 1] * R[3 + a] + G[r * 3 + 2] * R[6 + a];
  float gK[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float gD = R[a] * GR[a] + R[3 + a] * GR[3 + a] + R[6 + a] * GR[6 + a];
    gK[a] = gD * 2.f * cK[a] * cK[a] * Kd[a];
  }
  float gR[9], gM[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      gR[r * 3 + a] = 2.f * GR[r * 3 + a] * D[a] + M[r * 3 + a] * gK[a];
      gM[r * 3 + a] = R[r * 3 + a] * gK[a];
    }
  float A[9];  // R^T gR
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) A[a * 3 + b] = R[a] * gR[b] + R[3 + a] * gR[3 + b] + R[6 + a] * gR[6 + b];
  const float av[3] = {0.5f * (A[7] - A[5]), 0.5f * (A[2] - A[6]), 0.5f * (A[3] - A[1])};
  const float tr = S[0] + S[4] + S[8];
  float T[9], Ti[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) T[q] = -S[q];
  T[0] += tr;
  T[4] += tr;
  T[8] += tr;
  float om[3] = {0.f, 0.f, 0.f};
  if (inv_transpose3(T, Ti)) {  // T symmetric: inverse-transpose = inverse
#pragma unroll
    for (int r = 0; r < 3; ++r) om[r] = Ti[r * 3] * av[0] + Ti[r * 3 + 1] * av[1] + Ti[r * 3 + 2] * av[2];
  }
  const float Y[9] = {0.f, -om[2], om[1], om[2], 0.f, -om[0], -om[1], om[0], 0.f};
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a)
      gM[r * 3 + a] += 2.f * (R[r * 3] * Y[a] + R[r * 3 + 1] * Y[3 + a] + R[r * 3 + 2] * Y[6 + a]);
  const float gm[3] = {grad_pos[3 * (size_t)i] * (1.f / 6.f), grad_pos[3 * (size_t)i + 1] * (1.f / 6.f),
                       grad_pos[3 * (size_t)i + 2] * (1.f / 6.f)};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      gP[3 * (2 * a) + r] = gm[r] + 0.5f * gM[r * 3 + a];
      gP[3 * (2 * a + 1) + r] = gm[r] - 0.5f * gM[r * 3 + a];
    }
}

template <int K>
__global__ void __launch_bounds__(kSkinThreads)
    skin_gaussians_backward_kernel(int N, const float* __restrict__ ends_in, const int32_t* __restrict__ eidx,
                                   const float* __restrict__ ew, const float* __restrict__ table,
                                   const float* __restrict__ scale0, const uint8_t* __restrict__ static_mask,
                                   const float* __restrict__ grad_pos, const float* __restrict__ grad_cov,
                                   float* __restrict__ grad_node, int* __restrict__ status) {
  __shared__ int s_keys[kHashSlots];
  __shared__ float s_vals[kHashSlots][12];
  for (int q = threadIdx.x; q < kHashSlots; q += blockDim.x) {
    s_keys[q] = -1;
#pragma unroll
    for (int c = 0; c < 12; ++c) s_vals[q][c] = 0.f;
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N && !(static_mask && static_mask[i])) {
    float p0[18], e[18];
#pragma unroll
    for (int c = 0; c < 18; ++c) p0[c] = __ldg(ends_in + (size_t)c * N + i);
#pragma unroll
    for (int ep = 0; ep < 6; ++ep) {
      float ox = 0.f, oy = 0.f, oz = 0.f, ws = 0.f;
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const size_t o = (size_t)(j * 6 + ep) * N + i;
        const NodeXf x = load_node(table, __ldg(eidx + o));
        const float w = __ldg(ew + o);
        ws += w;
        ed_term(x, w, p0[3 * ep], p0[3 * ep + 1], p0[3 * ep + 2], ox, oy, oz);
      }
      e[3 * ep] = ed_finish(p0[3 * ep], ws, ox);
      e[3 * ep + 1] = ed_finish(p0[3 * ep + 1], ws, oy);
      e[3 * ep + 2] = ed_finish(p0[3 * ep + 2], ws, oz);
    }
    float M[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int r = 0; r < 3; ++r) M[r * 3 + a] = 0.5f * (e[3 * (2 * a) + r] - e[3 * (2 * a + 1) + r]);
    float R[9];
    if (!polar_factor<float>(M, R, 20, 2e-7f)) raise_status(status, ARAP_ENONFINITE);
    float gP[18];
    skin_adjoint_gP(i, M, R, scale0, grad_pos, grad_cov, gP);
#pragma unroll 1
    for (int ep = 0; ep < 6; ++ep) {
      float gpe[3], pe[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        gpe[r] = gP[3 * ep + r];
        pe[r] = p0[3 * ep + r];
      }
#pragma unroll 2
      for (int j = 0; j < K; ++j) {
        const size_t o = (size_t)(j * 6 + ep) * N + i;
        const int nid = __ldg(eidx + o);
        const float w = __ldg(ew + o);
        const float4 gg = __ldg(reinterpret_cast<const float4*>(table) + 4 * (size_t)nid + 2);
        const float d[3] = {pe[0] - gg.y, pe[1] - gg.z, pe[2] - gg.w};
        float v[12];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int r = 0; r < 3; ++r) v[3 * c + r] = w * gpe[r] * d[c];
#pragma unroll
        for (int r = 0; r < 3; ++r) v[9 + r] = w * gpe[r];
        hash_add(s_keys, s_vals, nid, v, grad_node);
      }
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kHashSlots; q += blockDim.x) {
    const int nid = s_keys[q];
    if (nid < 0) continue;
#pragma unroll
    for (int c = 0; c < 12; ++c) atomicAdd(grad_node + 12 * (size_t)nid + c, s_vals[q][c]);
  }
}

// The adjoint with the skinning plan (every tile within kPlanNodes nodes).
// Per tile: the node records are staged in tile-local affine form as in the
// planned forward; thread t recomputes Gaussian t's blend (weights and slots
// read from the plan block, coalesced), its polar factor and the chain of the
// unplanned kernel above down to the endpoint gradients gP, which go to
// shared memory with the endpoints' offsets from the tile's origin.  Then one
// thread per slot sums its references (the plan's inverse lists, fixed
// order): S0 = sum w gP_e, S1 = sum w gP_e (p_e - o)^T, so that
// dL/dR_j = S1 - S0 (g_j - o)^T and dL/dt_j = S0, and adds them to grad_node
// with one global atomic per (tile, node, component): no shared atomics.
template <int K>
__global__ void __launch_bounds__(kSkinThreads)
    skin_gaussians_backward_planned_kernel(int N, const float* __restrict__ ends_in, const float* __restrict__ table,
                                           const float* __restrict__ scale0,
                                           const uint8_t* __restrict__ static_mask,
                                           const float* __restrict__ grad_pos, const float* __restrict__ grad_cov,
                                           float* __restrict__ grad_node, SkinPlanDev plan,
                                           int* __restrict__ status) {
  using PT = PlanTile<K>;
  constexpr int KQ = PT::KQ;
  constexpr int kRefBytes = 6 * K * kSkinTile * 2;
  __shared__ __align__(16) float s_nodes[kPlanNodes * kPlanRec];
  __shared__ float s_gp[kSkinTile][19];  // endpoint gradients (18), padded
  __shared__ float s_pe[kSkinTile][19];  // endpoint offsets from the origin (18), padded
  // dynamic: the tile's plan block (weights, slots) and its inverse lists
  extern __shared__ __align__(16) unsigned char s_bk[];
  const int t = threadIdx.x;
  const int tile0 = blockIdx.x * kSkinTile;
  const int cnt = min(kSkinTile, N - tile0);
  const int i = tile0 + t;
  const int n_stage = __ldg(plan.tile_count + blockIdx.x);
  {
    const unsigned char* gb = plan.blk + (size_t)blockIdx.x * PT::kBytes;
    for (int q = t; q < PT::kBytes / 16; q += kSkinThreads) cp_async16(s_bk + 16 * q, gb + 16 * q);
    const unsigned char* gr =
        reinterpret_cast<const unsigned char*>(plan.inv_ref + (size_t)blockIdx.x * 6 * K * kSkinTile);
    for (int q = t; q < kRefBytes / 16; q += kSkinThreads) cp_async16(s_bk + PT::kBytes + 16 * q, gr + 16 * q);
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  const float o_x = __ldg(ends_in + tile0), o_y = __ldg(ends_in + (size_t)N + tile0),
              o_z = __ldg(ends_in + 2 * (size_t)N + tile0);
  {
    // every list slot holds a valid node id: both records are requested
    // without waiting for the tile's count
    const int32_t* list = plan.tile_nodes + (size_t)blockIdx.x * kPlanNodes;
    const int id0 = __ldg(list + t), id1 = __ldg(list + kSkinThreads + t);
    const NodeXf x0 = load_node(table, id0), x1 = load_node(table, id1);
    const NodeAf r0 = node_affine(x0, o_x, o_y, o_z), r1 = node_affine(x1, o_x, o_y, o_z);
    float4* d0 = reinterpret_cast<float4*>(s_nodes + t * kPlanRec);
    float4* d1 = reinterpret_cast<float4*>(s_nodes + (kSkinThreads + t) * kPlanRec);
    d0[0] = r0.a;
    d0[1] = r0.b;
    d0[2] = r0.c;
    d1[0] = r1.a;
    d1[1] = r1.b;
    d1[2] = r1.c;
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  const unsigned char* tb = s_bk;
  const float4* gw = reinterpret_cast<const float4*>(tb);
  const uint32_t* gl = reinterpret_cast<const uint32_t*>(tb + PT::kWBytes);
  const uint16_t* ir = reinterpret_cast<const uint16_t*>(s_bk + PT::kBytes);
  float gP[18];
#pragma unroll
  for (int c = 0; c < 18; ++c) gP[c] = 0.f;
  if (t < cnt && !(static_mask && static_mask[i])) {
    float p0[18], e[18];
#pragma unroll
    for (int c = 0; c < 18; ++c) p0[c] = __ldg(ends_in + (size_t)c * N + i);
#pragma unroll
    for (int ep = 0; ep < 6; ++ep) {
      float ox = 0.f, oy = 0.f, oz = 0.f, ws = 0.f;
      const float dx = p0[3 * ep] - o_x, dy = p0[3 * ep + 1] - o_y, dz = p0[3 * ep + 2] - o_z;
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        const float4 w4 = gw[(ep * KQ + q) * kSkinTile + t];
        const uint32_t lw = gl[(ep * KQ + q) * kSkinTile + t];
        const float wq[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          if (4 * q + r < K) {
            const float4* r4 = reinterpret_cast<const float4*>(s_nodes + ((lw >> (8 * r)) & 0xffu) * kPlanRec);
            NodeAf x;
            x.a = r4[0];
            x.b = r4[1];
            x.c = r4[2];
            ws += wq[r];
            ed_term_af(x, wq[r], dx, dy, dz, ox, oy, oz);
          }
        }
      }
      e[3 * ep] = ed_finish(p0[3 * ep], ws, ox);
      e[3 * ep + 1] = ed_finish(p0[3 * ep + 1], ws, oy);
      e[3 * ep + 2] = ed_finish(p0[3 * ep + 2], ws, oz);
    }
#pragma unroll
    for (int ep = 0; ep < 6; ++ep) {
      s_pe[t][3 * ep] = p0[3 * ep] - o_x;
      s_pe[t][3 * ep + 1] = p0[3 * ep + 1] - o_y;
      s_pe[t][3 * ep + 2] = p0[3 * ep + 2] - o_z;
    }
    float M[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int r = 0; r < 3; ++r) M[r * 3 + a] = 0.5f * (e[3 * (2 * a) + r] - e[3 * (2 * a + 1) + r]);
    float R[9];
    if (!polar_factor<float>(M, R, 20, 2e-7f)) raise_status(status, ARAP_ENONFINITE);
    skin_adjoint_gP(i, M, R, scale0, grad_pos, grad_cov, gP);
  }
#pragma unroll
  for (int c = 0; c < 18; ++c) s_gp[t][c] = gP[c];
  __syncthreads();
  // one thread per slot: its references in the plan's fixed order
  const uint16_t* io = plan.inv_off + (size_t)blockIdx.x * (kPlanNodes + 1);
  const int32_t* list = plan.tile_nodes + (size_t)blockIdx.x * kPlanNodes;
  for (int u = t; u < n_stage; u += kSkinThreads) {
    const int r0 = __ldg(io + u), r1 = __ldg(io + u + 1);
    if (r0 == r1) continue;
    float S0[3] = {0.f, 0.f, 0.f}, S1[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int q = r0; q < r1; ++q) {
      const int ref = ir[q];
      const int g = ref / (6 * K), rem = ref - g * 6 * K, ep = rem / K, j = rem - ep * K;
      const float w = reinterpret_cast<const float*>(tb)[((ep * KQ + (j >> 2)) * kSkinTile + g) * 4 + (j & 3)];
      float wg[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) wg[r] = w * s_gp[g][3 * ep + r];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float d = s_pe[g][3 * ep + c];
#pragma unroll
        for (int r = 0; r < 3; ++r) S1[3 * c + r] = fmaf(wg[r], d, S1[3 * c + r]);
      }
#pragma unroll
      for (int r = 0; r < 3; ++r) S0[r] += wg[r];
    }
    const int nid = __ldg(list + u);
    const float4 gg = __ldg(reinterpret_cast<const float4*>(table) + 4 * (size_t)nid + 2);
    const float go[3] = {gg.y - o_x, gg.z - o_y, gg.w - o_z};
    float* dst = grad_node + 12 * (size_t)nid;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < 3; ++r) atomicAdd(dst + 3 * c + r, fmaf(-S0[r], go[c], S1[3 * c + r]));
#pragma unroll
    for (int r = 0; r < 3; ++r) atomicAdd(dst + 9 + r, S0[r]);
  }
}

// Per-node quaternion of the polar factor (GaussianView.cpp:3172-3181).
template <bool MIXED>
__global__ void node_quat_kernel(int n, const float* __restrict__ rot, float* __restrict__ quat,
                                 int* __restrict__ status) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float* r = rot + 9 * (size_t)j;
  float M[9] = {r[0], r[3], r[6], r[1], r[4], r[7], r[2], r[5], r[8]};
  bool ok;
  if (MIXED) {
    // FP64 Newton when the smallest singular value is tiny (|det| / |M|^3 small)
    float nrm = 0.f;
#pragma unroll
    for (int t = 0; t < 9; ++t) nrm += M[t] * M[t];
    const float det = det3(M);
    if (fabsf(det) < 1e-6f * nrm * sqrtf(nrm)) {
      double Md[9];
#pragma unroll
      for (int t = 0; t < 9; ++t) Md[t] = M[t];
      ok = newton_polar_ref<double>(Md, 200);
#pragma unroll
      for (int t = 0; t < 9; ++t) M[t] = (float)Md[t];
    } else {
      ok = newton_polar_ref<float>(M, 100);
    }
  } else {
    ok = newton_polar_ref<float>(M, 100);
  }
  if (!ok) raise_status(status, ARAP_ENONFINITE);
  const float4 q = quat_normalize(quat_from_rowmajor(M));
  reinterpret_cast<float4*>(quat)[j] = q;
}

// Q_SlerpCUDA (cudakdtree.cu:113-148) in float32; the cosine is the float32
// dot in the reference's (x,y,z,w) order.  The two weights
// sin((1-t) a) / sin a and sin(t a) / sin a come from one sine-cosine pair:
// sin((1-t) a) = sin a cos(t a) - cos a sin(t a), so the first is
// cos(t a) - cos a * (second); a <= pi/2 after the sign flip, and the
// hardware sine and cosine (absolute error about 4e-7 there) stand in for the
// library's, far inside what the blended quaternion needs.
__device__ __forceinline__ float4 slerp(float4 s, float4 e, float t) {
  float c = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(s.y, e.y), __fmul_rn(s.z, e.z)), __fmul_rn(s.w, e.w)),
                      __fmul_rn(s.x, e.x));
  if (c < 0.f) {
    e = make_float4(-e.x, -e.y, -e.z, -e.w);
    c = -c;
  }
  float ra, rb;
  if (c > 0.99995f) {
    ra = 1.0f - t;
    rb = t;
  } else {
    const float sa = sqrtf(1.0f - c * c);
    const float ang = atan2f(sa, c);
    float st, ct;
    __sincosf(t * ang, &st, &ct);
    rb = st * __frcp_rn(sa);
    ra = ct - c * rb;
  }
  return quat_normalize(make_float4(ra * s.x + rb * e.x, ra * s.y + rb * e.y, ra * s.z + rb * e.z,
                                    ra * s.w + rb * e.w));
}

// Fused UpdatePositionforSamples (GaussianView.cpp:3060-3077) and RotateSHs
// (cudakdtree.cu:201-222): one thread per sample, kSkinTile per CTA.  The
// tile's positions (coalesced loads) and 48-float feature records (16-byte
// cp.async copies of the contiguous records, padded rows) go through shared
// memory, so that every global access is coalesced; the feature records
// arrive while the positions are blended and the node quaternions slerped,
// are rotated in place and leave with coalesced 16-byte stores.
template <int K>
__global__ void __launch_bounds__(kSkinThreads)
    skin_samples_kernel(int S, float* __restrict__ spos, const int32_t* __restrict__ idx,
                        const float* __restrict__ w, const float* __restrict__ table,
                        const float* __restrict__ nquat, float* __restrict__ feature,
                        const uint8_t* __restrict__ static_mask) {
  extern __shared__ float4 s_raw4[];
  float* s_ft = reinterpret_cast<float*>(s_raw4);                  // [T][52] feature records
  float* s_p = s_ft + (feature ? kSkinTile * kShStride : 0);        // [T * 3] positions
  const int t = threadIdx.x;
  const int tile0 = blockIdx.x * kSkinTile;
  const int cnt = min(kSkinTile, S - tile0);
  const int i = tile0 + t;
  if (feature) stage_sh(s_ft, feature, tile0, cnt);
  for (int q = t; q < 3 * cnt; q += kSkinThreads) s_p[q] = __ldcs(spos + 3 * (size_t)tile0 + q);
  __syncthreads();
  const bool moving = t < cnt && !(static_mask && static_mask[i]);
  float4 wq = make_float4(1.f, 0.f, 0.f, 0.f);
  if (moving) {
    const float px = s_p[3 * t], py = s_p[3 * t + 1], pz = s_p[3 * t + 2];
    float ox = 0.f, oy = 0.f, oz = 0.f, ws = 0.f;
    float last = 0.f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const int nid = __ldcs(idx + (size_t)j * S + i);
      const float wj = __ldcs(w + (size_t)j * S + i);
      const NodeXf x = load_node(table, nid);
      ws += wj;
      ed_term(x, wj, px, py, pz, ox, oy, oz);
      if (feature) {
        const float tj = __fdividef(wj, wj + last);
        wq = slerp(wq, __ldg(reinterpret_cast<const float4*>(nquat) + nid), tj);
        last += wj;
      }
    }
    s_p[3 * t] = ed_finish(px, ws, ox);
    s_p[3 * t + 1] = ed_finish(py, ws, oy);
    s_p[3 * t + 2] = ed_finish(pz, ws, oz);
  }
  if (feature) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    if (moving) {
      rotate_sh_record(s_ft + t * kShStride, quat_normalize(wq));
    }
  }
  __syncthreads();
  for (int q = t; q < 3 * cnt; q += kSkinThreads) __stcs(spos + 3 * (size_t)tile0 + q, s_p[q]);
  if (feature) store_sh(feature, s_ft, tile0, cnt);
}

// GaussianView.cpp:3042-3052: next node position from its anchor kNN.
__global__ void update_nodes_kernel(int n, int k, const float* __restrict__ pos,
                                    const int32_t* __restrict__ aidx, const float* __restrict__ aw,
                                    const float* __restrict__ table, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float px = pos[3 * (size_t)i], py = pos[3 * (size_t)i + 1], pz = pos[3 * (size_t)i + 2];
  float ox = 0.f, oy = 0.f, oz = 0.f, ws = 0.f;
  for (int j = 0; j < k; ++j) {
    const NodeXf x = load_node(table, aidx[(size_t)j * n + i]);
    const float w = aw[(size_t)j * n + i];
    ws += w;
    ed_term(x, w, px, py, pz, ox, oy, oz);
  }
  out[3 * (size_t)i] = ed_finish(px, ws, ox);
  out[3 * (size_t)i + 1] = ed_finish(py, ws, oy);
  out[3 * (size_t)i + 2] = ed_finish(pz, ws, oz);
}

__global__ void static_mask_kernel(int P, int planes, const int32_t* __restrict__ idx,
                                   const uint8_t* __restrict__ node_static, uint8_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  uint8_t all = 1;
  for (int p = 0; p < planes; ++p) all &= node_static[idx[(size_t)p * P + i]] ? 1 : 0;
  out[i] = all;
}

// ---------------------------------------------------- control targets ----
// One CTA; the centroid is summed in float64 over the listed nodes.
__device__ void block_centroid(const float* __restrict__ pos, const int32_t* __restrict__ ids, int m,
                               float* c) {
  double v[3] = {0.0, 0.0, 0.0};
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int j = ids[t];
    v[0] += pos[3 * (size_t)j];
    v[1] += pos[3 * (size_t)j + 1];
    v[2] += pos[3 * (size_t)j + 2];
  }
  block_sum<3>(v);
  c[0] = (float)(v[0] / m);
  c[1] = (float)(v[1] / m);
  c[2] = (float)(v[2] / m);
}

// PointRotateByAxis (helper.cpp:1077-1100): rotation by `rad` about the unit
// axis (x,y,z) through the point (a,b,c), the closed form of the rotation of a
// point about an arbitrary line.
__device__ __forceinline__ void rotate_about_line(float* p, const float* ctr, float ax, float ay,
                                                  float az, float rad) {
  const float ct = cosf(rad), st = sinf(rad);
  const float nrm = sqrtf(ax * ax + ay * ay + az * az);
  const float x = ax / nrm, y = ay / nrm, z = az / nrm;
  const float a = ctr[0], b = ctr[1], c = ctr[2];
  const float u = 1.0f - ct;
  const float px = p[0], py = p[1], pz = p[2];
  float o0 = (x * x * u + ct) * px + (x * y * u - z * st) * py + (x * z * u + y * st) * pz;
  float o1 = (y * x * u + z * st) * px + (y * y * u + ct) * py + (y * z * u - x * st) * pz;
  float o2 = (z * x * u - y * st) * px + (z * y * u + x * st) * py + (z * z * u + ct) * pz;
  o0 += (a * (y * y + z * z) - x * (b * y + c * z)) * u + (b * z - c * y) * st;
  o1 += (b * (x * x + z * z) - y * (a * x + c * z)) * u + (c * x - a * z) * st;
  o2 += (c * (x * x + y * y) - z * (a * x + b * y)) * u + (a * y - b * x) * st;
  p[0] = o0;
  p[1] = o1;
  p[2] = o2;
}

// op: 0 translate (v = delta), 1 twist (v = axis, s = radian), 2 scale (s).
__global__ void aims_kernel(int op, float* __restrict__ aims, const float* __restrict__ pos,
                            const int32_t* __restrict__ ids, int m, float v0, float v1, float v2,
                            float s) {
  __shared__ float ctr[3];
  if (op != 0) {
    float c[3];
    block_centroid(pos, ids, m, c);
    if (threadIdx.x == 0) {
      ctr[0] = c[0];
      ctr[1] = c[1];
      ctr[2] = c[2];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int j = ids[t];
    bool first = true;
    int reps = 0;
    for (int u = 0; u < m; ++u) {
      if (ids[u] == j) {
        if (u < t) first = false;
        ++reps;
      }
    }
    if (!first) continue;
    float p[3] = {aims[3 * (size_t)j], aims[3 * (size_t)j + 1], aims[3 * (size_t)j + 2]};
    for (int r = 0; r < reps; ++r) {
      if (op == 0) {
        p[0] += v0;
        p[1] += v1;
        p[2] += v2;
      } else if (op == 1) {
        rotate_about_line(p, ctr, v0, v1, v2, s);
      } else {
        p[0] = ctr[0] + s * (p[0] - ctr[0]);
        p[1] = ctr[1] + s * (p[1] - ctr[1]);
        p[2] = ctr[2] + s * (p[2] - ctr[2]);
      }
    }
    aims[3 * (size_t)j] = p[0];
    aims[3 * (size_t)j + 1] = p[1];
    aims[3 * (size_t)j + 2] = p[2];
  }
}

template <int K, bool PLANNED>
static int launch_skin_g(bool mixed, int N, float* ends, const int32_t* eidx, const float* ew,
                         const float* table, const float* scale0, const uint8_t* st, float* pos,
                         float* rot, float* scale, float* shs, float* cov, const SkinPlanDev& plan, int* status,
                         cudaStream_t s) {
  const int grid = grid_for(N, kSkinTile);
  if (PLANNED) {
    // at least 48 KB per CTA: four CTAs per SM.  The kernel's 96 registers
    // would allow five, which measured slower on a GB300 (98.9 against 88.7 us
    // at twist300k): the five CTAs' shared memory leaves L1 almost nothing.
    constexpr int smem = PlanTile<K>::kSmem > 48 * 1024 ? PlanTile<K>::kSmem : 48 * 1024;
    auto kern = mixed ? skin_gaussians_planned_kernel<K, true> : skin_gaussians_planned_kernel<K, false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
      (void)cudaGetLastError();
      return ARAP_ECUDA;
    }
    kern<<<grid, kSkinThreads, smem, s>>>(N, ends, eidx, ew, table, scale0, st, pos, rot, scale, shs, cov, plan,
                                          status);
  } else {
    constexpr size_t smem = skin_smem_bytes();
    auto kern = mixed ? skin_gaussians_kernel<K, true> : skin_gaussians_kernel<K, false>;
    kern<<<grid, kSkinThreads, smem, s>>>(N, ends, eidx, ew, table, scale0, st, pos, rot, scale, shs, cov, status);
  }
  return ARAP_OK;
}

// ---- skinning plan (set-up time)
// One CTA per tile.  It collects the distinct node ids of the tile's endpoint
// neighbours (shared-memory hash), orders each endpoint's neighbours by node
// id (the blend is a sum, so the order only changes its rounding), and then
// chooses each node's local index, that is, where its record sits in shared
// memory during a frame.  A warp's 128-bit record loads are served eight lanes
// at a time, and two different records conflict when their local indices are
// equal mod 8 (records are 48 bytes: bank group (3u + slot) mod 8).  So the
// local index of a node is col + 8 r, with the colour col in 0..7 chosen
// greedily (nodes in order of how many others they share a lane group with)
// to be the colour least used by the nodes already coloured in the lane
// groups (8 consecutive Gaussians, one endpoint, one neighbour slot) it
// appears in, at most 32 nodes per colour.  Indices left unused hold a copy
// of some node of the tile, so every staged record is valid.  The tile's
// count is then the number of records a frame stages (largest index + 1).
// A tile with more than kPlanNodes distinct nodes keeps only its count;
// frames then gather its nodes from the global table in kNN order.
constexpr int kPlanHash = 2048;
constexpr int kPlanThreads = 256;
constexpr int kPlanGroups = kSkinTile / 8;                   // lane groups of a tile
constexpr int kPlanPhases = kPlanGroups * 6 * ARAP_KNN_MAX;  // (lane group, endpoint, slot)
__global__ void __launch_bounds__(kPlanThreads)
    skin_plan_kernel(int N, int K, const int32_t* __restrict__ eidx, const float* __restrict__ ew,
                     int32_t* __restrict__ tile_count, int32_t* __restrict__ tile_nodes,
                     unsigned char* __restrict__ blk, int tile_bytes, uint16_t* __restrict__ inv_off,
                     uint16_t* __restrict__ inv_ref) {
  __shared__ int s_key[kPlanHash];
  __shared__ int s_list[kPlanNodes];                     // distinct ids, then ascending
  __shared__ unsigned char s_rk[kSkinTile * 6 * ARAP_KNN_MAX];  // rank of each sorted neighbour
  __shared__ unsigned char s_ph[kPlanPhases * 8];       // distinct ranks of each lane group's slot
  __shared__ unsigned char s_phn[kPlanPhases];          // their number
  __shared__ int s_deg[kPlanNodes], s_order[kPlanNodes], s_col[kPlanNodes], s_lid[kPlanNodes];
  __shared__ int s_cost[8], s_cap[8];
  __shared__ int s_n, s_over, s_maxlid;
  const int t = threadIdx.x;
  const int tile0 = blockIdx.x * kSkinTile;
  const int cnt = min(kSkinTile, N - tile0);
  for (int q = t; q < kPlanHash; q += kPlanThreads) s_key[q] = -1;
  if (t == 0) {
    s_n = 0;
    s_over = 0;
    s_maxlid = 0;
  }
  __syncthreads();
  const int total = cnt * 6 * K;
  for (int e = t; e < total; e += kPlanThreads) {
    const int g = e / (6 * K), c = e % (6 * K);  // plane c = j * 6 + ep
    const int id = eidx[(size_t)c * N + tile0 + g];
    unsigned h = ((unsigned)id * 2654435761u) & (kPlanHash - 1);
    for (int probe = 0; probe < kPlanHash; ++probe) {
      const int prev = atomicCAS(&s_key[h], -1, id);
      if (prev == -1) {
        const int slot = atomicAdd(&s_n, 1);
        if (slot < kPlanNodes)
          s_list[slot] = id;
        else
          s_over = 1;
        break;
      }
      if (prev == id) break;
      h = (h + 1) & (kPlanHash - 1);
    }
  }
  __syncthreads();
  const int n = s_n;
  if (n > kPlanNodes || s_over) {
    if (t == 0) tile_count[blockIdx.x] = kPlanNodes + 1;
    return;
  }
  // ascending order of the ids (rank by counting; one node per thread)
  static_assert(kPlanNodes <= kPlanThreads, "one node per thread");
  const int my_id = t < n ? s_list[t] : -1;
  int my_rank = 0;
  if (t < n)
    for (int b = 0; b < n; ++b) my_rank += s_list[b] < my_id;
  __syncthreads();
  if (t < n) s_list[my_rank] = my_id;
  __syncthreads();
  // each endpoint's neighbours sorted by id (insertion sort of at most 12);
  // the weights go to their slots now, the ranks wait for the local indices
  unsigned char* tb = blk + (size_t)blockIdx.x * tile_bytes;
  const int KQ = (K + 3) / 4;
  for (int task = t; task < cnt * 6; task += kPlanThreads) {
    const int g = task / 6, ep = task % 6;
    int rk[ARAP_KNN_MAX];
    float w[ARAP_KNN_MAX];
    for (int j = 0; j < K; ++j) {
      const int id = eidx[(size_t)(j * 6 + ep) * N + tile0 + g];
      int lo = 0, hi = n;  // rank of id in the sorted list
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s_list[mid] < id) lo = mid + 1; else hi = mid;
      }
      const float wj = ew[(size_t)(j * 6 + ep) * N + tile0 + g];
      int p = j;
      while (p > 0 && rk[p - 1] > lo) {
        rk[p] = rk[p - 1];
        w[p] = w[p - 1];
        --p;
      }
      rk[p] = lo;
      w[p] = wj;
    }
    for (int j = 0; j < K; ++j) {
      s_rk[(g * 6 + ep) * K + j] = (unsigned char)rk[j];
      const size_t slot = ((size_t)(ep * KQ + (j >> 2)) * kSkinTile + g) * 4 + (j & 3);
      reinterpret_cast<float*>(tb)[slot] = w[j];
    }
  }
  for (int a = t; a < kPlanNodes; a += kPlanThreads) {
    s_deg[a] = 0;
    s_col[a] = -1;
  }
  if (t < 8) s_cap[t] = 0;
  __syncthreads();
  // lane groups: the distinct ranks at one slot of one endpoint over 8
  // consecutive Gaussians, and each node's number of partners in them
  const int phases = kPlanGroups * 6 * K;
  for (int p = t; p < phases; p += kPlanThreads) {
    const int grp = p / (6 * K), r = p % (6 * K), ep = r / K, j = r % K;
    unsigned char m[8];
    int nm = 0;
    for (int l = 0; l < 8; ++l) {
      const int g = grp * 8 + l;
      if (g >= cnt) break;
      const unsigned char v = s_rk[(g * 6 + ep) * K + j];
      bool seen = false;
      for (int x = 0; x < nm; ++x) seen |= m[x] == v;
      if (!seen) m[nm++] = v;
    }
    for (int x = 0; x < nm; ++x) s_ph[p * 8 + x] = m[x];
    s_phn[p] = (unsigned char)nm;
    for (int x = 0; x < nm; ++x) atomicAdd(&s_deg[m[x]], nm - 1);
  }
  __syncthreads();
  // colouring order: most partners first, ties by rank
  for (int a = t; a < n; a += kPlanThreads) {
    int pos = 0;
    for (int b = 0; b < n; ++b) pos += s_deg[b] > s_deg[a] || (s_deg[b] == s_deg[a] && b < a);
    s_order[pos] = a;
  }
  __syncthreads();
  for (int s = 0; s < n; ++s) {
    const int a = s_order[s];
    if (t < 8) s_cost[t] = 0;
    __syncthreads();
    for (int p = t; p < phases; p += kPlanThreads) {
      const unsigned char* m = s_ph + p * 8;
      const int nm = s_phn[p];
      bool has = false;
      for (int x = 0; x < nm; ++x) has |= m[x] == a;
      if (has)
        for (int x = 0; x < nm; ++x)
          if (m[x] != a && s_col[m[x]] >= 0) atomicAdd(&s_cost[s_col[m[x]]], 1);
    }
    __syncthreads();
    if (t == 0) {
      int best = -1;
      for (int c = 0; c < 8; ++c)
        if (s_cap[c] < kPlanNodes / 8 && (best < 0 || s_cost[c] < s_cost[best])) best = c;
      s_col[a] = best;
      s_cap[best] += 1;
    }
    __syncthreads();
  }
  // local index col + 8 * (position among the nodes of its colour, by rank)
  for (int a = t; a < n; a += kPlanThreads) {
    const int c = s_col[a];
    int r = 0;
    for (int b = 0; b < a; ++b) r += s_col[b] == c;
    s_lid[a] = c + 8 * r;
    atomicMax(&s_maxlid, c + 8 * r);
  }
  __syncthreads();
  const int staged = s_maxlid + 1;
  int32_t* tn = tile_nodes + (size_t)blockIdx.x * kPlanNodes;
  for (int u = t; u < staged; u += kPlanThreads) tn[u] = s_list[0];  // unused indices: a valid record
  __syncthreads();
  for (int a = t; a < n; a += kPlanThreads) tn[s_lid[a]] = s_list[a];
  if (t == 0) tile_count[blockIdx.x] = staged;
  unsigned char* lb = tb + (size_t)6 * KQ * kSkinTile * 16;
  for (int e = t; e < cnt * 6 * K; e += kPlanThreads) {
    const int g = e / (6 * K), r = e % (6 * K), ep = r / K, j = r % K;
    lb[((size_t)(ep * KQ + (j >> 2)) * kSkinTile + g) * 4 + (j & 3)] =
        (unsigned char)s_lid[s_rk[(g * 6 + ep) * K + j]];
  }
  // the adjoint's inverse lists: references (g * 6 + ep) * K + j of each
  // slot, in ascending order (s_key, free now, holds the per-slot counts)
  int* s_cnt = s_key;
  for (int u = t; u <= kPlanNodes; u += kPlanThreads) s_cnt[u] = 0;
  __syncthreads();
  const int nref = cnt * 6 * K;
  for (int e = t; e < nref; e += kPlanThreads) atomicAdd(&s_cnt[s_lid[s_rk[e]] + 1], 1);
  __syncthreads();
  if (t == 0)
    for (int u = 1; u <= kPlanNodes; ++u) s_cnt[u] += s_cnt[u - 1];
  __syncthreads();
  uint16_t* io = inv_off + (size_t)blockIdx.x * (kPlanNodes + 1);
  uint16_t* ir = inv_ref + (size_t)blockIdx.x * 6 * K * kSkinTile;
  for (int u = t; u <= kPlanNodes; u += kPlanThreads) io[u] = (uint16_t)s_cnt[u];
  for (int u = t; u < kPlanNodes; u += kPlanThreads) {
    int pos = s_cnt[u];
    if (pos == s_cnt[u + 1]) continue;
    for (int e = 0; e < nref; ++e)
      if (s_lid[s_rk[e]] == u) ir[pos++] = (uint16_t)e;
  }
}


template <int K>
static void launch_skin_s(int S, float* spos, const int32_t* idx, const float* w, const float* table,
                          const float* nq, float* feat, const uint8_t* st, cudaStream_t s) {
  const size_t smem = sizeof(float) * ((feat ? (size_t)kSkinTile * kShStride : 0) + 3 * (size_t)kSkinTile);
  skin_samples_kernel<K><<<grid_for(S, kSkinTile), kSkinThreads, smem, s>>>(S, spos, idx, w, table, nq, feat, st);
}

}  // namespace arap

using namespace arap;

extern "C" int arap_node_table(int n, const float* rot, const float* trans, const float* node_pos,
                               float* table_out, arap_stream_t stream) {
  if (n <= 0 || !rot || !trans || !node_pos || !table_out) return n == 0 ? ARAP_OK : ARAP_EBADINPUT;
  if (reinterpret_cast<uintptr_t>(table_out) & 15) return ARAP_EBADINPUT;
  node_table_kernel<<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(n, rot, trans, node_pos, table_out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_end_points(int N, const float* pos, const float* rot, const float* scale,
                               float* ends_out, float* ends_xyz_out, arap_stream_t stream) {
  if (N == 0) return ARAP_OK;
  if (N < 0 || !pos || !rot || !scale || !ends_out) return ARAP_EBADINPUT;
  if (reinterpret_cast<uintptr_t>(rot) & 15) return ARAP_EBADINPUT;
  end_points_kernel<<<grid_for(N, 128), 128, 0, (cudaStream_t)stream>>>(N, pos, rot, scale, ends_out,
                                                                         ends_xyz_out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_skin_gaussians(int N, int k, float* ends, const int32_t* ends_idx,
                                   const float* ends_w, const float* node_table, const float* scale0,
                                   const uint8_t* static_mask, float* pos_out, float* rot_inout,
                                   float* scale_out, float* shs_inout, float* cov_out, int precision,
                                   int32_t* status, arap_stream_t stream) {
  if (N == 0) return ARAP_OK;
  if (N < 0 || !ends || !ends_idx || !ends_w || !node_table || !scale0 || !pos_out || !rot_inout ||
      !scale_out)
    return ARAP_EBADINPUT;
  if ((reinterpret_cast<uintptr_t>(node_table) | reinterpret_cast<uintptr_t>(rot_inout) |
       reinterpret_cast<uintptr_t>(shs_inout)) & 15)
    return ARAP_EBADINPUT;
  const bool mixed = precision == ARAP_PRECISION_MIXED;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ARAP_OK;
  switch (k) {
#define ARAP_SKG(K)                                                                                   \
  case K:                                                                                             \
    rc = launch_skin_g<K, false>(mixed, N, ends, ends_idx, ends_w, node_table, scale0, static_mask, pos_out, \
                                 rot_inout, scale_out, shs_inout, cov_out, SkinPlanDev{}, status, s);    \
    break;
    ARAP_SKG(1) ARAP_SKG(2) ARAP_SKG(3) ARAP_SKG(4) ARAP_SKG(5) ARAP_SKG(6)
    ARAP_SKG(7) ARAP_SKG(8) ARAP_SKG(9) ARAP_SKG(10) ARAP_SKG(11) ARAP_SKG(12)
#undef ARAP_SKG
    default:
      return ARAP_EUNSUPPORTED;
  }
  if (rc != ARAP_OK) return rc;
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

struct arap_skin_plan {
  int N = 0, k = 0, tiles = 0, tile_bytes = 0, overflow = 0, max_nodes = 0;
  void* block = nullptr;
  SkinPlanDev dev{};
  int* status = nullptr;  // the plan's device status word (inside block)
};

extern "C" int arap_skin_plan_create(arap_skin_plan** out, int N, int k, const int32_t* ends_idx,
                                     const float* ends_w, arap_stream_t stream) {
  if (!out) return ARAP_EBADINPUT;
  *out = nullptr;
  if (N < 1 || k < 1 || k > ARAP_KNN_MAX || !ends_idx || !ends_w) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  auto* p = new (std::nothrow) arap_skin_plan();
  if (!p) return ARAP_ENOMEM;
  p->N = N;
  p->k = k;
  p->tiles = (N + kSkinTile - 1) / kSkinTile;
  p->tile_bytes = plan_tile_bytes(k);
  const size_t b_count = ((sizeof(int32_t) * p->tiles) + 255) & ~size_t(255);
  const size_t b_nodes = ((sizeof(int32_t) * (size_t)p->tiles * kPlanNodes) + 255) & ~size_t(255);
  const size_t b_blk = ((size_t)p->tiles * p->tile_bytes + 255) & ~size_t(255);
  const size_t b_ioff = (sizeof(uint16_t) * (size_t)p->tiles * (kPlanNodes + 1) + 255) & ~size_t(255);
  const size_t b_iref = (sizeof(uint16_t) * (size_t)p->tiles * 6 * k * kSkinTile + 255) & ~size_t(255);
  if (cudaMalloc(&p->block, b_count + b_nodes + b_blk + b_ioff + b_iref + 256) != cudaSuccess) {
    (void)cudaGetLastError();
    delete p;
    return ARAP_ENOMEM;
  }
  char* base = static_cast<char*>(p->block);
  int32_t* count = reinterpret_cast<int32_t*>(base);
  int32_t* nodes = reinterpret_cast<int32_t*>(base + b_count);
  unsigned char* blk = reinterpret_cast<unsigned char*>(base + b_count + b_nodes);
  uint16_t* ioff = reinterpret_cast<uint16_t*>(base + b_count + b_nodes + b_blk);
  uint16_t* iref = reinterpret_cast<uint16_t*>(base + b_count + b_nodes + b_blk + b_ioff);
  p->dev = SkinPlanDev{count, nodes, blk, ioff, iref};
  p->status = reinterpret_cast<int*>(base + b_count + b_nodes + b_blk + b_ioff + b_iref);
  // padded neighbour slots (k not a multiple of 4) and the rows of a partial
  // last tile stay zero; node-list slots the plan kernel leaves unset (past a
  // tile's count, and every slot of an overflow tile) hold node 0
  if (cudaMemsetAsync(blk, 0, b_blk, st) != cudaSuccess || cudaMemsetAsync(p->status, 0, sizeof(int), st) != cudaSuccess ||
      cudaMemsetAsync(nodes, 0, b_nodes, st) != cudaSuccess) {
    arap_skin_plan_destroy(p);
    return ARAP_ECUDA;
  }
  skin_plan_kernel<<<p->tiles, kPlanThreads, 0, st>>>(N, k, ends_idx, ends_w, count, nodes, blk, p->tile_bytes,
                                                      ioff, iref);
  std::vector<int32_t> h(p->tiles);
  if (cudaPeekAtLastError() != cudaSuccess ||
      cudaMemcpyAsync(h.data(), count, sizeof(int32_t) * p->tiles, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    (void)cudaGetLastError();
    arap_skin_plan_destroy(p);
    return ARAP_ECUDA;
  }
  for (int v : h) {
    if (v > kPlanNodes) ++p->overflow;
    else p->max_nodes = std::max(p->max_nodes, v);
  }
  *out = p;
  return ARAP_OK;
}

extern "C" int arap_skin_plan_info(const arap_skin_plan* p, int* tiles, int* overflow_tiles, int* max_nodes) {
  if (!p) return ARAP_EBADINPUT;
  if (tiles) *tiles = p->tiles;
  if (overflow_tiles) *overflow_tiles = p->overflow;
  if (max_nodes) *max_nodes = p->max_nodes;
  return ARAP_OK;
}

extern "C" int arap_skin_plan_status(arap_skin_plan* p, arap_stream_t stream) {
  if (!p) return ARAP_EBADINPUT;
  return status_read_clear(p->status, (cudaStream_t)stream);
}

extern "C" void arap_skin_plan_destroy(arap_skin_plan* p) {
  if (!p) return;
  if (p->block) cudaFree(p->block);
  delete p;
}

extern "C" int arap_skin_gaussians_planned(const arap_skin_plan* plan, float* ends, const int32_t* ends_idx,
                                           const float* ends_w, const float* node_table, const float* scale0,
                                           const uint8_t* static_mask, float* pos_out, float* rot_inout,
                                           float* scale_out, float* shs_inout, float* cov_out, int precision,
                                           arap_stream_t stream) {
  if (!plan || !ends || !ends_idx || !ends_w || !node_table || !scale0 || !pos_out || !rot_inout || !scale_out)
    return ARAP_EBADINPUT;
  if ((reinterpret_cast<uintptr_t>(node_table) | reinterpret_cast<uintptr_t>(rot_inout) |
       reinterpret_cast<uintptr_t>(shs_inout)) & 15)
    return ARAP_EBADINPUT;
  const int N = plan->N;
  const bool mixed = precision == ARAP_PRECISION_MIXED;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ARAP_OK;
  switch (plan->k) {
#define ARAP_SKP(K)                                                                                       \
  case K:                                                                                                 \
    rc = launch_skin_g<K, true>(mixed, N, ends, ends_idx, ends_w, node_table, scale0, static_mask, pos_out, \
                                rot_inout, scale_out, shs_inout, cov_out, plan->dev, plan->status, s);    \
    break;
    ARAP_SKP(1) ARAP_SKP(2) ARAP_SKP(3) ARAP_SKP(4) ARAP_SKP(5) ARAP_SKP(6)
    ARAP_SKP(7) ARAP_SKP(8) ARAP_SKP(9) ARAP_SKP(10) ARAP_SKP(11) ARAP_SKP(12)
#undef ARAP_SKP
    default:
      return ARAP_EUNSUPPORTED;
  }
  if (rc != ARAP_OK) return rc;
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_skin_gaussians_backward(int N, int k, const float* ends_in, const int32_t* ends_idx,
                                            const float* ends_w, const float* node_table, const float* scale0,
                                            const uint8_t* static_mask, const float* grad_pos,
                                            const float* grad_cov, float* grad_node, int32_t* status,
                                            arap_stream_t stream) {
  if (N == 0) return ARAP_OK;
  if (N < 0 || !ends_in || !ends_idx || !ends_w || !node_table || !scale0 || !grad_pos || !grad_cov || !grad_node)
    return ARAP_EBADINPUT;
  if (reinterpret_cast<uintptr_t>(node_table) & 15) return ARAP_EBADINPUT;
  cudaStream_t s = (cudaStream_t)stream;
  const int grid = grid_for(N, kSkinThreads);
  switch (k) {
#define ARAP_SKB(K)                                                                                         \
  case K:                                                                                                   \
    skin_gaussians_backward_kernel<K><<<grid, kSkinThreads, 0, s>>>(N, ends_in, ends_idx, ends_w, node_table, \
                                                                    scale0, static_mask, grad_pos, grad_cov, \
                                                                    grad_node, status);                      \
    break;
    ARAP_SKB(1) ARAP_SKB(2) ARAP_SKB(3) ARAP_SKB(4) ARAP_SKB(5) ARAP_SKB(6)
    ARAP_SKB(7) ARAP_SKB(8) ARAP_SKB(9) ARAP_SKB(10) ARAP_SKB(11) ARAP_SKB(12)
#undef ARAP_SKB
    default:
      return ARAP_EUNSUPPORTED;
  }
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

template <int K>
static int launch_backward_planned(const arap_skin_plan* plan, const float* ends_in, const float* table,
                                   const float* scale0, const uint8_t* st, const float* gpos, const float* gcov,
                                   float* gnode, cudaStream_t s) {
  constexpr int smem = PlanTile<K>::kBytes + 6 * K * kSkinTile * 2;
  if (cudaFuncSetAttribute(skin_gaussians_backward_planned_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  skin_gaussians_backward_planned_kernel<K><<<plan->tiles, kSkinThreads, smem, s>>>(
      plan->N, ends_in, table, scale0, st, gpos, gcov, gnode, plan->dev, plan->status);
  return ARAP_OK;
}

extern "C" int arap_skin_gaussians_backward_planned(const arap_skin_plan* plan, const float* ends_in,
                                                    const int32_t* ends_idx, const float* ends_w,
                                                    const float* node_table, const float* scale0,
                                                    const uint8_t* static_mask, const float* grad_pos,
                                                    const float* grad_cov, float* grad_node, arap_stream_t stream) {
  if (!plan || !ends_in || !ends_idx || !ends_w || !node_table || !scale0 || !grad_pos || !grad_cov || !grad_node)
    return ARAP_EBADINPUT;
  if (reinterpret_cast<uintptr_t>(node_table) & 15) return ARAP_EBADINPUT;
  if (plan->overflow > 0)  // tiles over kPlanNodes nodes: the unplanned adjoint for all
    return arap_skin_gaussians_backward(plan->N, plan->k, ends_in, ends_idx, ends_w, node_table, scale0, static_mask,
                                        grad_pos, grad_cov, grad_node, plan->status, stream);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ARAP_OK;
  switch (plan->k) {
#define ARAP_SKBP(K)                                                                                   \
  case K:                                                                                              \
    rc = launch_backward_planned<K>(plan, ends_in, node_table, scale0, static_mask, grad_pos, grad_cov,      \
                                    grad_node, s);                                                      \
    break;
    ARAP_SKBP(1) ARAP_SKBP(2) ARAP_SKBP(3) ARAP_SKBP(4) ARAP_SKBP(5) ARAP_SKBP(6)
    ARAP_SKBP(7) ARAP_SKBP(8) ARAP_SKBP(9) ARAP_SKBP(10) ARAP_SKBP(11) ARAP_SKBP(12)
#undef ARAP_SKBP
    default:
      return ARAP_EUNSUPPORTED;
  }
  if (rc != ARAP_OK) return rc;
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_node_quaternions(int n, const float* rot, float* quat_out, int precision, int32_t* status,
                                     arap_stream_t stream) {
  if (n == 0) return ARAP_OK;
  if (n < 0 || !rot || !quat_out || (reinterpret_cast<uintptr_t>(quat_out) & 15)) return ARAP_EBADINPUT;
  if (precision == ARAP_PRECISION_MIXED)
    node_quat_kernel<true><<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(n, rot, quat_out, status);
  else
    node_quat_kernel<false><<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(n, rot, quat_out, status);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_skin_samples(int S, int k, float* sample_pos, const int32_t* idx, const float* w,
                                 const float* node_table, const float* node_quat, float* feature,
                                 const uint8_t* static_mask, arap_stream_t stream) {
  if (S == 0) return ARAP_OK;
  if (S < 0 || !sample_pos || !idx || !w || !node_table || (feature && !node_quat)) return ARAP_EBADINPUT;
  if ((reinterpret_cast<uintptr_t>(node_table) | reinterpret_cast<uintptr_t>(node_quat) |
       reinterpret_cast<uintptr_t>(feature)) & 15)
    return ARAP_EBADINPUT;
  cudaStream_t s = (cudaStream_t)stream;
  switch (k) {
#define ARAP_SKS(K)                                                                  \
  case K:                                                                            \
    launch_skin_s<K>(S, sample_pos, idx, w, node_table, node_quat, feature, static_mask, s); \
    break;
    ARAP_SKS(1) ARAP_SKS(2) ARAP_SKS(3) ARAP_SKS(4) ARAP_SKS(5) ARAP_SKS(6)
    ARAP_SKS(7) ARAP_SKS(8) ARAP_SKS(9) ARAP_SKS(10) ARAP_SKS(11) ARAP_SKS(12)
#undef ARAP_SKS
    default:
      return ARAP_EUNSUPPORTED;
  }
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_update_nodes(int n, int k, const float* node_pos, const int32_t* anchor_idx,
                                 const float* anchor_w, const float* node_table, float* node_pos_out,
                                 arap_stream_t stream) {
  if (n == 0) return ARAP_OK;
  if (n < 0 || k < 1 || k > ARAP_KNN_MAX || !node_pos || !anchor_idx || !anchor_w || !node_table ||
      !node_pos_out || node_pos_out == node_pos)
    return ARAP_EBADINPUT;
  update_nodes_kernel<<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(n, k, node_pos, anchor_idx,
                                                                          anchor_w, node_table, node_pos_out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_static_mask(int P, int k, int groups, const int32_t* idx,
                                const uint8_t* node_is_static, uint8_t* mask_out, arap_stream_t stream) {
  if (P == 0) return ARAP_OK;
  if (P < 0 || k < 1 || groups < 1 || !idx || !node_is_static || !mask_out) return ARAP_EBADINPUT;
  static_mask_kernel<<<grid_for(P, 256), 256, 0, (cudaStream_t)stream>>>(P, k * groups, idx, node_is_static,
                                                                         mask_out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

static int launch_aims(int op, float* aims, const float* pos, const int32_t* ids, int m, float a,
                       float b, float c, float s, cudaStream_t st) {
  if (m == 0) return ARAP_OK;
  if (m < 0 || !aims || !ids || (op != 0 && !pos)) return ARAP_EBADINPUT;
  aims_kernel<<<1, 256, 0, st>>>(op, aims, pos, ids, m, a, b, c, s);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_aims_translate(float* aims, const int32_t* active_nodes, int n_active, float dx,
                                   float dy, float dz, arap_stream_t stream) {
  return launch_aims(0, aims, nullptr, active_nodes, n_active, dx, dy, dz, 0.f, (cudaStream_t)stream);
}

extern "C" int arap_aims_twist(float* aims, const float* node_pos, const int32_t* active_nodes,
                               int n_active, float ax, float ay, float az, float radian,
                               arap_stream_t stream) {
  if (!(ax * ax + ay * ay + az * az > 0.f)) return ARAP_EBADINPUT;
  return launch_aims(1, aims, node_pos, active_nodes, n_active, ax, ay, az, radian, (cudaStream_t)stream);
}

extern "C" int arap_aims_scale(float* aims, const float* node_pos, const int32_t* active_nodes,
                               int n_active, float s, arap_stream_t stream) {
  return launch_aims(2, aims, node_pos, active_nodes, n_active, 0.f, 0.f, 0.f, s, (cudaStream_t)stream);
}
