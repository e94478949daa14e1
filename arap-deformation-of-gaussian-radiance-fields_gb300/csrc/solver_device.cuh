// Device side of the Gauss-Newton / PCG solver: per-node residual, gradient
// and energy of the reference's energy (Deform.cpp:378-581) with its Jacobian
// (Deform.cpp:180-376), the matrix-free product (J^T J) p, and the 12x12
// block-Jacobi preconditioner.  One warp owns one free node at a time; lanes
// stride over the node's coupling items and the warp reduces the 12-vector.
#pragma once

#include <type_traits>

#include "solver.cuh"

namespace arap {

constexpr int kSolveThreads = 512;
constexpr int kSolveWarps = kSolveThreads / 32;
constexpr int kRcPerThread = (kMaxCoarse + kSolveThreads - 1) / kSolveThreads;

// ------------------------------------------------------- float-float ----
// The residual, gradient and energy of the mixed form are float-float
// numbers hi + lo (|lo| <= ulp(hi) / 2, about 48 significant bits) computed
// with FP32 operations: this part's FP64 pipe retires a warp instruction
// every 16 SM cycles, against four FP32 instructions a cycle.  Sums are the
// accurate double-word addition (two TwoSums and two fast renormalisations:
// M. Joldes, J.-M. Muller, V. Popescu, "Tight and rigorous error bounds for
// basic building blocks of double-word arithmetic", ACM TOMS 44 (2017),
// algorithm 6, relative error below 3 u^2), products use the FMA for the
// exact error of hi * hi (their algorithm 11 without the lo * lo term).  Every
// step is an explicit round-to-nearest intrinsic, so no contraction into an
// FMA changes it.
struct ff {
  float hi, lo;
  ff() = default;
  __device__ __forceinline__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ ff(float v) : hi(v), lo(0.f) {}
  __device__ __forceinline__ explicit ff(int v) : hi((float)v), lo(0.f) {}
  __device__ __forceinline__ explicit ff(double v) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
  }
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ explicit operator float() const { return __fadd_rn(hi, lo); }
};
__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void ff_fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ ff operator+(ff a, ff b) {
  float s, e, t, f;
  ff_two_sum(a.hi, b.hi, s, e);
  ff_two_sum(a.lo, b.lo, t, f);
  e = __fadd_rn(e, t);
  ff_fast_two_sum(s, e, s, e);
  e = __fadd_rn(e, f);
  ff_fast_two_sum(s, e, s, e);
  return ff(s, e);
}
__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float h, l;
  ff_fast_two_sum(p, e, h, l);
  return ff(h, l);
}
__device__ __forceinline__ ff& operator+=(ff& a, ff b) { return a = a + b; }
__device__ __forceinline__ ff& operator*=(ff& a, ff b) { return a = a * b; }
__device__ __forceinline__ bool operator!=(ff a, ff b) { return a.hi != b.hi || a.lo != b.lo; }
__device__ __forceinline__ ff ff_shfl_xor(ff v, int off) {
  return ff(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
}
__device__ __forceinline__ ff ff_shfl(ff v, int src) {
  return ff(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
__device__ __forceinline__ ff warp_sum(ff v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = v + ff_shfl_xor(v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T shfl_xor_any(T v, int off) {
  if constexpr (std::is_same<T, ff>::value)
    return ff_shfl_xor(v, off);
  else
    return __shfl_xor_sync(0xffffffffu, v, off);
}
template <typename T>
__device__ __forceinline__ T shfl_any(T v, int src) {
  if constexpr (std::is_same<T, ff>::value)
    return ff_shfl(v, src);
  else
    return __shfl_sync(0xffffffffu, v, src);
}
// The energy accumulator of a residual type: float-float for ff, double
// otherwise (the FP32 form's energy is FP64 too).
template <typename RT>
struct EnergyAcc {
  using type = double;
};
template <>
struct EnergyAcc<ff> {
  using type = ff;
};
template <typename RT>
__device__ __forceinline__ void energy_add3(typename EnergyAcc<RT>::type& e, const RT (&f)[3]) {
  if constexpr (std::is_same<RT, ff>::value)
    e += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
  else
    e += double(f[0]) * double(f[0]) + double(f[1]) * double(f[1]) + double(f[2]) * double(f[2]);
}
template <typename RT>
__device__ __forceinline__ void energy_add1(typename EnergyAcc<RT>::type& e, RT f) {
  if constexpr (std::is_same<RT, ff>::value)
    e += f * f;
  else
    e += double(f) * double(f);
}
// A weight sqrt(w) in the residual type (ff: the float rounding and its error,
// kept by the host).
template <typename RT>
__device__ __forceinline__ RT weight_rt(double d, float hi, float lo) {
  if constexpr (std::is_same<RT, ff>::value)
    return ff(hi, lo);
  else
    return RT(d);
}

// Mutable per-node vectors are read through L2 (ld.global.cg): other CTAs
// write them between grid barriers, and L1 is not coherent across SMs.
__device__ __forceinline__ void ld12cg(const float* base, int r, float (&v)[12]) {
  const float4* p = reinterpret_cast<const float4*>(base + 12 * (size_t)r);
  const float4 a = __ldcg(p), b = __ldcg(p + 1), c = __ldcg(p + 2);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  v[8] = c.x; v[9] = c.y; v[10] = c.z; v[11] = c.w;
}

__device__ __forceinline__ void ld3t_cg(const float* base, int r, float (&v)[3]) {
  const float4 c = __ldcg(reinterpret_cast<const float4*>(base + 12 * (size_t)r) + 2);
  v[0] = c.y; v[1] = c.z; v[2] = c.w;
}

// The CTA's shared-memory copy of the coarse correction zc, staged at the
// start of the products phase (12 floats per aggregate, read by its ~64
// nodes and by the constraint items touching it).
__shared__ __align__(16) float s_zc[kMaxCoarse];

// CTA-resident node tables in dynamic shared memory.  Slot s of a CTA is the
// s-th free node it processes (order position s * nbk + bid).  For n staged
// slots, ni coupling items, nl coarse-list entries and nc constraint items the
// layout is
//   [inverse blocks: n x 144 floats][nodes: n int4 {r, item base, items, aggregate}]
//   [bases: n int4 {list base, constraint-item base}][offsets: n float4 g_j - g_pivot]
//   [items: ni int4][geometry: ni float4][list V_ga: nl float4]
//   resident mode only: [PCG vectors: n x 8 x 12 floats][x: n x 12 floats]
//                       [other node's offset: ni float4][w_con J_g u_f: nc float4]
//                       [rotation blocks: n x 9 x 12 floats][coarse blocks: na x 144 floats]
//                       [zc of each coupled aggregate: na x 12 floats]
//                       [coarse-inverse rows of the CTA: nrows x NC floats]
//                       [member-anchor slot geometry: nsl float4][slot range per constraint item: nc int2]
//   [list aggregate: nl int] resident mode only: [constraint group: nc int]
//                                                [coupled aggregate: na int][slot free rank: nsl int]
// Staged constraint items carry {kind | constraint-item index << 4, list base,
// g, list length} and, for every item, the geometry a product needs
// ({sgn (g_k - g_j), w scale} for regularisation items, {a, v_c - g_l} for
// constraint items).
extern __shared__ __align__(16) unsigned char s_dyn[];
struct StageLayout {
  int n;                                   // staged slots (even unless all of the CTA's nodes are staged)
  int nd, nx, dp, it, ax, gv, vec, xf, yd, cu, rot, mm, zz, crow, gsg, cgs, ga, cg, mag, gsr;  // byte offsets
  int ncon;                                // constraint items of the staged slots
  int nent;                                // coupled-aggregate entries of the staged slots
  int nrows;                               // coarse-inverse rows held (resident mode)
};
__shared__ StageLayout s_stg;

__device__ __forceinline__ float* stg_dinv(int s) { return reinterpret_cast<float*>(s_dyn) + 144 * s; }
__device__ __forceinline__ int4* stg_node() { return reinterpret_cast<int4*>(s_dyn + s_stg.nd); }
__device__ __forceinline__ int4* stg_base() { return reinterpret_cast<int4*>(s_dyn + s_stg.nx); }
__device__ __forceinline__ float4* stg_dpiv() { return reinterpret_cast<float4*>(s_dyn + s_stg.dp); }
__device__ __forceinline__ int4* stg_item() { return reinterpret_cast<int4*>(s_dyn + s_stg.it); }
__device__ __forceinline__ float4* stg_geo() { return reinterpret_cast<float4*>(s_dyn + s_stg.ax); }
__device__ __forceinline__ float4* stg_lv() { return reinterpret_cast<float4*>(s_dyn + s_stg.gv); }
__device__ __forceinline__ int* stg_la() { return reinterpret_cast<int*>(s_dyn + s_stg.ga); }
// resident mode: PCG vector k of slot s (12 floats), x of slot s, the other
// node's offset of item i, w_con J_g u_f and group of constraint item c
// In the V-cycle iteration: RV_UF holds z1 = D^-1 r (phases 1-4), then z3
// (phases 4-5); RV_WF holds A z1 (phases 2-4), then A z2 (phases 4-5); RV_W
// holds the regularisation part of a product while it is formed, then w;
// RV_R, RV_P, RV_S, RV_H, RV_U are the PCG's r, p, s = A p, h and u.
enum { RV_UF = 0, RV_R, RV_P, RV_S, RV_H, RV_U, RV_W, RV_WF };
__device__ __forceinline__ float* stg_vec(int s, int k) {
  return reinterpret_cast<float*>(s_dyn + s_stg.vec) + 12 * (kResVecs * s + k);
}
__device__ __forceinline__ float* stg_xf(int s) { return reinterpret_cast<float*>(s_dyn + s_stg.xf) + 12 * s; }
__device__ __forceinline__ float4* stg_ydp() { return reinterpret_cast<float4*>(s_dyn + s_stg.yd); }
__device__ __forceinline__ float* stg_rot(int s) { return reinterpret_cast<float*>(s_dyn + s_stg.rot) + 108 * s; }
__device__ __forceinline__ float* stg_mm(int e) { return reinterpret_cast<float*>(s_dyn + s_stg.mm) + 144 * e; }
__device__ __forceinline__ float* stg_crow(int j, int NC) {
  return reinterpret_cast<float*>(s_dyn + s_stg.crow) + (size_t)j * NC;
}
__device__ __forceinline__ int* stg_mag() { return reinterpret_cast<int*>(s_dyn + s_stg.mag); }
__device__ __forceinline__ float* stg_zz(int e) { return reinterpret_cast<float*>(s_dyn + s_stg.zz) + 12 * e; }
__device__ __forceinline__ float4* stg_gsg() { return reinterpret_cast<float4*>(s_dyn + s_stg.gsg); }
__device__ __forceinline__ int2* stg_cgs() { return reinterpret_cast<int2*>(s_dyn + s_stg.cgs); }
__device__ __forceinline__ int* stg_gsr() { return reinterpret_cast<int*>(s_dyn + s_stg.gsr); }
__device__ __forceinline__ float4* stg_cuz() { return reinterpret_cast<float4*>(s_dyn + s_stg.cu); }
__device__ __forceinline__ int* stg_cg() { return reinterpret_cast<int*>(s_dyn + s_stg.cg); }

// Coarse correction of a free node with offset dp = g_j - g_pivot(a) in
// aggregate a: z += P_j zc[a] with dR_j = dR_a, dt_j = dR_a dp + dT_a, zc
// from s_zc.
__device__ __forceinline__ void coarse_prolong_dp(const float4 dp, int a, float (&v)[12]) {
  const float d0 = dp.x, d1 = dp.y, d2 = dp.z;
  const float4* c4 = reinterpret_cast<const float4*>(s_zc + 12 * a);
  const float4 ca = c4[0], cb = c4[1], cc = c4[2];
  const float c[12] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w, cc.x, cc.y, cc.z, cc.w};
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] += c[i];
#pragma unroll
  for (int r = 0; r < 3; ++r) v[9 + r] += c[9 + r] + d0 * c[r] + d1 * c[3 + r] + d2 * c[6 + r];
}

__device__ __forceinline__ void coarse_prolong(const SolveParams& P, int rr, int a, float (&v)[12]) {
  coarse_prolong_dp(__ldcg(P.dpiv + rr), a, v);
}

// Preconditioned residual u = u_f + P zc of free node rr in aggregate agg,
// formed on the fly (u_f = Dinv r in P.z; the coarse correction, from s_zc,
// when the two-level preconditioner is on).
__device__ __forceinline__ void load_u(const SolveParams& P, int rr, int agg, float (&v)[12]) {
  ld12cg(P.z, rr, v);
  if (P.NA) coarse_prolong(P, rr, agg, v);
}

// Translation part of u for free node rr.
__device__ __forceinline__ void load_ut(const SolveParams& P, int rr, int agg, float (&v)[3]) {
  if (P.NA) {
    float f[12];
    load_u(P, rr, agg, f);
    v[0] = f[9];
    v[1] = f[10];
    v[2] = f[11];
    return;
  }
  ld3t_cg(P.z, rr, v);
}

// Offset from the identity transform, dx = x + scale*h - [I | 0], of free
// node rr.  Residuals are evaluated from dx so that float32 arithmetic does not
// cancel O(1) terms ((R - I) d instead of R d - d, 2 dx_00 + |dx_0|^2 instead
// of |c_0|^2 - 1); the formulas are algebraically those of Deform.cpp:378-581.
template <typename RT>
__device__ __forceinline__ void load_x(const SolveParams& P, int rr, RT scale, RT (&v)[12]) {
  if constexpr (std::is_same<RT, ff>::value) {
    // the float-float copy of x - [I | 0], kept beside x
    const float4* xo = reinterpret_cast<const float4*>(P.xo + 12 * (size_t)rr);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const float4 u = __ldcg(xo + q);
      v[2 * q] = ff(u.x, u.y);
      v[2 * q + 1] = ff(u.z, u.w);
    }
    if (scale != RT(0)) {
      float hv[12];
      ld12cg(P.h, rr, hv);
#pragma unroll
      for (int i = 0; i < 12; ++i) v[i] = v[i] + scale * RT(hv[i]);
    }
    return;
  }
  const double* xp = P.x + 12 * (size_t)rr;
  double d[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) d[i] = __ldcg(xp + i) - ((i == 0 || i == 4 || i == 8) ? 1.0 : 0.0);
  if (scale != RT(0)) {
    float hv[12];
    ld12cg(P.h, rr, hv);
#pragma unroll
    for (int i = 0; i < 12; ++i) v[i] = RT(d[i]) + scale * RT(hv[i]);
  } else {
#pragma unroll
    for (int i = 0; i < 12; ++i) v[i] = RT(d[i]);
  }
}

template <typename RT>
__device__ __forceinline__ void load_xt(const SolveParams& P, int rr, RT scale, RT (&v)[3]) {
  if constexpr (std::is_same<RT, ff>::value) {
    const float2* xo = P.xo + 12 * (size_t)rr + 9;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float2 u = __ldcg(xo + i);
      v[i] = ff(u.x, u.y);
    }
    if (scale != RT(0)) {
      float hv[3];
      ld3t_cg(P.h, rr, hv);
#pragma unroll
      for (int i = 0; i < 3; ++i) v[i] = v[i] + scale * RT(hv[i]);
    }
    return;
  }
  const double* xp = P.x + 12 * (size_t)rr + 9;
  if (scale != RT(0)) {
    float hv[3];
    ld3t_cg(P.h, rr, hv);
#pragma unroll
    for (int i = 0; i < 3; ++i) v[i] = RT(__ldcg(xp + i)) + scale * RT(hv[i]);
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) v[i] = RT(__ldcg(xp + i));
  }
}

// A constraint group's residual component, stored by the group pass: a
// double, or for float-float the (hi, lo) pair in the same 8 bytes.
template <typename RT>
__device__ __forceinline__ RT load_grp_f(const SolveParams& P, int g, int c) {
  if constexpr (std::is_same<RT, ff>::value) {
    const float2 u = __ldcg(reinterpret_cast<const float2*>(P.grp_f) + 3 * (size_t)g + c);
    return ff(u.x, u.y);
  } else {
    return RT(__ldcg(P.grp_f + 3 * (size_t)g + c));
  }
}
template <typename RT>
__device__ __forceinline__ void store_grp_f(const SolveParams& P, int g, int c, RT f) {
  if constexpr (std::is_same<RT, ff>::value)
    reinterpret_cast<float2*>(P.grp_f)[3 * (size_t)g + c] = make_float2(f.hi, f.lo);
  else
    P.grp_f[3 * (size_t)g + c] = double(f);
}

template <typename RT>
__device__ __forceinline__ void load_pos(const SolveParams& P, int node, RT (&v)[3]) {
  const float* p = P.node_pos + 3 * (size_t)node;
  v[0] = RT(__ldg(p));
  v[1] = RT(__ldg(p + 1));
  v[2] = RT(__ldg(p + 2));
}

// Constraint-group residual f_g (Deform.cpp:484-580) at x + scale*h:
// wc * (sum_members sum_anchors a (R_l (v_c - g_l) + g_l + t_l)  [free l]
//                                 a v_c                           [other l]
//        - mult * target)
// evaluated as wc * (sum_u [sum_free a ((R_l - I)(v_c - g_l) + t_l) + v_c sum a]
//                    - mult * target).
// One warp, lanes over the group's (member, anchor) slots; every lane returns f.
template <typename RT>
__device__ void con_residual_warp(const SolveParams& P, int g, RT scale, RT (&f)[3]) {
  const int lane = threadIdx.x & 31;
  const int k = P.k;
  const int s0 = __ldg(P.grp_off + g) * k, s1 = __ldg(P.grp_off + g + 1) * k;
  RT acc[3] = {RT(0), RT(0), RT(0)}, base[3] = {RT(0), RT(0), RT(0)};
  for (int slot = s0 + lane; slot < s1; slot += 32) {
    RT v[3];
    load_pos<RT>(P, __ldg(P.grp_member + slot / k), v);
    const RT a = RT(__ldg(P.mem_w + slot));
#pragma unroll
    for (int c = 0; c < 3; ++c) base[c] += a * v[c];
    const int rk = __ldg(P.mem_rank + slot);
    if (rk >= 0) {
      RT gl[3], X[12];
      load_pos<RT>(P, __ldg(P.mem_node + slot), gl);
      load_x<RT>(P, rk, scale, X);
      const RT d0 = v[0] - gl[0], d1 = v[1] - gl[1], d2 = v[2] - gl[2];
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] += a * (X[c] * d0 + X[3 + c] * d1 + X[6 + c] * d2 + X[9 + c]);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    acc[c] = warp_sum(acc[c]);
    base[c] = warp_sum(base[c]);
  }
  const float4 tg = P.grp_target[g];
  const RT wc = weight_rt<RT>(P.wc, P.wcf, P.wc_lo);
  f[0] = wc * (acc[0] + (base[0] - RT(tg.w) * RT(tg.x)));
  f[1] = wc * (acc[1] + (base[1] - RT(tg.w) * RT(tg.y)));
  f[2] = wc * (acc[2] + (base[2] - RT(tg.w) * RT(tg.z)));
}

// J_g u of a constraint group (linear part only), from the anchors' u.
__device__ void con_ju(const SolveParams& P, int g, float (&u)[3]) {
  u[0] = u[1] = u[2] = 0.f;
  const int k = P.k;
  const int s0 = __ldg(P.grp_off + g), s1 = __ldg(P.grp_off + g + 1);
  for (int s = s0; s < s1; ++s) {
#pragma unroll 4
    for (int t = 0; t < k; ++t) {
      const int slot = s * k + t;
      const int rk = __ldg(P.mem_rank + slot);
      if (rk < 0) continue;
      const float4 geo = __ldcg(P.mem_geo + slot);
      float pl[12];
      load_u(P, rk, P.NA ? __ldg(P.mem_agg + slot) : 0, pl);
#pragma unroll
      for (int c = 0; c < 3; ++c)
        u[c] = fmaf(geo.x, fmaf(geo.y, pl[c], fmaf(geo.z, pl[3 + c], fmaf(geo.w, pl[6 + c], pl[9 + c]))), u[c]);
    }
  }
  const float wcf = P.wcf;
  u[0] *= wcf;
  u[1] *= wcf;
  u[2] *= wcf;
}

// J_g u of a constraint group with the two-level preconditioner, by
// linearity of u = u_f + P zc: w_con J_g u_f (computed once per group in the
// coarse-solve phase) plus the coarse part w_con sum_a V_ga . zc_a.
__device__ void con_ju_coarse(const SolveParams& P, int g, float (&u)[3]) {
  const float4 uz = __ldcg(P.uzg + g);
  u[0] = uz.x;
  u[1] = uz.y;
  u[2] = uz.z;
  const float wcf = P.wcf;
  const int f0 = __ldg(P.gca_off + g), f1 = __ldg(P.gca_off + g + 1);
  for (int f = f0; f < f1; ++f) {
    const float4 V = __ldcg(P.gcv + f);
    const float4* c4 = reinterpret_cast<const float4*>(s_zc + 12 * __ldg(P.gca + f));
    const float4 ca = c4[0], cb = c4[1], cc = c4[2];
    const float C[12] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w, cc.x, cc.y, cc.z, cc.w};
#pragma unroll
    for (int c = 0; c < 3; ++c)
      u[c] = fmaf(wcf, fmaf(V.x, C[c], fmaf(V.y, C[3 + c], fmaf(V.z, C[6 + c], V.w * C[9 + c]))), u[c]);
  }
}

// con_ju_coarse of a staged constraint item: the group's aggregates and
// V_ga are the len entries of the CTA's coarse list from off.
__device__ __forceinline__ void con_ju_list(const SolveParams& P, int g, int off, int len, float (&u)[3]) {
  const float4 uz = __ldcg(P.uzg + g);
  u[0] = uz.x;
  u[1] = uz.y;
  u[2] = uz.z;
  const float wcf = P.wcf;
  for (int f = off; f < off + len; ++f) {
    const float4 V = stg_lv()[f];
    const float4* c4 = reinterpret_cast<const float4*>(s_zc + 12 * stg_la()[f]);
    const float4 ca = c4[0], cb = c4[1], cc = c4[2];
    const float C[12] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w, cc.x, cc.y, cc.z, cc.w};
#pragma unroll
    for (int c = 0; c < 3; ++c)
      u[c] = fmaf(wcf, fmaf(V.x, C[c], fmaf(V.y, C[3 + c], fmaf(V.z, C[6 + c], V.w * C[9 + c]))), u[c]);
  }
}

// w_con J_g u_f of group g (u_f = Dinv r in P.z); one warp, lane 0 stores it,
// every lane returns it in u.
__device__ __forceinline__ void con_jz_group(const SolveParams& P, int g, float (&u)[3]) {
  const int lane = threadIdx.x & 31;
  const int k = P.k;
  const int s0 = __ldg(P.grp_off + g) * k, s1 = __ldg(P.grp_off + g + 1) * k;
  u[0] = u[1] = u[2] = 0.f;
  for (int slot = s0 + lane; slot < s1; slot += 32) {
    const int rk = __ldg(P.mem_rank + slot);
    if (rk < 0) continue;
    const float4 geo = __ldcg(P.mem_geo + slot);
    float zl[12];
    ld12cg(P.z, rk, zl);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      u[c] = fmaf(geo.x, fmaf(geo.y, zl[c], fmaf(geo.z, zl[3 + c], fmaf(geo.w, zl[6 + c], zl[9 + c]))), u[c]);
  }
  const float wcf = P.wcf;
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = wcf * warp_sum(u[c]);
  if (lane == 0) P.uzg[g] = make_float4(u[0], u[1], u[2], 0.f);
}
__device__ __forceinline__ void con_jz_group(const SolveParams& P, int g) {
  float u[3];
  con_jz_group(P, g, u);
}

// 4x4 symmetric accumulator index (a <= b).
__device__ __forceinline__ constexpr int qi(int a, int b) {
  return a == 0 ? b : (a == 1 ? 3 + b : (a == 2 ? 5 + b : 9));
}

__device__ __forceinline__ void q_add(float (&Q)[10], float v0, float v1, float v2, float v3) {
  const float v[4] = {v0, v1, v2, v3};
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = a; b < 4; ++b) Q[qi(a, b)] = fmaf(v[a], v[b], Q[qi(a, b)]);
}

enum { PASS_GRAD = 0, PASS_ENERGY = 1 };

// One of three values, chosen by i in 0..2 (selects, no indexed registers).
template <typename T>
__device__ __forceinline__ T sel3(int i, T a, T b, T c) {
  return i == 0 ? a : (i == 1 ? b : c);
}

// Sums v[0..15] over the warp by recursive halving: at each step a lane keeps
// the half of its values that its partner sends away, so 16 values take
// 8 + 4 + 2 + 1 + 1 additions instead of 16 x 5.  Lane l returns the total
// of value l >> 1.  The FP64 pipe of this part retires a warp instruction
// every 16 SM cycles, shared by all warps of the SM; the butterfly of each
// value separately was a third of the gradient pass.
template <typename T>
__device__ __forceinline__ T warp_reduce_scatter16(T (&v)[16]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int h = 8, off = 16; h >= 1; h >>= 1, off >>= 1) {
    const bool up = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const T keep = up ? v[h + i] : v[i];
      const T send = up ? v[i] : v[h + i];
      v[i] = keep + shfl_xor_any(send, off);
    }
  }
  return v[0] + shfl_xor_any(v[0], 1);
}

// Residual rows owned by free node r, at x + scale*h.  PASS_GRAD also returns
// in g_lane the lane's entry of (J^T f)_r (every item touching x_r; lanes
// 0..11, the others 0) and Q, the 4x4 kernel of the non-rotation part of the
// diagonal block of J^T J (valid in every lane).  All lanes of the warp call
// it; energy is warp-reduced and valid in every lane.
template <typename RT, int PASS>
__device__ void residual_node(const SolveParams& P, int r, RT scale, RT& g_lane, float (&Q)[10],
                              double& energy) {
  const int lane = threadIdx.x & 31;
  const int j = __ldg(P.free_ids + r);
  RT gj[3];
  load_pos<RT>(P, j, gj);
  const float gjf[3] = {__ldg(P.node_pos + 3 * (size_t)j), __ldg(P.node_pos + 3 * (size_t)j + 1),
                        __ldg(P.node_pos + 3 * (size_t)j + 2)};
  RT xj[12];
  load_x<RT>(P, r, scale, xj);
  RT acc[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) acc[i] = RT(0);
#pragma unroll
  for (int i = 0; i < 10; ++i) Q[i] = 0.f;
  typename EnergyAcc<RT>::type e(0);
  const RT w = weight_rt<RT>(P.wg, P.wgf, P.wg_lo);
  const int b0 = __ldg(P.item_off + r), b1 = __ldg(P.item_off + r + 1);
  // Every item kind in one instruction stream: a lane's operands are chosen
  // by its item's kind, and the FP64 arithmetic (whose pipe retires a warp
  // instruction every 16 SM cycles here, shared by the SM's warps) runs once
  // for all kinds instead of once per kind present in the warp.  Per kind
  // (Deform.cpp:421-449, 458-482, 484-580; the Jacobian's float differences
  // and unscaled t_j column, Deform.cpp:254-257):
  //   OUT     f = w s (R_j d + t_j - t_k), d = g_k - g_j   acc_R += w s dJ f, acc_t += w f
  //   IN      f = w s (R_i d + t_i - t_j), d = g_j - g_i   acc_t += -w s f
  //   STATIC  f = -w t_j                                    acc_t += -w f
  //   CON     f = f_g (the group pass's residual)           acc_R += w_c a dv f, acc_t += w_c a f
  // evaluated as f = ws (X d + (tA - tB)) and acc_R(c) += alpha_c f,
  // acc_t += beta f, with the same operations per kind as the formulas.
  for (int it = b0 + lane; it < b1; it += 32) {
    const int4 m = __ldg(P.items + it);
    const int kind = m.x & 15;
    if (PASS == PASS_ENERGY && (kind == ITEM_IN || kind == ITEM_CON)) continue;
    const bool out = kind == ITEM_OUT, in = kind == ITEM_IN, con = kind == ITEM_CON;
    const float s = __int_as_float(m.w);
    RT X[12], tA[3], tB[3], d[3];
    RT ws = w;
    float4 geo = make_float4(0.f, 0.f, 0.f, 0.f);
    float dJ[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 0; i < 12; ++i) X[i] = xj[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      tA[c] = RT(0);
      tB[c] = xj[9 + c];
      d[c] = RT(0);
    }
    if (out || in) {
      ws = w * RT(s);
      RT go[3];
      load_pos<RT>(P, m.z, go);
      if (out) {
        RT tk[3] = {RT(0), RT(0), RT(0)};
        if (m.y >= 0) load_xt<RT>(P, m.y, scale, tk);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          d[c] = go[c] - gj[c];
          tA[c] = xj[9 + c];
          tB[c] = tk[c];
          dJ[c] = __ldg(P.node_pos + 3 * (size_t)m.z + c) - gjf[c];
        }
      } else {
        load_x<RT>(P, m.y, scale, X);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          d[c] = gj[c] - go[c];
          tA[c] = X[9 + c];
        }
      }
    } else if (con) {
      geo = __ldcg(P.mem_geo + m.y);
      ws = RT(1);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        tA[c] = load_grp_f<RT>(P, m.z, c);
        tB[c] = RT(0);
      }
    }
    RT f[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] = ws * (X[c] * d[0] + X[3 + c] * d[1] + X[6 + c] * d[2] + (tA[c] - tB[c]));
    if (!in && !con) energy_add3<RT>(e, f);
    if (PASS == PASS_GRAD) {
      const RT wa = con ? weight_rt<RT>(P.wc, P.wcf, P.wc_lo) * RT(geo.x) : RT(0);
      const RT beta = out ? w : (con ? wa : -ws);  // IN: -w s; STATIC: -w
      const RT acoef = out ? ws : wa;              // 0 for IN and STATIC
      const float vec[3] = {con ? geo.y : dJ[0], con ? geo.z : dJ[1], con ? geo.w : dJ[2]};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const RT alpha = acoef * RT(vec[c]);
#pragma unroll
        for (int rr = 0; rr < 3; ++rr) acc[3 * c + rr] += alpha * f[rr];
      }
#pragma unroll
      for (int rr = 0; rr < 3; ++rr) acc[9 + rr] += beta * f[rr];
      // the 4x4 kernel of the diagonal block (float)
      if (out) {
        const float wgf = P.wgf;
        const float wsf = wgf * s;
        q_add(Q, wsf * dJ[0], wsf * dJ[1], wsf * dJ[2], wgf);
      } else if (in) {
        Q[9] += (float)((P.wg * s) * (P.wg * s));
      } else if (con) {
        // this item's share, summed once per solve over the group's anchors
        // equal to j (zero for all but the first item of a run)
        const float4 cq = __ldcg(P.item_cq + it);
        if (cq.w != 0.f) {
          const float wcf = P.wcf;
          q_add(Q, wcf * cq.x, wcf * cq.y, wcf * cq.z, wcf * cq.w);
        }
      } else {
        Q[9] += (float)(P.wg * P.wg);
      }
    }
  }
  // orthogonality rows (Deform.cpp:384-404) from the offsets D = R - I, one
  // row per lane 0..5 (the same instructions for all six, the operands chosen
  // per lane): rows (a, b) = (0,1) (0,2) (1,2) (0,0) (1,1) (2,2),
  //   f = w_rot (D_ab + D_ba + D_a . D_b)
  // (c_a . c_b for a != b, |c_a|^2 - 1 for a == b; D_a is column a)
  const RT wr = weight_rt<RT>(P.wr, P.wrf, P.wr_lo);
  RT fo = RT(0);
  {
    const int a = (lane == 2 || lane == 4) ? 1 : (lane == 5 ? 2 : 0);
    const int b = (lane == 0 || lane == 4) ? 1 : ((lane == 1 || lane == 2 || lane == 5) ? 2 : 0);
    RT Da[3], Db[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Da[i] = sel3(a, xj[i], xj[3 + i], xj[6 + i]);
      Db[i] = sel3(b, xj[i], xj[3 + i], xj[6 + i]);
    }
    const RT f = wr * (sel3(b, Da[0], Da[1], Da[2]) + sel3(a, Db[0], Db[1], Db[2]) +
                       (Da[0] * Db[0] + Da[1] * Db[1] + Da[2] * Db[2]));
    if (lane < 6) fo = f;
  }
  energy_add1<RT>(e, fo);
  if (PASS == PASS_GRAD) {
    // lane L < 9 adds d/dR(col, c) of the six rows, col = L / 3, c = L % 3:
    //   col 0: w_rot (f0 c1 + f1 c2 + 2 f3 c0), col 1: w_rot (f0 c0 + f2 c2 + 2 f4 c1),
    //   col 2: w_rot (f1 c0 + f2 c1 + 2 f5 c2), c_X = column X of R, entry c
    const int col = lane < 3 ? 0 : (lane < 6 ? 1 : 2), c = lane - 3 * col;
    const RT fA = shfl_any(fo, col == 2 ? 1 : 0);
    const RT fB = shfl_any(fo, col == 0 ? 1 : 2);
    const RT fD = shfl_any(fo, 3 + col);
    const int pA = col == 0 ? 1 : 0, pB = col == 1 ? 2 : (col == 0 ? 2 : 1);
    RT cc[3];  // entry c of the columns of R
#pragma unroll
    for (int X = 0; X < 3; ++X)
      cc[X] = sel3(c, xj[3 * X], xj[3 * X + 1], xj[3 * X + 2]) + ((X == c) ? RT(1) : RT(0));
    const RT go = wr * (fA * sel3(pA, cc[0], cc[1], cc[2]) + fB * sel3(pB, cc[0], cc[1], cc[2]) +
                        RT(2) * fD * sel3(col, cc[0], cc[1], cc[2]));
    RT v[16];
#pragma unroll
    for (int i = 0; i < 12; ++i) v[i] = acc[i];
#pragma unroll
    for (int i = 12; i < 16; ++i) v[i] = RT(0);
    const RT tot = warp_reduce_scatter16(v);  // lane l: entry l >> 1
    g_lane = shfl_any(tot, 2 * (lane & 15));
    if (lane < 9) g_lane += go;
    if (lane >= 12) g_lane = RT(0);
#pragma unroll
    for (int i = 0; i < 10; ++i) Q[i] = warp_sum(Q[i]);
  }
  energy = (double)warp_sum(e);
}

// One coupling item of a product, fetched: the item, its geometry (d, ws for
// regularisation rows, mem_geo for constraint items) and the other node's
// vector (u_k translation for ITEM_OUT, u_i for ITEM_IN, J_g u for ITEM_CON).
struct CouplingData {
  int kind;
  float4 aux;
  float v[12];
};

__device__ __forceinline__ void fetch_item(const SolveParams& P, int it, const float (&gj)[3], float w,
                                           CouplingData& D) {
  const int4 m = __ldg(P.items + it);
  D.kind = m.x & 15;
#pragma unroll
  for (int i = 0; i < 12; ++i) D.v[i] = 0.f;
  if (D.kind == ITEM_OUT || D.kind == ITEM_IN) {
    const float sgn = D.kind == ITEM_OUT ? 1.f : -1.f;
    D.aux = make_float4(sgn * (__ldg(P.node_pos + 3 * (size_t)m.z) - gj[0]),
                        sgn * (__ldg(P.node_pos + 3 * (size_t)m.z + 1) - gj[1]),
                        sgn * (__ldg(P.node_pos + 3 * (size_t)m.z + 2) - gj[2]), w * __int_as_float(m.w));
    if (D.kind == ITEM_IN) {
      load_u(P, m.y, m.x >> 4, D.v);
    } else if (m.y >= 0) {
      float t3[3];
      load_ut(P, m.y, m.x >> 4, t3);
      D.v[0] = t3[0];
      D.v[1] = t3[1];
      D.v[2] = t3[2];
    }
  } else if (D.kind == ITEM_CON) {
    float u[3];
    if (P.NA)
      con_ju_coarse(P, m.z, u);
    else
      con_ju(P, m.z, u);
    D.v[0] = u[0];
    D.v[1] = u[1];
    D.v[2] = u[2];
    D.aux = __ldcg(P.mem_geo + m.y);
  }
}

__device__ __forceinline__ void apply_item(const SolveParams& P, const CouplingData& D, float w,
                                           const float (&pj)[12], float (&acc)[12]) {
  if (D.kind == ITEM_OUT) {
    const float ws = D.aux.w;
    const float d[3] = {D.aux.x, D.aux.y, D.aux.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float u = ws * fmaf(pj[c], d[0], fmaf(pj[3 + c], d[1], pj[6 + c] * d[2])) + w * pj[9 + c] - ws * D.v[c];
      acc[c] = fmaf(ws * d[0], u, acc[c]);
      acc[3 + c] = fmaf(ws * d[1], u, acc[3 + c]);
      acc[6 + c] = fmaf(ws * d[2], u, acc[6 + c]);
      acc[9 + c] = fmaf(w, u, acc[9 + c]);
    }
  } else if (D.kind == ITEM_IN) {
    const float ws = D.aux.w;
    const float d[3] = {D.aux.x, D.aux.y, D.aux.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float u = ws * fmaf(D.v[c], d[0], fmaf(D.v[3 + c], d[1], D.v[6 + c] * d[2])) + w * D.v[9 + c] -
                      ws * pj[9 + c];
      acc[9 + c] = fmaf(-ws, u, acc[9 + c]);
    }
  } else if (D.kind == ITEM_STATIC) {
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[9 + c] = fmaf(w * w, pj[9 + c], acc[9 + c]);
  } else {
    const float wa = P.wcf * D.aux.x;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      acc[c] = fmaf(wa * D.aux.y, D.v[c], acc[c]);
      acc[3 + c] = fmaf(wa * D.aux.z, D.v[c], acc[3 + c]);
      acc[6 + c] = fmaf(wa * D.aux.w, D.v[c], acc[6 + c]);
      acc[9 + c] = fmaf(wa, D.v[c], acc[9 + c]);
    }
  }
}

// w = (J^T J u)_r for free node r, computed by one half-warp (16 lanes), with
// u formed on the fly for every node it touches; also returns this node's u in
// every lane of the half.  A half with valid == false does no loads but takes
// part in the warp shuffles.
static __device__ __noinline__ void spmv_node(const SolveParams& P, int r, bool valid, float (&acc)[12], float (&pj)[12]) {
  const int lane = threadIdx.x & 15;
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    acc[i] = 0.f;
    pj[i] = 0.f;
  }
  if (valid) {
  const int j = __ldg(P.free_ids + r);
  const float gj[3] = {__ldg(P.node_pos + 3 * (size_t)j), __ldg(P.node_pos + 3 * (size_t)j + 1),
                       __ldg(P.node_pos + 3 * (size_t)j + 2)};
  load_u(P, r, P.NA ? __ldg(P.agg + r) : 0, pj);
  const float w = P.wgf;
  const int b0 = __ldg(P.item_off + r), b1 = __ldg(P.item_off + r + 1);
  // two items per lane per round: both items' loads are issued before either
  // is used, so a round costs one round trip
  for (int it = b0 + lane; it < b1; it += 32) {
    const bool hasB = it + 16 < b1;
    CouplingData A, B;
    fetch_item(P, it, gj, w, A);
    if (hasB) fetch_item(P, it + 16, gj, w, B);
    apply_item(P, A, w, pj, acc);
    if (hasB) apply_item(P, B, w, pj, acc);
  }
  if (lane == 0) {
    // J_rot^T J_rot p with J_rot at the current x (float copy)
    float X[9];
    const float4* xp = reinterpret_cast<const float4*>(P.xf + 12 * (size_t)r);
    const float4 a = __ldcg(xp), b = __ldcg(xp + 1), c = __ldcg(xp + 2);
    X[0] = a.x; X[1] = a.y; X[2] = a.z; X[3] = a.w; X[4] = b.x; X[5] = b.y; X[6] = b.z; X[7] = b.w; X[8] = c.x;
    const float* c0 = X;
    const float* c1 = X + 3;
    const float* c2 = X + 6;
    const float* p0 = pj;
    const float* p1 = pj + 3;
    const float* p2 = pj + 6;
    const float wr = P.wrf;
    auto dot = [](const float* a3, const float* b3) { return a3[0] * b3[0] + a3[1] * b3[1] + a3[2] * b3[2]; };
    const float u0 = wr * (dot(c1, p0) + dot(c0, p1));
    const float u1 = wr * (dot(c2, p0) + dot(c0, p2));
    const float u2 = wr * (dot(c2, p1) + dot(c1, p2));
    const float u3 = 2.f * wr * dot(c0, p0);
    const float u4 = 2.f * wr * dot(c1, p1);
    const float u5 = 2.f * wr * dot(c2, p2);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      acc[i] += wr * (u0 * c1[i] + u1 * c2[i] + 2.f * u3 * c0[i]);
      acc[3 + i] += wr * (u0 * c0[i] + u2 * c2[i] + 2.f * u4 * c1[i]);
      acc[6 + i] += wr * (u1 * c0[i] + u2 * c1[i] + 2.f * u5 * c2[i]);
    }
  }
  }
#pragma unroll
  for (int i = 0; i < 12; ++i) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
  }
}

// Translation part of coarse_prolong_dp (the same expression for v[9..11]).
__device__ __forceinline__ void coarse_prolong_t(const float4 dp, int a, float (&t)[3]) {
  const float d0 = dp.x, d1 = dp.y, d2 = dp.z;
  const float4* c4 = reinterpret_cast<const float4*>(s_zc + 12 * a);
  const float4 ca = c4[0], cb = c4[1], cc = c4[2];
  const float c[12] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w, cc.x, cc.y, cc.z, cc.w};
#pragma unroll
  for (int r = 0; r < 3; ++r) t[r] += c[9 + r] + d0 * c[r] + d1 * c[3 + r] + d2 * c[6 + r];
}

// A staged coupling item in two steps: issue() starts every global load the
// item needs (the other node's u_f and offset, or the group's w_con J_g u_f)
// without using any of them, so that the loads of all items of a round are in
// flight together; finish() adds the coarse parts from shared memory.  The
// result equals fetch_item's.
struct StagedItem {
  CouplingData d;
  float4 dp;     // offset of the other node (ITEM_IN / ITEM_OUT, coarse level on)
  int a;         // its aggregate; for ITEM_CON the list base
  int len;       // ITEM_CON: coarse-list length
};

__device__ __forceinline__ void item_issue(const SolveParams& P, int i, StagedItem& S) {
  const int4 m = stg_item()[i];
  CouplingData& D = S.d;
  D.kind = m.x & 15;
  D.aux = stg_geo()[i];
  S.a = m.x >> 4;
  S.len = 0;
  S.dp = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int q = 0; q < 12; ++q) D.v[q] = 0.f;
  if (D.kind == ITEM_IN) {
    ld12cg(P.z, m.y, D.v);
    if (P.NA) S.dp = __ldcg(P.dpiv + m.y);
  } else if (D.kind == ITEM_OUT) {
    if (m.y >= 0) {
      float t3[3];
      ld3t_cg(P.z, m.y, t3);
      D.v[0] = t3[0];
      D.v[1] = t3[1];
      D.v[2] = t3[2];
      if (P.NA) S.dp = __ldcg(P.dpiv + m.y);
    } else {
      D.kind = ITEM_OUT | 16;  // static neighbour: no vector
    }
  } else if (D.kind == ITEM_CON) {
    if (P.NA) {
      const float4 uz = __ldcg(P.uzg + m.z);
      D.v[0] = uz.x;
      D.v[1] = uz.y;
      D.v[2] = uz.z;
      S.a = m.y;
      S.len = m.w;
    } else {
      float u[3];
      con_ju(P, m.z, u);
      D.v[0] = u[0];
      D.v[1] = u[1];
      D.v[2] = u[2];
    }
  }
}

__device__ __forceinline__ void item_finish(const SolveParams& P, StagedItem& S) {
  CouplingData& D = S.d;
  if (D.kind == (ITEM_OUT | 16)) {
    D.kind = ITEM_OUT;
    return;
  }
  if (!P.NA) return;
  if (D.kind == ITEM_IN) {
    coarse_prolong_dp(S.dp, S.a, D.v);
  } else if (D.kind == ITEM_OUT) {
    float t3[3] = {D.v[0], D.v[1], D.v[2]};
    coarse_prolong_t(S.dp, S.a, t3);
    D.v[0] = t3[0];
    D.v[1] = t3[1];
    D.v[2] = t3[2];
  } else if (D.kind == ITEM_CON) {
    const float wcf = P.wcf;
    for (int f = S.a; f < S.a + S.len; ++f) {
      const float4 V = stg_lv()[f];
      const float4* c4 = reinterpret_cast<const float4*>(s_zc + 12 * stg_la()[f]);
      const float4 ca = c4[0], cb = c4[1], cc = c4[2];
      const float C[12] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w, cc.x, cc.y, cc.z, cc.w};
#pragma unroll
      for (int c = 0; c < 3; ++c)
        D.v[c] = fmaf(wcf, fmaf(V.x, C[c], fmaf(V.y, C[3 + c], fmaf(V.z, C[6 + c], V.w * C[9 + c]))), D.v[c]);
    }
  }
}

// spmv_node for staged slot s (free node r): the same arithmetic in the same
// order, with the node's items, geometry and aggregate offset in shared
// memory.  All global loads of a round (the node's own u_f, x and the other
// nodes' vectors) are issued before any is used, so a product costs one
// round trip to L2 instead of a chain of dependent global loads.  The
// rotation term's x comes from lanes 0..8 of the half.
__device__ __forceinline__ void spmv_node_stg(const SolveParams& P, int s, int r, bool valid, float (&acc)[12],
                                              float (&pj)[12]) {
  const int lane = threadIdx.x & 15;
  const int base = threadIdx.x & 16;
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    acc[i] = 0.f;
    pj[i] = 0.f;
  }
  float xr = 0.f;
  if (valid) {
    const int4 nd = stg_node()[s];
    if (lane < 9) xr = __ldcg(P.xf + 12 * (size_t)r + lane);
    ld12cg(P.z, r, pj);
    bool own = !P.NA;  // own coarse part added
    const float w = P.wgf;
    for (int q = lane; q < nd.z; q += 32) {
      const bool hasB = q + 16 < nd.z;
      StagedItem A, B;
      item_issue(P, nd.y + q, A);
      if (hasB) item_issue(P, nd.y + q + 16, B);
      if (!own) {
        coarse_prolong_dp(stg_dpiv()[s], nd.w, pj);
        own = true;
      }
      item_finish(P, A);
      apply_item(P, A.d, w, pj, acc);
      if (hasB) {
        item_finish(P, B);
        apply_item(P, B.d, w, pj, acc);
      }
    }
    if (!own) coarse_prolong_dp(stg_dpiv()[s], nd.w, pj);
  }
  float X[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) X[i] = __shfl_sync(0xffffffffu, xr, base + i);
  if (valid && lane == 0) {
    // J_rot^T J_rot p with J_rot at the current x (float copy)
    const float* c0 = X;
    const float* c1 = X + 3;
    const float* c2 = X + 6;
    const float* p0 = pj;
    const float* p1 = pj + 3;
    const float* p2 = pj + 6;
    const float wr = P.wrf;
    auto dot = [](const float* a3, const float* b3) { return a3[0] * b3[0] + a3[1] * b3[1] + a3[2] * b3[2]; };
    const float u0 = wr * (dot(c1, p0) + dot(c0, p1));
    const float u1 = wr * (dot(c2, p0) + dot(c0, p2));
    const float u2 = wr * (dot(c2, p1) + dot(c1, p2));
    const float u3 = 2.f * wr * dot(c0, p0);
    const float u4 = 2.f * wr * dot(c1, p1);
    const float u5 = 2.f * wr * dot(c2, p2);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      acc[i] += wr * (u0 * c1[i] + u1 * c2[i] + 2.f * u3 * c0[i]);
      acc[3 + i] += wr * (u0 * c0[i] + u2 * c2[i] + 2.f * u4 * c1[i]);
      acc[6 + i] += wr * (u1 * c0[i] + u2 * c1[i] + 2.f * u5 * c2[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < 12; ++i) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
  }
}

// Diagonal 12x12 block of J^T J for free node r from Q and the rotation rows
// at x (float copy), inverted by Gauss-Jordan without pivoting (the block is
// symmetric positive definite) across 24 lanes: lane j < 12 holds column j of
// the block, lane 12 + j column j of the identity, and every step takes the
// pivot column from its lane by shuffle.  Lanes 12..23 end with the columns of
// the inverse (= its rows) and store them into P.dinv (row-major).  A block
// that is not positive definite falls back to the inverse of its diagonal.
template <bool STG>
__device__ void build_dinv(const SolveParams& P, int r, int slot, const float (&Q)[10]) {
  const int lane = threadIdx.x & 31;
  float X[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) X[i] = __ldcg(P.xf + 12 * (size_t)r + i);
  // rotation rows: [c1|c0|0], [c2|0|c0], [0|c2|c1], [2c0|0|0], [0|2c1|0], [0|0|2c2]
  const float wr = P.wrf;
  float J[6][9];
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b < 9; ++b) J[a][b] = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    J[0][c] = wr * X[3 + c]; J[0][3 + c] = wr * X[c];
    J[1][c] = wr * X[6 + c]; J[1][6 + c] = wr * X[c];
    J[2][3 + c] = wr * X[6 + c]; J[2][6 + c] = wr * X[3 + c];
    J[3][c] = 2.f * wr * X[c];
    J[4][3 + c] = 2.f * wr * X[3 + c];
    J[5][6 + c] = 2.f * wr * X[6 + c];
  }
  // column `lane` (= row, the block is symmetric); unknown u is R[u % 3][u / 3]
  // for u < 9 and t[u - 9] otherwise
  float col[12];
  const int L = lane < 12 ? lane : 0;
  const int aL = L < 9 ? L / 3 : 3, rL = L < 9 ? L % 3 : L - 9;
#pragma unroll
  for (int b = 0; b < 12; ++b) {
    const int ab = b < 9 ? b / 3 : 3, rb = b < 9 ? b % 3 : b - 9;
    float v = 0.f;
    if (rL == rb) {
      const int lo = aL < ab ? aL : ab, hi = aL < ab ? ab : aL;
      float qv = 0.f;
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = x; y < 4; ++y)
          if (x == lo && y == hi) qv = Q[qi(x, y)];
      v = qv;
    }
    if (b < 9 && L < 9) {
      float jj = 0.f;
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        float jl = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) jl = (q == L) ? J[t][q] : jl;
        jj = fmaf(jl, J[t][b], jj);
      }
      v += jj;
    }
    col[b] = lane < 12 ? v : ((lane == 12 + b) ? 1.f : 0.f);
  }
  float dg = 0.f;  // this lane's diagonal entry, for the fallback
#pragma unroll
  for (int b = 0; b < 12; ++b)
    if (b == L) dg = col[b];
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    float ck[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) ck[i] = __shfl_sync(0xffffffffu, col[i], k);
    const float piv = ck[k];
    ok = ok && piv > 0.f;
    const float akj = col[k] / piv;
#pragma unroll
    for (int i = 0; i < 12; ++i)
      if (i != k) col[i] = fmaf(-ck[i], akj, col[i]);
    col[k] = akj;
  }
  const float dgj = __shfl_sync(0xffffffffu, dg, lane >= 12 && lane < 24 ? lane - 12 : 0);
  if (lane >= 12 && lane < 24) {
    const int j = lane - 12;
    float* out;
    if constexpr (STG)
      out = stg_dinv(slot) + 12 * j;
    else
      out = P.dinv + 144 * (size_t)r + 12 * j;
#pragma unroll
    for (int i = 0; i < 12; ++i) out[i] = ok ? col[i] : ((i == j) ? 1.f / fmaxf(dgj, 1e-20f) : 0.f);
  }
  __syncwarp();
}

// Half-warp form: lane c < 12 of each 16-lane half holds r_c of its node rr.
__device__ __forceinline__ float apply_dinv_h(const SolveParams& P, int rr, bool valid, float rc) {
  const int lane = threadIdx.x & 31;
  const int l16 = lane & 15, base = lane & 16;
  float zc = 0.f;
  const float* row = P.dinv + 144 * (size_t)(valid ? rr : 0) + 12 * (l16 < 12 ? l16 : 0);
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const float ri = __shfl_sync(0xffffffffu, rc, base + i);
    if (valid) zc = fmaf(__ldcg(row + i), ri, zc);
  }
  return (valid && l16 < 12) ? zc : 0.f;
}

// apply_dinv_h with the inverse block of staged slot s (three accumulators,
// the row read as float4s).
__device__ __forceinline__ float apply_dinv_h_stg(int s, bool valid, float rc) {
  const int lane = threadIdx.x & 31;
  const int l16 = lane & 15, base = lane & 16;
  const float4* row = reinterpret_cast<const float4*>(stg_dinv(valid ? s : 0) + 12 * (l16 < 12 ? l16 : 0));
  float ri[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) ri[i] = __shfl_sync(0xffffffffu, rc, base + i);
  float z[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const float4 d = row[q];
    z[q] = fmaf(d.x, ri[4 * q], fmaf(d.y, ri[4 * q + 1], fmaf(d.z, ri[4 * q + 2], d.w * ri[4 * q + 3])));
  }
  return (valid && l16 < 12) ? (z[0] + z[1]) + z[2] : 0.f;
}

// z = Dinv r for free node rr (staged: slot's inverse block in shared
// memory); lane c < 12 holds r_c and returns z_c.
template <bool STG>
__device__ __forceinline__ float apply_dinv(const SolveParams& P, int rr, int slot, float rc) {
  const int lane = threadIdx.x & 31;
  float zc = 0.f;
  const int L = lane < 12 ? lane : 0;
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const float ri = __shfl_sync(0xffffffffu, rc, i);
    float d;
    if constexpr (STG)
      d = stg_dinv(slot)[12 * L + i];
    else
      d = __ldcg(P.dinv + 144 * (size_t)rr + 12 * L + i);
    zc = fmaf(d, ri, zc);
  }
  return lane < 12 ? zc : 0.f;
}


// ------------------------------------------------------ coarse level ----
// 4x4 kernel index: unknowns (R[r][0], R[r][1], R[r][2], t[r]) of one row r;
// coarse unknown u of an aggregate is R col-major (3c + r) for u < 9, t[u-9].
__device__ __forceinline__ void coarse_add(const SolveParams& P, int a, int b, const float (&va)[4],
                                           const float (&vb)[4]) {
  double* q = P.Qd + ((size_t)a * P.NA + b) * 16;
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) atomicAdd(q + 4 * x + y, (double)va[x] * (double)vb[y]);
}

// Coefficients of one regularisation / static / constraint row (all three r
// share them) on the coarse unknowns of aggregate a: a J-row with R-part w_R
// (per column c) and t-part w_t on node j maps to (w_R + w_t d_j, w_t).
__device__ __forceinline__ void coarse_vec(const SolveParams& P, int rr, int node, float wr0, float wr1,
                                           float wr2, float wt, float (&v)[4]) {
  const int a = __ldg(P.agg + rr);
  const int pv = __ldg(P.pivot + a);
  v[0] = wr0 + wt * (__ldg(P.node_pos + 3 * (size_t)node) - __ldg(P.node_pos + 3 * (size_t)pv));
  v[1] = wr1 + wt * (__ldg(P.node_pos + 3 * (size_t)node + 1) - __ldg(P.node_pos + 3 * (size_t)pv + 1));
  v[2] = wr2 + wt * (__ldg(P.node_pos + 3 * (size_t)node + 2) - __ldg(P.node_pos + 3 * (size_t)pv + 2));
  v[3] = wt;
}

// Coarse matrix kernels of the rows owned by free node r (its outgoing
// regularisation rows and the static rows pointing at it).
__device__ void coarse_rows_node(const SolveParams& P, int r) {
  const int lane = threadIdx.x & 31;
  const int j = __ldg(P.free_ids + r);
  const int a = __ldg(P.agg + r);
  const float w = P.wgf;
  const float gj[3] = {__ldg(P.node_pos + 3 * (size_t)j), __ldg(P.node_pos + 3 * (size_t)j + 1),
                       __ldg(P.node_pos + 3 * (size_t)j + 2)};
  const int b0 = __ldg(P.item_off + r), b1 = __ldg(P.item_off + r + 1);
  for (int it = b0 + lane; it < b1; it += 32) {
    const int4 m = __ldg(P.items + it);
    if ((m.x & 15) == ITEM_OUT) {
      const float ws = w * __int_as_float(m.w);
      const float d[3] = {__ldg(P.node_pos + 3 * (size_t)m.z) - gj[0], __ldg(P.node_pos + 3 * (size_t)m.z + 1) - gj[1],
                          __ldg(P.node_pos + 3 * (size_t)m.z + 2) - gj[2]};
      float va[4], vb[4];
      coarse_vec(P, r, j, ws * d[0], ws * d[1], ws * d[2], w, va);
      if (m.y >= 0) {
        coarse_vec(P, m.y, m.z, 0.f, 0.f, 0.f, -ws, vb);
        const int b = __ldg(P.agg + m.y);
        if (b == a) {
          float v[4] = {va[0] + vb[0], va[1] + vb[1], va[2] + vb[2], va[3] + vb[3]};
          coarse_add(P, a, a, v, v);
        } else {
          coarse_add(P, a, a, va, va);
          coarse_add(P, a, b, va, vb);
          coarse_add(P, b, a, vb, va);
          coarse_add(P, b, b, vb, vb);
        }
      } else {
        coarse_add(P, a, a, va, va);
      }
    } else if ((m.x & 15) == ITEM_STATIC) {
      float v[4];
      coarse_vec(P, r, j, 0.f, 0.f, 0.f, -w, v);
      coarse_add(P, a, a, v, v);
    }
  }
}

// Coarse kernels of constraint group g (one thread): J_g restricted to the
// aggregates its free anchors belong to, then every pair.
__device__ void coarse_rows_group(const SolveParams& P, int g) {
  constexpr int kMaxAgg = 24;
  int ids[kMaxAgg];
  float vv[kMaxAgg][4];
  int na = 0;
  const float wc = P.wcf;
  const int s0 = __ldg(P.grp_off + g), s1 = __ldg(P.grp_off + g + 1);
  for (int s = s0; s < s1; ++s) {
    const int c = __ldg(P.grp_member + s);
    for (int t = 0; t < P.k; ++t) {
      const int slot = s * P.k + t;
      const int rk = __ldg(P.mem_rank + slot);
      if (rk < 0) continue;
      const int b = __ldg(P.agg + rk);
      const int pv = __ldg(P.pivot + b);
      const float a = wc * __ldg(P.mem_w + slot);
      // R-part a (v_c - g_l) plus t-part a (g_l - g_pivot) = a (v_c - g_pivot)
      float v[4];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float dv = __ldg(P.node_pos + 3 * (size_t)c + q) - __ldg(P.node_pos + 3 * (size_t)__ldg(P.mem_node + slot) + q);
        const float dl = __ldg(P.node_pos + 3 * (size_t)__ldg(P.mem_node + slot) + q) - __ldg(P.node_pos + 3 * (size_t)pv + q);
        v[q] = a * (dv + dl);
      }
      v[3] = a;
      int f = -1;
      for (int q = 0; q < na; ++q)
        if (ids[q] == b) f = q;
      if (f < 0) {
        if (na == kMaxAgg) {
          raise_status(&P.bar->status, ARAP_EUNSUPPORTED);
          continue;
        }
        f = na++;
        ids[f] = b;
        vv[f][0] = vv[f][1] = vv[f][2] = vv[f][3] = 0.f;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) vv[f][q] += v[q];
    }
  }
  for (int x = 0; x < na; ++x)
    for (int y = 0; y < na; ++y) {
      float vx[4] = {vv[x][0], vv[x][1], vv[x][2], vv[x][3]};
      float vy[4] = {vv[y][0], vv[y][1], vv[y][2], vv[y][3]};
      coarse_add(P, ids[x], ids[y], vx, vy);
    }
}

// J_rot^T J_rot (9x9) of free node rr at the current x (float copy), added to
// its aggregate's sum (all lanes of the warp call it).
__device__ __forceinline__ void coarse_rot_node(const SolveParams& P, int rr, double* rotagg) {
  const int lane = threadIdx.x & 31;
  float X[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) X[i] = __ldcg(P.xf + 12 * (size_t)rr + i);
  const float wr = P.wrf;
  float J[6][9];
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b < 9; ++b) J[a][b] = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    J[0][c] = wr * X[3 + c]; J[0][3 + c] = wr * X[c];
    J[1][c] = wr * X[6 + c]; J[1][6 + c] = wr * X[c];
    J[2][3 + c] = wr * X[6 + c]; J[2][6 + c] = wr * X[3 + c];
    J[3][c] = 2.f * wr * X[c];
    J[4][3 + c] = 2.f * wr * X[3 + c];
    J[5][6 + c] = 2.f * wr * X[6 + c];
  }
  double* dst = rotagg + 81 * (size_t)__ldg(P.agg + rr);
  for (int e = lane; e < 81; e += 32) {
    const int a = e / 9, b = e % 9;
    float v = 0.f;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      // select J[t][a] * J[t][b] without dynamic register indexing
      float ja = 0.f, jb = 0.f;
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        ja = (q == a) ? J[t][q] : ja;
        jb = (q == b) ? J[t][q] : jb;
      }
      v = fmaf(ja, jb, v);
    }
    atomicAdd(dst + e, (double)v);
  }
}

// Dense coarse matrix entry (I, J): the 4x4 kernels expanded over the three
// rows r, plus the aggregate's sum of orthogonality blocks at the current x.
__device__ __forceinline__ float coarse_entry_x(const SolveParams& P, const double* rotagg, int I, int J) {
  const int a = I / 12, iI = I % 12, b = J / 12, iJ = J % 12;
  const int rI = iI < 9 ? iI % 3 : iI - 9, pI = iI < 9 ? iI / 3 : 3;
  const int rJ = iJ < 9 ? iJ % 3 : iJ - 9, pJ = iJ < 9 ? iJ / 3 : 3;
  double v = (rI == rJ) ? P.Qd[((size_t)a * P.NA + b) * 16 + 4 * pI + pJ] : 0.0;
  if (a == b && iI < 9 && iJ < 9) v += __ldcg(rotagg + 81 * (size_t)a + 9 * iI + iJ);
  return (float)v;
}

// Half-warp form of coarse_restrict.
__device__ __forceinline__ void coarse_restrict_h(const SolveParams& P, int rr, bool valid, float rc_lane,
                                                  double* rc) {
  const int lane = threadIdx.x & 31;
  const int l16 = lane & 15, base = lane & 16;
  const int c = l16 < 9 ? l16 / 3 : 0, r = l16 < 9 ? l16 % 3 : 0;
  const float rt = __shfl_sync(0xffffffffu, rc_lane, base + 9 + r);
  if (valid && l16 < 12) {
    const int a = __ldg(P.agg + rr);
    float v = rc_lane;
    if (l16 < 9) {
      const float4 dp = __ldcg(P.dpiv + rr);
      v += (c == 0 ? dp.x : (c == 1 ? dp.y : dp.z)) * rt;
    }
    atomicAdd(rc + 12 * a + l16, (double)v);
  }
}

// coarse_restrict_h of staged slot s (aggregate and offset from shared memory).
__device__ __forceinline__ void coarse_restrict_h_stg(int s, bool valid, float rc_lane, double* rc) {
  const int lane = threadIdx.x & 31;
  const int l16 = lane & 15, base = lane & 16;
  const int c = l16 < 9 ? l16 / 3 : 0, r = l16 < 9 ? l16 % 3 : 0;
  const float rt = __shfl_sync(0xffffffffu, rc_lane, base + 9 + r);
  if (valid && l16 < 12) {
    const int a = stg_node()[s].w;
    float v = rc_lane;
    if (l16 < 9) {
      const float4 dp = stg_dpiv()[s];
      v += (c == 0 ? dp.x : (c == 1 ? dp.y : dp.z)) * rt;
    }
    atomicAdd(rc + 12 * a + l16, (double)v);
  }
}

// Restriction of free node rr's residual (lane c < 12 holds r_c) into rc:
// (P_j^T r_j)_{3c+r} = r_{3c+r} + d_c r_{9+r}, (P_j^T r_j)_{9+r} = r_{9+r}.
__device__ __forceinline__ void coarse_restrict(const SolveParams& P, int rr, float rc_lane, double* rc) {
  const int lane = threadIdx.x & 31;
  const int a = __ldg(P.agg + rr);
  const int node = __ldg(P.free_ids + rr);
  const int pv = __ldg(P.pivot + a);
  const int c = lane < 9 ? lane / 3 : 0, r = lane < 9 ? lane % 3 : 0;
  const float rt = __shfl_sync(0xffffffffu, rc_lane, 9 + r);
  if (lane < 12) {
    float v = rc_lane;
    if (lane < 9) v += (__ldg(P.node_pos + 3 * (size_t)node + c) - __ldg(P.node_pos + 3 * (size_t)pv + c)) * rt;
    atomicAdd(rc + 12 * a + lane, (double)v);
  }
}

// ---------------------------------------------------- resident PCG ----
// With every node of a CTA resident, the CTA's nodes keep their PCG vectors
// in shared memory, and A P zc of a node comes from its coarse blocks: per
// aggregate coupled to it, the 12x12 block of (J^T J)_{reg,static,con} P
// restricted to that aggregate (built once per solve), plus its rotation
// block on P_j zc.  The products of fine vectors (A z1, A z3 of the V-cycle
// below) read the neighbours' vectors from L2.

// P_k e_i: the prolongation of coarse unknown i of node k's own aggregate
// (coarse_prolong_dp with zc = e_i): identity on the rotation part, and
// dt = e_t + dR dp on the translation part.
__device__ __forceinline__ void prolong_unit(const float4 dp, int i, float (&v)[12]) {
#pragma unroll
  for (int q = 0; q < 9; ++q) v[q] = q == i ? 1.f : 0.f;
#pragma unroll
  for (int r = 0; r < 3; ++r)
    v[9 + r] = (9 + r == i ? 1.f : 0.f) + (i == r ? dp.x : 0.f) + (i == 3 + r ? dp.y : 0.f) + (i == 6 + r ? dp.z : 0.f);
}

// Coarse blocks of resident slot s (one warp): the aggregates a coupled to the
// node (its own, its regularisation neighbours', its constraint groups') and,
// for each, M_a = the node's rows of (J^T J)_{reg,static,con} P restricted to
// aggregate a, column by column: column i is the product with zc = e_i on a
// (apply_item over the node's items, the constraint items with their coarse
// parts V_ga only).  Stored row-major so that lane c reads row c.
static __device__ __noinline__ void build_coarse_blocks(const SolveParams& P, int s) {
  const int lane = threadIdx.x & 31;
  const int4 nd = stg_node()[s];
  const int4 bs = stg_base()[s];
  const int na = bs.z >> 16, mb = bs.w;
  int cnt = 0;
  if (lane == 0) {
    auto add = [&](int a) {
      for (int t = 0; t < cnt; ++t)
        if (stg_mag()[mb + t] == a) return;
      if (cnt < na) stg_mag()[mb + cnt++] = a;
    };
    add(nd.w);
    for (int q = 0; q < nd.z; ++q) {
      const int4 m = stg_item()[nd.y + q];
      const int kind = m.x & 15;
      if ((kind == ITEM_IN || kind == ITEM_OUT) && m.y >= 0) add(m.x >> 4);
      if (kind == ITEM_CON)
        for (int f = m.y; f < m.y + m.w; ++f) add(stg_la()[f]);
    }
    // (the host counts the same set; any spare entry gets a zero block)
    for (int t = cnt; t < na; ++t) stg_mag()[mb + t] = nd.w;
  }
  cnt = __shfl_sync(0xffffffffu, cnt, 0);
  __syncwarp();
  const float4 dpj = stg_dpiv()[s];
  const float w = P.wgf, wcf = P.wcf;
  for (int t = 0; t < na; ++t) {
    const int a = t < cnt ? stg_mag()[mb + t] : -1;
    for (int i = 0; i < 12; ++i) {
      float acc[12], yj[12];
#pragma unroll
      for (int q = 0; q < 12; ++q) acc[q] = 0.f;
      if (a == nd.w) {
        prolong_unit(dpj, i, yj);
      } else {
#pragma unroll
        for (int q = 0; q < 12; ++q) yj[q] = 0.f;
      }
      for (int q = lane; q < nd.z; q += 32) {
        const int it = nd.y + q;
        const int4 m = stg_item()[it];
        CouplingData D;
        D.kind = m.x & 15;
        D.aux = stg_geo()[it];
#pragma unroll
        for (int c = 0; c < 12; ++c) D.v[c] = 0.f;
        if ((D.kind == ITEM_IN || D.kind == ITEM_OUT) && m.y >= 0 && (m.x >> 4) == a) {
          float v[12];
          prolong_unit(stg_ydp()[it], i, v);
          if (D.kind == ITEM_IN) {
#pragma unroll
            for (int c = 0; c < 12; ++c) D.v[c] = v[c];
          } else {
            D.v[0] = v[9];
            D.v[1] = v[10];
            D.v[2] = v[11];
          }
        } else if (D.kind == ITEM_CON) {
          for (int f = m.y; f < m.y + m.w; ++f) {
            if (stg_la()[f] != a) continue;
            const float4 V = stg_lv()[f];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float vc = i == c ? V.x : (i == 3 + c ? V.y : (i == 6 + c ? V.z : (i == 9 + c ? V.w : 0.f)));
              D.v[c] = fmaf(wcf, vc, D.v[c]);
            }
          }
        }
        apply_item(P, D, w, yj, acc);
      }
#pragma unroll
      for (int c = 0; c < 12; ++c) acc[c] = warp_sum(acc[c]);
      if (lane < 12) {
        float v = 0.f;
#pragma unroll
        for (int c = 0; c < 12; ++c)
          if (c == lane) v = acc[c];
        stg_mm(mb + t)[12 * lane + i] = v;
      }
    }
  }
  __syncwarp();
}

// The rotation block J_rot^T J_rot (9x9) of resident slot s at the staged x
// (one warp; lane c < 9 writes row c, padded to 12).
__device__ __forceinline__ void rot_block(const SolveParams& P, int s) {
  const int lane = threadIdx.x & 31;
  if (lane >= 9) return;
  const float* X = stg_xf(s);
  const float wr = P.wrf;
  // rows of J_rot (Deform.cpp:186-214 as products): [c1|c0|0], [c2|0|c0],
  // [0|c2|c1], 2[c0|0|0], 2[0|c1|0], 2[0|0|c2]
  auto jrow = [&](int t, int b) -> float {
    const int blk = b / 3, e = b % 3;
    switch (t) {
      case 0: return blk == 0 ? wr * X[3 + e] : (blk == 1 ? wr * X[e] : 0.f);
      case 1: return blk == 0 ? wr * X[6 + e] : (blk == 2 ? wr * X[e] : 0.f);
      case 2: return blk == 1 ? wr * X[6 + e] : (blk == 2 ? wr * X[3 + e] : 0.f);
      case 3: return blk == 0 ? 2.f * wr * X[e] : 0.f;
      case 4: return blk == 1 ? 2.f * wr * X[3 + e] : 0.f;
      default: return blk == 2 ? 2.f * wr * X[6 + e] : 0.f;
    }
  };
  float* row = stg_rot(s) + 12 * lane;
  for (int b = 0; b < 9; ++b) {
    float v = 0.f;
    for (int t = 0; t < 6; ++t) v = fmaf(jrow(t, lane), jrow(t, b), v);
    row[b] = v;
  }
  row[9] = row[10] = row[11] = 0.f;
}

// ------------------------------------------- V-cycle preconditioner ----
// The resident two-level PCG applies the symmetric two-grid cycle
//   z1 = D^-1 r,  zc = C^-1 P^T (r - A z1),  z2 = z1 + P zc,
//   u = z2 + D^-1 (r - A z2),  w = A u = A z2 + A z3 (z3 = D^-1 (r - A z2))
// with the block-Jacobi smoother D before and after the coarse correction.
// It needs about half the iterations of the additive form D^-1 + P C^-1 P^T
// on these problems, for two more barriers per iteration.  A z1 and A z3 take
// the neighbours' vectors from L2; A P zc comes from the coarse blocks.

// Rotation block of slot s applied to the first nine entries of v (lane c < 9).
__device__ __forceinline__ float rot_apply(int s, int c, const float (&v)[12]) {
  const float4* R4 = reinterpret_cast<const float4*>(stg_rot(s) + 12 * c);
  const float4 ra = R4[0], rb = R4[1], rc = R4[2];
  const float R[9] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w, rc.x};
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a0 = fmaf(R[i], v[i], a0);
    a1 = fmaf(R[3 + i], v[3 + i], a1);
    a2 = fmaf(R[6 + i], v[6 + i], a2);
  }
  return (a0 + a1) + a2;
}

// Constraint rows of slot s on the staged w_con J_g v of its constraint
// items (apply_item's ITEM_CON; the node's constraint items are its last ncon
// items and consecutive in the CTA's constraint list); entry c.
__device__ __forceinline__ float con_apply(const SolveParams& P, const int4& nd, const int4& bs, int c) {
  const int ncon = bs.z & 0xffff;
  const int g3 = c / 3, cc = c - 3 * g3;
  const int c0 = nd.y + nd.z - ncon;
  float v = 0.f;
  for (int q = 0; q < ncon; ++q) {
    const float4 ax = stg_geo()[c0 + q];
    const float4 uz = stg_cuz()[bs.y + q];
    const float wa = P.wcf * ax.x;
    const float coef = g3 == 0 ? ax.y : (g3 == 1 ? ax.z : (g3 == 2 ? ax.w : 1.f));
    const float uzc = cc == 0 ? uz.x : (cc == 1 ? uz.y : uz.z);
    v = fmaf(wa * coef, uzc, v);
  }
  return v;
}

__device__ __forceinline__ void ld12s(const float* p, float (&v)[12]) {
  const float4* p4 = reinterpret_cast<const float4*>(p);
  const float4 a = p4[0], b = p4[1], c = p4[2];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
  v[6] = b.z; v[7] = b.w; v[8] = c.x; v[9] = c.y; v[10] = c.z; v[11] = c.w;
}

// (J^T J)_{reg,static} v of resident slot s (regularisation and static-node
// items; the node's own v is slot vector k, the neighbours' v come from P.z),
// reduced over the half-warp: every lane of the half holds the 12 entries.
__device__ __forceinline__ void reg_product(const SolveParams& P, int s, bool valid, int k, float (&acc)[12]) {
  const int lane = threadIdx.x & 15;
  float pj[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    acc[i] = 0.f;
    pj[i] = 0.f;
  }
  if (valid) {
    const int4 nd = stg_node()[s];
    ld12s(stg_vec(s, k), pj);
    const float w = P.wgf;
    for (int q = lane; q < nd.z; q += 32) {
      const bool hasB = q + 16 < nd.z;
      CouplingData A, B;
      auto fetch = [&](int i, CouplingData& D) {
        const int4 m = stg_item()[i];
        D.kind = m.x & 15;
        D.aux = stg_geo()[i];
#pragma unroll
        for (int t = 0; t < 12; ++t) D.v[t] = 0.f;
        if (D.kind == ITEM_IN) {
          ld12cg(P.z, m.y, D.v);
        } else if (D.kind == ITEM_OUT && m.y >= 0) {
          float t3[3];
          ld3t_cg(P.z, m.y, t3);
          D.v[0] = t3[0];
          D.v[1] = t3[1];
          D.v[2] = t3[2];
        }
      };
      fetch(nd.y + q, A);
      if (hasB) fetch(nd.y + q + 16, B);
      if (A.kind != ITEM_CON) apply_item(P, A, w, pj, acc);
      if (hasB && B.kind != ITEM_CON) apply_item(P, B, w, pj, acc);
    }
  }
#pragma unroll
  for (int i = 0; i < 12; ++i) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
  }
}

__device__ __forceinline__ float pick12(const float (&v)[12], int c) {
  float x = 0.f;
#pragma unroll
  for (int i = 0; i < 12; ++i)
    if (i == c) x = v[i];
  return x;
}

// w_con J_g v of constraint item ci of the CTA, in two steps so that its
// global loads overlap the node products: group_issue loads the anchor row of
// slot q8 of the group's member-anchor slots (eight lanes per item),
// group_finish adds the remaining slots, reduces over the eight lanes and
// stores the staged value.
struct GroupLoad {
  float v[12];
  float4 geo;
  bool has;
};
__device__ __forceinline__ void group_issue(const SolveParams& P, int ci, bool valid, GroupLoad& G) {
  const int q8 = threadIdx.x & 7;
  G.has = false;
  G.geo = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 12; ++i) G.v[i] = 0.f;
  if (!valid) return;
  const int2 sr = stg_cgs()[ci];
  if (q8 >= sr.y) return;
  const int rk = stg_gsr()[sr.x + q8];
  if (rk < 0) return;
  G.geo = stg_gsg()[sr.x + q8];
  ld12cg(P.z, rk, G.v);
  G.has = true;
}
__device__ __forceinline__ void group_finish(const SolveParams& P, int ci, bool valid, const GroupLoad& G) {
  const int q8 = threadIdx.x & 7;
  const unsigned mask = 0xffu << (threadIdx.x & 24);
  float u[3] = {0.f, 0.f, 0.f};
  auto add = [&](const float4 geo, const float (&zl)[12]) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      u[c] = fmaf(geo.x, fmaf(geo.y, zl[c], fmaf(geo.z, zl[3 + c], fmaf(geo.w, zl[6 + c], zl[9 + c]))), u[c]);
  };
  if (G.has) add(G.geo, G.v);
  if (valid) {
    const int2 sr = stg_cgs()[ci];
    for (int e = q8 + 8; e < sr.y; e += 8) {
      const int rk = stg_gsr()[sr.x + e];
      if (rk < 0) continue;
      float zl[12];
      ld12cg(P.z, rk, zl);
      add(stg_gsg()[sr.x + e], zl);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) u[c] += __shfl_xor_sync(mask, u[c], o);
  }
  if (valid && q8 == 0) stg_cuz()[ci] = make_float4(P.wcf * u[0], P.wcf * u[1], P.wcf * u[2], 0.f);
}

// (J^T J)_{reg,static} v of resident slot s into slot vector RV_W (the
// constraint and rotation rows are added by full_product_finish).
static __device__ __noinline__ void reg_product_store(const SolveParams& P, int s, bool valid, int k) {
  const int c = threadIdx.x & 15;
  float acc[12];
  reg_product(P, s, valid, k, acc);
  if (valid && c < 12) stg_vec(s, RV_W)[c] = pick12(acc, c);
}

// Entry c of the full (J^T J) v of resident slot s: the stored
// regularisation part, the constraint rows on the staged w_con J_g v, the
// rotation block on v (slot vector k).
__device__ __forceinline__ float full_product_finish(const SolveParams& P, int s, int k, int c) {
  const int4 nd = stg_node()[s];
  const int4 bs = stg_base()[s];
  float v[12];
  ld12s(stg_vec(s, k), v);
  float a = stg_vec(s, RV_W)[c] + con_apply(P, nd, bs, c);
  if (c < 9) a += rot_apply(s, c, v);
  return a;
}

// Phase 1: p = u + beta p, s = w + beta s, h += alpha p, r -= alpha s,
// z1 = D^-1 r for resident slot s; z1 and h also to global memory.
static __device__ __noinline__ void vc_update(const SolveParams& P, int s, bool valid, float alpha, float beta,
                                              bool first) {
  const int l16 = threadIdx.x & 15;
  const bool own = valid && l16 < 12;
  float rv = 0.f, hv = 0.f;
  int r = 0;
  if (own) {
    r = stg_node()[s].x;
    const float uo = stg_vec(s, RV_U)[l16], wo = stg_vec(s, RV_W)[l16];
    const float pn = first ? uo : fmaf(beta, stg_vec(s, RV_P)[l16], uo);
    const float sn = first ? wo : fmaf(beta, stg_vec(s, RV_S)[l16], wo);
    stg_vec(s, RV_P)[l16] = pn;
    stg_vec(s, RV_S)[l16] = sn;
    hv = fmaf(alpha, pn, stg_vec(s, RV_H)[l16]);
    stg_vec(s, RV_H)[l16] = hv;
    rv = fmaf(-alpha, sn, stg_vec(s, RV_R)[l16]);
    stg_vec(s, RV_R)[l16] = rv;
  }
  const float zv = apply_dinv_h_stg(s, valid, rv);
  if (own) {
    stg_vec(s, RV_UF)[l16] = zv;
    P.z[12 * (size_t)r + l16] = zv;
    P.h[12 * (size_t)r + l16] = hv;
  }
}

// Phase 2, after the products: a1 = (J^T J) z1 of resident slot s (kept in
// RV_WF) and the restriction of r - a1 into rc (of r in the additive form,
// vc = false).
static __device__ __noinline__ void vc_restrict(const SolveParams& P, int s, bool valid, double* rc, bool vc) {
  const int c = threadIdx.x & 15;
  float t = 0.f;
  if (valid && c < 12) {
    const float a1 = full_product_finish(P, s, RV_UF, c);
    stg_vec(s, RV_WF)[c] = a1;
    t = stg_vec(s, RV_R)[c] - (vc ? a1 : 0.f);
  }
  coarse_restrict_h_stg(s, valid, t, rc);
}

// Restart of the resident PCG (after a V-cycle breakdown): r from the
// gradient pass (P.r), h = 0, z1 = D^-1 r, for resident slot s.
static __device__ __noinline__ void vc_restart(const SolveParams& P, int s, bool valid) {
  const int c = threadIdx.x & 15;
  const bool own = valid && c < 12;
  float rv = 0.f;
  int r = 0;
  if (own) {
    r = stg_node()[s].x;
    rv = __ldcg(P.r + 12 * (size_t)r + c);
    stg_vec(s, RV_R)[c] = rv;
    stg_vec(s, RV_H)[c] = 0.f;
  }
  const float zv = apply_dinv_h_stg(s, valid, rv);
  if (own) {
    stg_vec(s, RV_UF)[c] = zv;
    P.z[12 * (size_t)r + c] = zv;
    P.h[12 * (size_t)r + c] = 0.f;
  }
}

// Phase 4: z2 = z1 + P zc, A z2 = a1 + A P zc (coarse blocks, rotation block
// on P_j zc), z3 = D^-1 (r - A z2), u = z2 + z3 for resident slot s.  Keeps
// u, A z2 (RV_WF) and z3 (RV_UF, also to P.z for the neighbours).  The zc
// entries must be staged.
static __device__ __noinline__ void vc_precond(const SolveParams& P, int s, bool valid, bool vc) {
  const int c = threadIdx.x & 15;
  float t = 0.f, z2 = 0.f, az2 = 0.f;
  int r = 0;
  if (valid && c < 12) {
    const int4 nd = stg_node()[s];
    const int4 bs = stg_base()[s];
    const int na = bs.z >> 16;
    r = nd.x;
    float wq[3] = {0.f, 0.f, 0.f};
#pragma unroll 4
    for (int e = 0; e < na; ++e) {
      const float4* m4 = reinterpret_cast<const float4*>(stg_mm(bs.w + e) + 12 * c);
      const float4* z4 = reinterpret_cast<const float4*>(stg_zz(bs.w + e));
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float4 mq = m4[q], zq = z4[q];
        wq[q] = fmaf(mq.x, zq.x, fmaf(mq.y, zq.y, fmaf(mq.z, zq.z, fmaf(mq.w, zq.w, wq[q]))));
      }
    }
    float zj[12];
    ld12s(stg_zz(bs.w), zj);  // the node's own aggregate is its first entry
    float pz;
    if (c < 9) {
      pz = pick12(zj, c);
    } else {
      const float4 dp = stg_dpiv()[s];
      const int rr = c - 9;
      pz = pick12(zj, 9 + rr) + dp.x * pick12(zj, rr) + dp.y * pick12(zj, 3 + rr) + dp.z * pick12(zj, 6 + rr);
    }
    float apz = (wq[0] + wq[1]) + wq[2];
    if (c < 9) apz += rot_apply(s, c, zj);
    z2 = stg_vec(s, RV_UF)[c] + pz;
    az2 = stg_vec(s, RV_WF)[c] + apz;
    t = vc ? stg_vec(s, RV_R)[c] - az2 : 0.f;
  }
  const float z3 = apply_dinv_h_stg(s, valid, t);
  if (valid && c < 12) {
    stg_vec(s, RV_U)[c] = z2 + z3;
    stg_vec(s, RV_WF)[c] = az2;
    stg_vec(s, RV_UF)[c] = z3;
    P.z[12 * (size_t)r + c] = z3;
  }
}

// The additive form's last step (no post-smoothing, z3 = 0): w = A z2 for
// resident slot s; adds r.u, w.u and r.r into f3.
static __device__ __noinline__ void vc_finish_additive(const SolveParams& P, int s, bool valid, float (&f3)[3]) {
  const int c = threadIdx.x & 15;
  if (!valid || c >= 12) return;
  const float wv = stg_vec(s, RV_WF)[c];
  const float uc = stg_vec(s, RV_U)[c];
  const float rv = stg_vec(s, RV_R)[c];
  stg_vec(s, RV_W)[c] = wv;
  f3[0] = fmaf(rv, uc, f3[0]);
  f3[1] = fmaf(wv, uc, f3[1]);
  f3[2] = fmaf(rv, rv, f3[2]);
}

// Phase 5, after the products: w = A z2 + A z3 for resident slot s; adds
// r.u, w.u and r.r into f3.
static __device__ __noinline__ void vc_finish(const SolveParams& P, int s, bool valid, float (&f3)[3]) {
  const int c = threadIdx.x & 15;
  if (!valid || c >= 12) return;
  const float wv = stg_vec(s, RV_WF)[c] + full_product_finish(P, s, RV_UF, c);
  const float uc = stg_vec(s, RV_U)[c];
  const float rv = stg_vec(s, RV_R)[c];
  stg_vec(s, RV_W)[c] = wv;
  f3[0] = fmaf(rv, uc, f3[0]);
  f3[1] = fmaf(wv, uc, f3[1]);
  f3[2] = fmaf(rv, rv, f3[2]);
}

// zc for the CTA's rows of the coarse inverse (resident mode): row j of the
// CTA is row bid + j nbk, held in shared memory; rc (float) in s_rc.
__device__ __forceinline__ void coarse_rows_res(const SolveParams& P, int bid, int nbk, int ok, const float* s_rc) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int NC = P.NC, n4 = NC / 4;
  const float4* s4 = reinterpret_cast<const float4*>(s_rc);
  for (int j = wib; j < s_stg.nrows; j += kSolveWarps) {
    const float4* row = reinterpret_cast<const float4*>(stg_crow(j, NC));
    float a0 = 0.f, a1 = 0.f;
    for (int q = lane; q < n4; q += 32) {
      const float4 v = row[q], r4 = s4[q];
      a0 = fmaf(v.x, r4.x, fmaf(v.y, r4.y, a0));
      a1 = fmaf(v.z, r4.z, fmaf(v.w, r4.w, a1));
    }
    const float a = warp_sum(a0 + a1);
    if (lane == 0) P.zc[bid + j * nbk] = ok ? a : 0.f;
  }
}

// Shared-memory bytes of one node's tables (host and device use the same sum).
__host__ __device__ __forceinline__ int stage_node_bytes(int items, int lists, int cons, int aggs, int slots,
                                                         bool resident) {
  int b = kStageNodeBytes + kStageItemBytes * items + kStageListBytes * lists;
  if (resident)
    b += kResNodeBytes + kResItemBytes * items + kResConBytes * cons + kResAggBytes * aggs + kResSlotBytes * slots;
  return b;
}

// Coarse-inverse rows CTA bid of nbk holds in resident mode (rows bid, bid + nbk, ...).
__host__ __device__ __forceinline__ int stage_coarse_rows(int NC, int bid, int nbk) {
  return bid < NC ? (NC - bid + nbk - 1) / nbk : 0;
}

// Fills the CTA's resident node tables for this solve (after the per-solve
// geometry: member offsets, aggregate offsets and V_ga).  Warp 0 finds how
// many of the CTA's nodes fit in stage_cap bytes and lays the regions out;
// then one warp per staged node copies its items with their geometry and
// coarse lists.  Nothing is staged in gradient-only mode.  In resident mode
// every node of the CTA must fit (the host sizes stage_cap so).
__device__ void stage_build(const SolveParams& P, int bid, int nbk) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int F = P.F;
  const bool res = P.resident != 0 && P.mode == 0 && P.NA > 0;
  const int cnt = bid < F ? (F - bid + nbk - 1) / nbk : 0;
  auto node_counts = [&](int s, int& r, int& a, int& l, int& c, int& g, int& z) {
    r = 0;
    a = 0;
    l = 0;
    c = 0;
    g = 0;
    z = 0;
    if (s < cnt) {
      r = __ldg(P.order + s * nbk + bid);
      a = __ldg(P.item_off + r + 1) - __ldg(P.item_off + r);
      const int4 ci = __ldg(P.con_info + r);
      l = ci.x;
      c = ci.y;
      g = ci.z;
      z = ci.w;
    }
  };
  auto scan = [&](int v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    return v;
  };
  if (wib == 0) {
    const int nrows = res ? stage_coarse_rows(P.NC, bid, nbk) : 0;
    int used = nrows * P.NC * 4, n = 0, ni = 0, nl = 0, nc = 0, na = 0, nz = 0;
    bool more = P.stage_cap > 0 && P.mode == 0;
    for (int c0 = 0; c0 < cnt && more; c0 += 32) {
      int r, a, l, c, g, z;
      node_counts(c0 + lane, r, a, l, c, g, z);
      const int bytes = c0 + lane < cnt ? stage_node_bytes(a, l, c, g, z, res) : 0;
      const int ib = scan(bytes), ia = scan(a), il = scan(l), ic = scan(c), ig = scan(g), iz = scan(z);
      // inclusive byte sums grow with the lane, so the slots that fit are a prefix
      const unsigned fit = __ballot_sync(0xffffffffu, c0 + lane < cnt && used + ib <= P.stage_cap);
      const int kf = __popc(fit);
      if (kf > 0) {
        used += __shfl_sync(0xffffffffu, ib, kf - 1);
        ni += __shfl_sync(0xffffffffu, ia, kf - 1);
        nl += __shfl_sync(0xffffffffu, il, kf - 1);
        nc += __shfl_sync(0xffffffffu, ic, kf - 1);
        na += __shfl_sync(0xffffffffu, ig, kf - 1);
        nz += __shfl_sync(0xffffffffu, iz, kf - 1);
        n += kf;
      }
      more = kf == 32;
    }
    // the two halves of a warp are staged together: an even count unless all fit
    if (n < cnt) {
      n &= ~1;
      if (res && lane == 0) raise_status(&P.bar->status, ARAP_EUNSUPPORTED);
    }
    if (lane == 0) {
      StageLayout L;
      L.n = n;
      L.ncon = res ? nc : 0;
      L.nrows = nrows;
      if (!res) {
        na = 0;
        nz = 0;
      }
      L.nd = 576 * n;
      L.nx = L.nd + 16 * n;
      L.dp = L.nx + 16 * n;
      L.it = L.dp + 16 * n;
      L.ax = L.it + 16 * ni;
      L.gv = L.ax + 16 * ni;
      L.vec = L.gv + 16 * nl;
      L.xf = L.vec + (res ? kResVecs * 48 * n : 0);
      L.yd = L.xf + (res ? 48 * n : 0);
      L.cu = L.yd + (res ? 16 * ni : 0);
      L.rot = L.cu + (res ? 16 * nc : 0);
      L.mm = L.rot + (res ? 432 * n : 0);
      L.zz = L.mm + 576 * na;
      L.crow = L.zz + 48 * na;
      L.nent = na;
      L.gsg = L.crow + 4 * nrows * P.NC;
      L.cgs = L.gsg + 16 * nz;
      L.ga = L.cgs + (res ? 8 * nc : 0);
      L.cg = L.ga + 4 * nl;
      L.mag = L.cg + (res ? 4 * nc : 0);
      L.gsr = L.mag + 4 * na;
      s_stg = L;
    }
  }
  __syncthreads();
  const int n = s_stg.n;
  if (n == 0) return;
  if (wib == 0) {
    // node records, list, constraint-item and coupled-aggregate bases
    int ib = 0, lb = 0, cb = 0, gb = 0, zb = 0;
    for (int c0 = 0; c0 < n; c0 += 32) {
      const int sl = c0 + lane;
      int r, a, l, c, g, z;
      node_counts(sl < n ? sl : cnt, r, a, l, c, g, z);
      const int ia = scan(a), il = scan(l), ic = scan(c), ig = scan(g), iz = scan(z);
      if (sl < n) {
        stg_node()[sl] = make_int4(r, ib + ia - a, a, P.NA ? __ldg(P.agg + r) : 0);
        stg_base()[sl] = make_int4(lb + il - l, cb + ic - c, c | (g << 16), gb + ig - g);
        // the offset's fourth word holds the slot base of the node's member-anchor slots
        const float4 dp = P.NA ? __ldcg(P.dpiv + r) : make_float4(0.f, 0.f, 0.f, 0.f);
        stg_dpiv()[sl] = make_float4(dp.x, dp.y, dp.z, __int_as_float(zb + iz - z));
      }
      ib += __shfl_sync(0xffffffffu, ia, 31);
      lb += __shfl_sync(0xffffffffu, il, 31);
      cb += __shfl_sync(0xffffffffu, ic, 31);
      gb += __shfl_sync(0xffffffffu, ig, 31);
      zb += __shfl_sync(0xffffffffu, iz, 31);
    }
  }
  __syncthreads();
  const float w = P.wgf;
  for (int sl = wib; sl < n; sl += kSolveWarps) {
    const int4 nd = stg_node()[sl];
    const int r = nd.x;
    const int b0 = __ldg(P.item_off + r);
    const int j = __ldg(P.free_ids + r);
    const float gj[3] = {__ldg(P.node_pos + 3 * (size_t)j), __ldg(P.node_pos + 3 * (size_t)j + 1),
                         __ldg(P.node_pos + 3 * (size_t)j + 2)};
    const int4 bs = stg_base()[sl];
    int lb = bs.x, cb = bs.y, zb = __float_as_int(stg_dpiv()[sl].w);
    for (int q0 = 0; q0 < nd.z; q0 += 32) {
      const int q = q0 + lane;
      const bool has = q < nd.z;
      int4 m = has ? __ldg(P.items + b0 + q) : make_int4(ITEM_STATIC, -1, 0, 0);
      const int kind = m.x & 15;
      float4 ax = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 yd = make_float4(0.f, 0.f, 0.f, 0.f);
      int f0 = 0, len = 0;
      if (kind == ITEM_OUT || kind == ITEM_IN) {
        // the geometry fetch_item forms: sgn (g_k - g_j), w * scale
        const float sgn = kind == ITEM_OUT ? 1.f : -1.f;
        ax = make_float4(sgn * (__ldg(P.node_pos + 3 * (size_t)m.z) - gj[0]),
                         sgn * (__ldg(P.node_pos + 3 * (size_t)m.z + 1) - gj[1]),
                         sgn * (__ldg(P.node_pos + 3 * (size_t)m.z + 2) - gj[2]), w * __int_as_float(m.w));
        if (res && P.NA && m.y >= 0) yd = __ldcg(P.dpiv + m.y);
      } else if (kind == ITEM_CON) {
        ax = __ldcg(P.mem_geo + m.y);
        if (P.NA) {
          f0 = __ldg(P.gca_off + m.z);
          len = __ldg(P.gca_off + m.z + 1) - f0;
        }
      }
      const int il = scan(len);
      const int ic = scan(kind == ITEM_CON && P.NA ? 1 : 0);
      const int loff = lb + il - len;
      if (kind == ITEM_CON && P.NA) {
        for (int e = 0; e < len; ++e) {
          stg_lv()[loff + e] = __ldcg(P.gcv + f0 + e);
          stg_la()[loff + e] = __ldg(P.gca + f0 + e);
        }
        if (res) {
          const int ci = cb + ic - 1;
          stg_cg()[ci] = m.z;
          m.x = ITEM_CON | (ci << 4);
        }
      }
      // member-anchor slots of the constraint item's group (resident mode)
      int zs = 0, z0 = 0;
      if (res && kind == ITEM_CON) {
        z0 = __ldg(P.grp_off + m.z) * P.k;
        zs = __ldg(P.grp_off + m.z + 1) * P.k - z0;
      }
      const int iz = scan(zs);
      if (res && kind == ITEM_CON) {
        const int off = zb + iz - zs;
        stg_cgs()[cb + ic - 1] = make_int2(off, zs);
        for (int e = 0; e < zs; ++e) {
          stg_gsr()[off + e] = __ldg(P.mem_rank + z0 + e);
          stg_gsg()[off + e] = __ldcg(P.mem_geo + z0 + e);
        }
      }
      if (kind == ITEM_CON && P.NA) {
        m.y = loff;
        m.w = len;
      }
      if (has) {
        stg_item()[nd.y + q] = m;
        stg_geo()[nd.y + q] = ax;
        if (res) stg_ydp()[nd.y + q] = yd;
      }
      lb += __shfl_sync(0xffffffffu, il, 31);
      cb += __shfl_sync(0xffffffffu, ic, 31);
      zb += __shfl_sync(0xffffffffu, iz, 31);
    }
  }
  __syncthreads();
  if (res) {
    for (int sl = wib; sl < n; sl += kSolveWarps) build_coarse_blocks(P, sl);
    __syncthreads();
  }
}

}  // namespace arap
