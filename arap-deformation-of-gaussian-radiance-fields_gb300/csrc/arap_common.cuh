// Shared device code for the sm_103a ARAP library: status word, bounded grid
// barrier with a deterministic FP64 reduction, small 3x3 / quaternion math,
// polar factors and real-SH band rotation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/arap_gb300.h"

#define ARAP_CUDA_TRY(expr)                   \
  do {                                        \
    cudaError_t _e = (expr);                  \
    if (_e != cudaSuccess) return ARAP_ECUDA; \
  } while (0)

#define ARAP_LAUNCH_CHECK()                                  \
  do {                                                       \
    if (cudaPeekAtLastError() != cudaSuccess) {              \
      (void)cudaGetLastError();                              \
      return ARAP_ECUDA;                                     \
    }                                                        \
  } while (0)

namespace arap {

// Device-side error word of one handle (solver, grid, skinning plan) or the
// caller's own word passed to a stateless call: the first ARAP_* code raised
// wins until the host reads and clears it (status_read_clear).  A null word
// records nothing (the outputs still carry the NaNs).
__device__ __forceinline__ void raise_status(int* st, int code) {
  if (st) atomicCAS(st, 0, code);
}

// Host: copy a device status word to the host, clear it, synchronise the
// stream; returns the word, or ARAP_ECUDA when a copy fails (api.cu).
int status_read_clear(int* status_dev, cudaStream_t stream);

// ------------------------------------------------------------ barrier ----
// Grid-wide barrier for cooperative launches (all CTAs co-resident).  Every
// wait is bounded: after its limit of polls a waiting CTA records the
// timeout, marks the barrier failed and returns false; callers then leave the
// kernel.
//
// Counter barrier with a reduction.  Arrivals go to one monotonic counter
// (zeroed before each launch): the arrivals of the e-th barrier of a launch
// are the counts e*nb .. (e+1)*nb-1, so a CTA that has passed e barriers
// waits for the count (e+1)*nb and nothing is ever reset.  Each barrier
// carries up to kReduceSlots FP64 sums: a CTA's sums go to
// partials[e & 1][cta][slot] before the release-add of its arrival; after the
// acquire that sees every arrival, warp 0 of every CTA loads all partials at
// once and adds them in CTA order, so every CTA gets the same bits.  Two
// partial buffers suffice: a CTA can only reach barrier e+2 once every CTA has
// arrived at e+1, i.e. has finished reading barrier e.
// count and failed are zeroed before each launch (the first 8 bytes);
// spin_limit is written once by the barrier's owner (the configured limit,
// read by the waits of GridSyncT<true>).  A wait that runs out sets failed,
// which the owner reports as ARAP_ETIMEOUT.  status is the owner's device
// status word (raise_status), kept across launches until the host reads it.
struct GridBarrier {
  unsigned int count;
  int failed;
  unsigned int spin_limit;  // polls of one wait before it gives up (GridSyncT<true>)
  int status;
};

constexpr long long kSpinLimit = 1ll << 23;  // default polls of a barrier wait
constexpr int kReduceSlots = 4;
constexpr int kMaxGridCtas = 160;  // CTAs a barrier reduction supports (5 per lane)

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned int* p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int ld_relaxed_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Float-float addition (hi, lo) += (bh, bl): TwoSum of the high parts
// (Knuth, TAOCP vol. 2, 4.2.2) plus the low parts, renormalised.  No
// multiplications, so no contraction into FMA can change it.
__device__ __forceinline__ void dd_add(float& hi, float& lo, float bh, float bl) {
  const float s = hi + bh;
  const float bb = s - hi;
  float err = (hi - (s - bb)) + (bh - bb);
  err += lo + bl;
  hi = s + err;
  lo = err - (hi - s);
}

// Float-float products and quotients (Dekker's method with an FMA for the
// exact product error), for the few scalars that must not lose the precision
// the float-float sums keep.
__device__ __forceinline__ float2 dd_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, fmaf(a.y, b.x, e));
  const float hi = p + e;
  return make_float2(hi, e - (hi - p));
}
__device__ __forceinline__ float2 dd_sub(float2 a, float2 b) {
  float hi = a.x, lo = a.y;
  dd_add(hi, lo, -b.x, -b.y);
  return make_float2(hi, lo);
}
__device__ __forceinline__ float2 dd_div(float2 a, float2 b) {
  const float q1 = a.x / b.x;
  const float2 r = dd_sub(a, dd_mul(b, make_float2(q1, 0.f)));
  const float q2 = r.x / b.x;
  const float hi = q1 + q2;
  return make_float2(hi, q2 - (hi - q1));
}

// Butterfly float-float sum over the warp; lane 0's result is the one used.
__device__ __forceinline__ void dd_warp_sum(float& hi, float& lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    dd_add(hi, lo, h2, l2);
  }
}

// Per-thread handle of the grid barrier over a group of nb co-resident CTAs
// (the whole grid, or one instance's share of a batched launch); bid is this
// CTA's index in the group.  Every thread of every CTA of the group must make
// the same sequence of calls (the epoch is counted in registers).
//
// A wait gives up after kSpinLimit polls, or with kCfgLimit after the
// barrier record's spin_limit polls (read at every poll).  The two are kept
// apart because the wait is inlined at every barrier of the persistent solve,
// and any form of a run-time limit there (a register, a parameter, a field of
// this handle, a load every 64 polls, an offset start count, an out-of-line
// wait) made the whole solve kernel 9-10 % slower on a GB300, against a
// constant bound; the solver runs the kCfgLimit form only when a spin limit
// is configured.
template <bool kCfgLimit>
struct GridSyncT {
  GridBarrier* bar;
  double* partials;  // [2][nb][kReduceSlots]
  unsigned int epoch;
  unsigned int nb;
  unsigned int bid;

  __device__ __forceinline__ long long spin_cap() const {
    if constexpr (kCfgLimit)
      return (long long)ld_relaxed_u32(&bar->spin_limit);
    else
      return kSpinLimit;
  }

  // One thread per CTA: arrive at barrier e (release) and wait (acquire) for
  // every CTA; bounded, false on failure.
  __device__ bool arrive_and_wait(unsigned int e) {
    red_release_add_u32(&bar->count, 1u);
    const unsigned int target = (e + 1u) * nb;
    long long it = 0;
    while ((int)(ld_acquire_u32(&bar->count) - target) < 0) {
      ++it;
      if ((it & 63) == 0 && ld_relaxed_i32(&bar->failed)) return false;
      if (it > spin_cap()) {
        atomicExch(&bar->failed, 1);
        return false;
      }
      if (it > 1024) __nanosleep(32);
    }
    return true;
  }

  // v[] holds this thread's contributions on entry and the grid-wide sums on
  // return (the same bits in every thread of every CTA).  Returns false when
  // the barrier failed (timed out here or elsewhere).
  template <int NSLOT>
  __device__ bool reduce(double (&v)[NSLOT]) {
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) v[s] = warp_sum(v[s]);
    return reduce_warp_sums<NSLOT>(v);
  }

  // As reduce, for float contributions, in FP32 only (FP64 arithmetic has
  // ~64-cycle latency on this part): float warp sums, then float-float
  // (hi, lo) sums above the warp (Knuth's TwoSum), so the grid-wide sum keeps
  // about twice float's precision; returned as float-float pairs.  Every CTA
  // adds the same terms in the same order, so all get the same bits.
  template <int NSLOT>
  __device__ bool reduce_f(const float (&vf)[NSLOT], float2 (&out)[NSLOT]) {
    static_assert(NSLOT >= 1 && NSLOT <= kReduceSlots, "slots");
    __shared__ float s_redf[32][NSLOT];
    __shared__ float2 s_outf[NSLOT];
    __shared__ int s_okf;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned int e = epoch++;
    float2* buf = reinterpret_cast<float2*>(partials + (size_t)(e & 1u) * kReduceSlots * nb);
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) {
      const float ws = warp_sum(vf[s]);
      if (lane == 0) s_redf[w][s] = ws;
    }
    __syncthreads();
    if (w == 0) {
      const int nw = blockDim.x >> 5;
#pragma unroll
      for (int s = 0; s < NSLOT; ++s) {
        float hi = lane < nw ? s_redf[lane][s] : 0.f, lo = 0.f;
        dd_warp_sum(hi, lo);
        if (lane == 0) buf[(size_t)bid * kReduceSlots + s] = make_float2(hi, lo);
      }
      int ok = 1;
      if (lane == 0) ok = arrive_and_wait(e);
      __syncwarp();
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (ok) {
        constexpr int kQ = kMaxGridCtas / 32;
        float2 t[kQ][NSLOT];
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
          const unsigned int c = lane + 32u * q;
#pragma unroll
          for (int s = 0; s < NSLOT; ++s)
            t[q][s] = c < nb ? __ldcg(buf + (size_t)c * kReduceSlots + s) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int s = 0; s < NSLOT; ++s) {
          float hi = 0.f, lo = 0.f;
#pragma unroll
          for (int q = 0; q < kQ; ++q) dd_add(hi, lo, t[q][s].x, t[q][s].y);
          dd_warp_sum(hi, lo);
          if (lane == 0) s_outf[s] = make_float2(hi, lo);  // lane 0's association order, as in every CTA
        }
      }
      if (lane == 0) s_okf = ok;
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) out[s] = s_outf[s];
    return s_okf != 0;
  }

  // v[] holds the warp's sums (valid in lane 0) on entry.
  template <int NSLOT>
  __device__ bool reduce_warp_sums(double (&v)[NSLOT]) {
    static_assert(NSLOT >= 1 && NSLOT <= kReduceSlots, "slots");
    __shared__ double s_red[32][NSLOT];
    __shared__ double s_out[NSLOT];
    __shared__ int s_ok;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned int e = epoch++;
    double* buf = partials + (size_t)(e & 1u) * kReduceSlots * nb;
    if (lane == 0) {
#pragma unroll
      for (int s = 0; s < NSLOT; ++s) s_red[w][s] = v[s];
    }
    __syncthreads();
    if (w == 0) {
      const int nw = blockDim.x >> 5;
#pragma unroll
      for (int s = 0; s < NSLOT; ++s) {
        double c = lane < nw ? s_red[lane][s] : 0.0;
        c = warp_sum(c);
        if (lane == 0) buf[(size_t)bid * kReduceSlots + s] = c;
      }
      int ok = 1;
      if (lane == 0) ok = arrive_and_wait(e);
      __syncwarp();
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (ok) {
        // every slot of every CTA requested at once, then added in CTA order
        constexpr int kQ = kMaxGridCtas / 32;
        double t[kQ][NSLOT];
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
          const unsigned int c = lane + 32u * q;
#pragma unroll
          for (int s = 0; s < NSLOT; ++s) t[q][s] = c < nb ? __ldcg(buf + (size_t)c * kReduceSlots + s) : 0.0;
        }
#pragma unroll
        for (int s = 0; s < NSLOT; ++s) {
          double a = 0.0;
#pragma unroll
          for (int q = 0; q < kQ; ++q) a += t[q][s];
          a = warp_sum(a);
          if (lane == 0) s_out[s] = a;  // lane 0's association order, as in every CTA
        }
      }
      if (lane == 0) s_ok = ok;
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) v[s] = s_out[s];
    return s_ok != 0;
  }

  // Plain barrier (no sums): one arrival per CTA, as in reduce.
  __device__ bool sync() {
    __shared__ int s_sync_ok;
    const unsigned int e = epoch++;
    __syncthreads();
    if (threadIdx.x == 0) s_sync_ok = arrive_and_wait(e) ? 1 : 0;
    __syncthreads();
    return s_sync_ok != 0;
  }
};
using GridSync = GridSyncT<false>;

// Block-wide FP64 sum (blockDim.x multiple of 32, <= 1024); all threads get it.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double s_red[32][NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) s_red[w][i] = v[i];
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double a = 0.0;
    for (int j = 0; j < nw; ++j) a += s_red[j][i];
    v[i] = a;
  }
  __syncthreads();
}

// ----------------------------------------------------------- 3x3 math ----
// Row-major 3x3 in m[r*3+c].
template <typename T>
__device__ __forceinline__ T det3(const T* m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// Inverse-transpose by cofactors: out = (m^{-1})^T = cof(m)/det.
template <typename T>
__device__ __forceinline__ bool inv_transpose3(const T* m, T* out) {
  T c[9];
  c[0] = m[4] * m[8] - m[5] * m[7];
  c[1] = m[5] * m[6] - m[3] * m[8];
  c[2] = m[3] * m[7] - m[4] * m[6];
  c[3] = m[2] * m[7] - m[1] * m[8];
  c[4] = m[0] * m[8] - m[2] * m[6];
  c[5] = m[1] * m[6] - m[0] * m[7];
  c[6] = m[1] * m[5] - m[2] * m[4];
  c[7] = m[2] * m[3] - m[0] * m[5];
  c[8] = m[0] * m[4] - m[1] * m[3];
  const T det = m[0] * c[0] + m[1] * c[1] + m[2] * c[2];
  if (!(det != T(0))) return false;
  const T inv = T(1) / det;
#pragma unroll
  for (int i = 0; i < 9; ++i) out[i] = c[i] * inv;
  return true;
}

// Orthogonal polar factor U V^T of a non-singular M by Newton's iteration
// X <- (g X + X^{-T}/g)/2 with Higham's Frobenius-norm scaling g for the first
// steps (N. J. Higham, "Computing the polar decomposition -- with
// applications", SIAM J. Sci. Stat. Comput. 7 (1986)).  Keeps det's sign, so a
// reflection stays a reflection, as U V^T of an SVD does.  Returns false when
// an iterate is singular.
template <typename T>
__device__ __forceinline__ bool polar_factor(const T* M, T* R, int max_it, T tol) {
  T X[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) X[i] = M[i];
  for (int it = 0; it < max_it; ++it) {
    T Y[9];
    if (!inv_transpose3(X, Y)) return false;
    T g = T(1), ig = T(1);
    if (it < 3) {
      T nx = 0, ny = 0;
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        nx += X[i] * X[i];
        ny += Y[i] * Y[i];
      }
      g = sqrt(sqrt(ny / nx));
      ig = T(1) / g;
    }
    T delta = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const T xn = T(0.5) * (g * X[i] + Y[i] * ig);
      delta = fmax(delta, fabs(xn - X[i]));
      X[i] = xn;
    }
    if (delta < tol) break;
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = X[i];
  return true;
}

// Unscaled Newton iteration M <- (M + M^{-T})/2 stopped when max|dM| < 1e-6,
// returning the iterate before the final update (helper.cpp:506-517).
template <typename T>
__device__ __forceinline__ bool newton_polar_ref(T* M, int max_it) {
  for (int it = 0; it < max_it; ++it) {
    T Y[9];
    if (!inv_transpose3(M, Y)) return false;
    T delta = 0;
    T nxt[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      nxt[i] = T(0.5) * (M[i] + Y[i]);
      delta = fmax(delta, fabs(M[i] - nxt[i]));
    }
    if (delta < T(1e-6)) return true;
#pragma unroll
    for (int i = 0; i < 9; ++i) M[i] = nxt[i];
  }
  return true;
}

// ---------------------------------------------------------- quaternions --
// (w,x,y,z).  Matrix -> quaternion by Shoemake's trace / largest-diagonal
// method (K. Shoemake, "Animating rotation with quaternion curves",
// SIGGRAPH 1985).  Not normalised.
__device__ __forceinline__ float4 quat_from_rowmajor(const float* m) {
  float4 q;
  const float tr = m[0] + m[4] + m[8];
  if (tr > 0.0f) {
    float t = sqrtf(tr + 1.0f);
    q.x = 0.5f * t;
    t = 0.5f / t;
    q.y = (m[7] - m[5]) * t;
    q.z = (m[2] - m[6]) * t;
    q.w = (m[3] - m[1]) * t;
  } else {
    int i = 0;
    if (m[4] > m[0]) i = 1;
    if (m[8] > m[i * 4]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    float t = sqrtf(m[i * 4] - m[j * 4] - m[k * 4] + 1.0f);
    float v[3];
    v[i] = 0.5f * t;
    t = 0.5f / t;
    const float w = (m[k * 3 + j] - m[j * 3 + k]) * t;
    v[j] = (m[j * 3 + i] + m[i * 3 + j]) * t;
    v[k] = (m[k * 3 + i] + m[i * 3 + k]) * t;
    q.x = w;
    q.y = v[0];
    q.z = v[1];
    q.w = v[2];
  }
  return q;  // .x=w .y=x .z=y .w=z
}

__device__ __forceinline__ float4 quat_normalize(float4 q) {
  const float n = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  const float inv = 1.0f / n;
  return make_float4(q.x * inv, q.y * inv, q.z * inv, q.w * inv);
}

// Hamilton product a*b, (w,x,y,z) stored in (.x,.y,.z,.w).
__device__ __forceinline__ float4 quat_mul(float4 a, float4 b) {
  return make_float4(a.x * b.x - a.y * b.y - a.z * b.z - a.w * b.w,
                     a.x * b.y + a.y * b.x + a.z * b.w - a.w * b.z,
                     a.x * b.z - a.y * b.w + a.z * b.x + a.w * b.y,
                     a.x * b.w + a.y * b.z - a.z * b.y + a.w * b.x);
}

__device__ __forceinline__ float4 quat_inverse(float4 q) {
  const float n2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
  const float inv = 1.0f / n2;
  return make_float4(q.x * inv, -q.y * inv, -q.z * inv, -q.w * inv);
}

// Unit quaternion -> row-major rotation.
__device__ __forceinline__ void quat_to_rowmajor(float4 q, float* R) {
  const float w = q.x, x = q.y, y = q.z, z = q.w;
  R[0] = 1.0f - 2.0f * (y * y + z * z);
  R[1] = 2.0f * (x * y - w * z);
  R[2] = 2.0f * (x * z + w * y);
  R[3] = 2.0f * (x * y + w * z);
  R[4] = 1.0f - 2.0f * (x * x + z * z);
  R[5] = 2.0f * (y * z - w * x);
  R[6] = 2.0f * (x * z - w * y);
  R[7] = 2.0f * (y * z + w * x);
  R[8] = 1.0f - 2.0f * (x * x + y * y);
}

// ------------------------------------------------------- SH rotation -----
// Rotation of the real spherical harmonics of bands 1..3 (coefficient index
// l*l + l + m, m = -l..l; band 1 in the (y, z, x) order of the 3DGS /
// reference layout), given the rotation as the unit quaternion
// q = (w, x, y, z) in (.x, .y, .z, .w).  It is applied in Euler form: with
// R = Rz(a) Ry(b) Rz(g) and Ry(b) = Rx(-pi/2) Rz(b) Rx(pi/2), every band's
// matrix is D(R) = Dz(a) Dx^T Dz(b) Dx Dz(g).  Dz(t) turns each coefficient
// pair (m, -m) by the angle m t; Dx is the fixed band matrix of a quarter
// turn about x (entries 0, +-1, +-1/2, +-sqrt(3)/2, +-1/4, +-sqrt(6)/4,
// +-sqrt(10)/4, +-sqrt(15)/4: the Ivanic-Ruedenberg band matrices, J. Phys.
// Chem. 100 (1996) 6342, erratum 102 (1998) 9099, at Rx(pi/2)).  The
// angles' cosines and sines come from q without trigonometric calls: with
// A = w^2 + z^2 = cos^2(b/2) and B = x^2 + y^2 = sin^2(b/2),
//   e^{ib} = (A - B) + 2i sqrt(AB),
//   e^{ia} = (w + iz)(y - ix) / sqrt(AB),  e^{ig} = (w + iz)(y + ix) / sqrt(AB).
// Near b = 0 or b = pi only a + g or a - g is defined, and the two half-angle
// factors carry the same rounding into a and g, so the product stays
// accurate; at AB = 0 exactly a = 0 and g takes the whole turn.  No band
// matrix is formed: about 130 multiply-adds per colour channel.
namespace shq {
constexpr float kR3h = 0.866025403784438647f;   // sqrt(3)/2
constexpr float kS10q = 0.790569415042094833f;  // sqrt(10)/4
constexpr float kS6q = 0.612372435695794525f;   // sqrt(6)/4
constexpr float kS15q = 0.968245836551854221f;  // sqrt(15)/4

struct Turns {
  float c[3], s[3];  // cos and sin of 1, 2, 3 times the angle
};
__device__ __forceinline__ Turns turns(float c1, float s1) {
  Turns t;
  t.c[0] = c1;
  t.s[0] = s1;
  t.c[1] = c1 * c1 - s1 * s1;
  t.s[1] = 2.0f * c1 * s1;
  t.c[2] = t.c[1] * c1 - t.s[1] * s1;
  t.s[2] = t.s[1] * c1 + t.c[1] * s1;
  return t;
}
// Dz on one channel: c[0..15] are coefficients 0..15 (index l*l + l + m)
__device__ __forceinline__ void dz(float* c, const Turns& t) {
#pragma unroll
  for (int l = 1; l <= 3; ++l) {
    const int o = l * l + l;
#pragma unroll
    for (int m = 1; m <= l; ++m) {
      const float lo = c[o - m], hi = c[o + m];
      c[o - m] = t.c[m - 1] * lo + t.s[m - 1] * hi;
      c[o + m] = t.c[m - 1] * hi - t.s[m - 1] * lo;
    }
  }
}
// Dx (T = false) or its transpose (T = true) on one channel
template <bool T>
__device__ __forceinline__ void dx(float* c) {
  // band 1 (indices 1..3 = m -1, 0, 1): (-c0, c-1, c1) or its inverse
  {
    const float a = c[1], b = c[2];
    c[1] = T ? b : -b;
    c[2] = T ? -a : a;
  }
  // band 2 (indices 4..8 = m -2..2)
  {
    const float m2 = c[4], m1 = c[5], z = c[6], p1 = c[7], p2 = c[8];
    if (!T) {
      c[4] = -p1;
      c[5] = -m1;
      c[6] = -0.5f * z - kR3h * p2;
      c[7] = m2;
      c[8] = -kR3h * z + 0.5f * p2;
    } else {
      c[4] = p1;
      c[5] = -m1;
      c[6] = -0.5f * z - kR3h * p2;
      c[7] = -m2;
      c[8] = -kR3h * z + 0.5f * p2;
    }
  }
  // band 3 (indices 9..15 = m -3..3)
  {
    const float m3 = c[9], m2 = c[10], m1 = c[11], z = c[12], p1 = c[13], p2 = c[14], p3 = c[15];
    if (!T) {
      c[9] = kS10q * z - kS6q * p2;
      c[10] = -m2;
      c[11] = kS6q * z + kS10q * p2;
      c[12] = -kS10q * m3 - kS6q * m1;
      c[13] = -0.25f * p1 - kS15q * p3;
      c[14] = kS6q * m3 - kS10q * m1;
      c[15] = -kS15q * p1 + 0.25f * p3;
    } else {
      c[9] = -kS10q * z + kS6q * p2;
      c[10] = -m2;
      c[11] = -kS6q * z - kS10q * p2;
      c[12] = kS10q * m3 + kS6q * m1;
      c[13] = -0.25f * p1 - kS15q * p3;
      c[14] = -kS6q * m3 + kS10q * m1;
      c[15] = -kS15q * p1 + 0.25f * p3;
    }
  }
}
}  // namespace shq

// Rotates interleaved SH s[coef*3 + rgb] (16 coefficients) by q.  With FLIP
// the odd coefficients are negated before and after the band rotation (the
// sign convention of cudakdtree.cu:160-196 and GaussianView.cpp:3138-3154).
template <bool FLIP>
__device__ __forceinline__ void rotate_sh48(float4 q, float* s) {
  const float w = q.x, x = q.y, y = q.z, z = q.w;
  const float A = w * w + z * z, B = x * x + y * y;
  float ca = w * y + x * z, sa = y * z - w * x, cg = w * y - x * z, sg = y * z + w * x;
  const float n2 = ca * ca + sa * sa;
  if (n2 > 1e-30f) {
    const float inv = rsqrtf(n2);
    ca *= inv;
    sa *= inv;
    cg *= inv;
    sg *= inv;
  } else if (A >= B) {  // b = 0: g = 2 arg(w + iz)
    ca = 1.0f;
    sa = 0.0f;
    cg = (w * w - z * z) / A;
    sg = 2.0f * w * z / A;
  } else {  // b = pi: g = 2 arg(y + ix)
    ca = 1.0f;
    sa = 0.0f;
    cg = (y * y - x * x) / B;
    sg = 2.0f * x * y / B;
  }
  const shq::Turns ta = shq::turns(ca, sa), tb = shq::turns(A - B, 2.0f * sqrtf(A * B)),
                   tg = shq::turns(cg, sg);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    float c[16];
    c[0] = s[ch];  // band 0: unchanged
#pragma unroll
    for (int k = 1; k < 16; ++k) c[k] = (FLIP && (k & 1)) ? -s[k * 3 + ch] : s[k * 3 + ch];
    shq::dz(c, tg);
    shq::dx<false>(c);
    shq::dz(c, tb);
    shq::dx<true>(c);
    shq::dz(c, ta);
#pragma unroll
    for (int k = 1; k < 16; ++k) s[k * 3 + ch] = (FLIP && (k & 1)) ? -c[k] : c[k];
  }
}

// ------------------------------------------------------ segment sort ----
// Ascending sort of one segment keys[0..L) of DISTINCT keys by one CTA, for
// segments longer than a shared-memory sort holds: chunks of CHUNK keys are
// bitonic-sorted in shared memory (s_keys, CHUNK keys, padded with `pad`,
// larger than every key), then runs are merged pairwise through scratch[0..L)
// (global memory of the caller's), each key going straight to its place: its
// index in its own run plus its rank in the other run (a binary search; the
// keys being distinct, no two keys claim one place).
template <typename T, int CHUNK>
__device__ void cta_sort_distinct(T* keys, T* scratch, int L, T pad, T* s_keys) {
  const int tid = threadIdx.x, bd = blockDim.x;
  for (int c0 = 0; c0 < L; c0 += CHUNK) {
    const int n = min(CHUNK, L - c0);
    int P2 = 1;
    while (P2 < n) P2 <<= 1;
    for (int t = tid; t < P2; t += bd) s_keys[t] = t < n ? keys[c0 + t] : pad;
    __syncthreads();
    for (int k = 2; k <= P2; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = tid; t < P2; t += bd) {
          const int u = t ^ j;
          if (u > t) {
            const T a = s_keys[t], b = s_keys[u];
            if ((a > b) == ((t & k) == 0)) {
              s_keys[t] = b;
              s_keys[u] = a;
            }
          }
        }
        __syncthreads();
      }
    for (int t = tid; t < n; t += bd) keys[c0 + t] = s_keys[t];
    __syncthreads();
  }
  T* a = keys;
  T* b = scratch;
  for (int w = CHUNK; w < L; w <<= 1) {
    for (int i = tid; i < L; i += bd) {
      const int base = (i / (2 * w)) * (2 * w);
      const bool left = i - base < w;
      const int o0 = left ? base + w : base;  // the other run
      const int on = left ? max(0, min(w, L - (base + w))) : w;
      const T x = a[i];
      int lo = 0, hi = on;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[o0 + mid] < x) lo = mid + 1; else hi = mid;
      }
      b[base + (left ? i - base : i - base - w) + lo] = x;
    }
    __syncthreads();
    T* t = a;
    a = b;
    b = t;
  }
  if (a != keys) {
    for (int i = tid; i < L; i += bd) keys[i] = a[i];
    __syncthreads();
  }
}

// ------------------------------------------------------------ helpers ----
__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// Exactly rounded float32 distance as (dx*dx + dy*dy) + dz*dz without FMA
// contraction (Deform.hpp:164-165).
__device__ __forceinline__ float dist2_rn(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

inline int grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  return (int)(g > 0x7fffffffll ? 0x7fffffff : (g < 1 ? 1 : g));
}

}  // namespace arap
