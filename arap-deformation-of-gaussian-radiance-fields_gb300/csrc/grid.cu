// Density grid (sm_103a): scene box, Gaussian -> cell CSR, grid samples,
// adaptive low-pass filter and Gaussian-mixture density sampling.
//
// Reference: getOverallAABB (GaussianView.cpp:3601-3631), the per-Gaussian
// boxes and cell binning of getGridSamples / UpdateContainingRelationship
// (GaussianView.cpp:3634-3867, 3870-4149; GetBoxesGsGrid cudakdtree.cu:425-451),
// the serial list fill (GaussianView.cpp:4077-4100) whose per-cell order --
// ascending Gaussian index -- is reproduced by a per-cell sort after an
// atomic fill, GetAdaLpfRatio (GaussianView.cpp:4670-4751) and the host
// contract of CudaRasterizer::forward3d_grid (GaussianView.cpp:4222-4249),
// and the library's definition of the Stage-II alignment step
// (GaussianView.cpp:4363-4486: L1loss3d, backward3d_grid, update3d, whose
// source is not in the reference tree).
#include <atomic>
#include <climits>
#include <cmath>
#include <new>
#include <vector>

#include "arap_common.cuh"

namespace arap {

struct GridParams {
  float mn[3];
  float mx[3];
  float step;
  float interval;
  int g;
  int padding;
};

__device__ __forceinline__ unsigned int f2ord(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned int u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void minmax_kernel(int N, const float* __restrict__ pos, unsigned int* __restrict__ mm) {
  unsigned int lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const unsigned int o = f2ord(pos[3 * (size_t)i + c]);
      lo[c] = min(lo[c], o);
      hi[c] = max(hi[c], o);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = min(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = max(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      atomicMin(mm + c, lo[c]);
      atomicMax(mm + 3 + c, hi[c]);
    }
  }
}

// getOverallAABB in float32, then grid_step = max over axes of extent / g.
__global__ void params_kernel(const unsigned int* __restrict__ mm, int g, int padding, GridParams* P) {
  if (threadIdx.x != 0) return;
  float mn[3], mx[3];
  for (int c = 0; c < 3; ++c) {
    const float a = ord2f(mm[c]), b = ord2f(mm[3 + c]);
    const float mean = (b + a) / 2.0f;
    const float lo = (a - mean) * 1.1f + mean;
    const float hi = ((b - mean) * 1.1f + mean - lo) * 1.0078125f + lo;
    mn[c] = fminf(lo, -0.75f);
    mx[c] = fmaxf(hi, 0.75f);
  }
  float step = 0.f;
  for (int c = 0; c < 3; ++c) {
    P->mn[c] = mn[c];
    P->mx[c] = mx[c];
    step = fmaxf(step, (mx[c] - mn[c]) / (float)g);
  }
  P->step = step;
  P->interval = step / 4.0f;
  P->g = g;
  P->padding = padding;
}

// Per-Gaussian cell range of its box (GaussianView.cpp:3961-4019, 4077-4085)
// and the per-cell counts.
__global__ void ranges_kernel(int N, const float* __restrict__ pos, const float* __restrict__ rot,
                              const float* __restrict__ scale, const float* __restrict__ opacity,
                              const GridParams* __restrict__ Pg, int* __restrict__ ranges,
                              int* __restrict__ cell_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const GridParams P = *Pg;
  const float a = opacity[i];
  const float cut = 1.0f / 255.0f;
  float f = 0.f;
  if (!(a <= cut)) f = sqrtf(-2.0f * logf(cut / a));
  float R[9];
  quat_to_rowmajor(quat_normalize(__ldg(reinterpret_cast<const float4*>(rot) + i)), R);
  const float p[3] = {pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2]};
  float lo[3] = {p[0], p[1], p[2]}, hi[3] = {p[0], p[1], p[2]};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float s3 = f * scale[3 * (size_t)i + d];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float e = R[c * 3 + d] * s3;
      const float u = p[c] + e, v = p[c] - e;
      lo[c] = fminf(lo[c], fminf(u, v));
      hi[c] = fmaxf(hi[c], fmaxf(u, v));
    }
  }
  int r[6];
  int cnt = 1;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    r[2 * c] = max((int)floorf((lo[c] - P.mn[c]) / P.step) - P.padding, 0);
    r[2 * c + 1] = min((int)floorf((hi[c] - P.mn[c]) / P.step) + P.padding, P.g - 1);
    cnt *= max(0, r[2 * c + 1] - r[2 * c] + 1);
  }
#pragma unroll
  for (int t = 0; t < 6; ++t) ranges[6 * (size_t)i + t] = r[t];
  if (cnt <= 0) return;
  const int g = P.g;
  for (int x = r[0]; x <= r[1]; ++x)
    for (int y = r[2]; y <= r[3]; ++y)
      for (int z = r[4]; z <= r[5]; ++z) atomicAdd(cell_count + ((size_t)x * g + y) * g + z, 1);
}

__global__ void fill_kernel(int N, const int* __restrict__ ranges, const GridParams* __restrict__ Pg,
                            const int* __restrict__ off, int* __restrict__ cursor, int* __restrict__ lists) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int g = Pg->g;
  const int* r = ranges + 6 * (size_t)i;
  for (int x = r[0]; x <= r[1]; ++x)
    for (int y = r[2]; y <= r[3]; ++y)
      for (int z = r[4]; z <= r[5]; ++z) {
        const size_t c = ((size_t)x * g + y) * g + z;
        const int slot = atomicAdd(cursor + c, 1);
        lists[off[c] + slot] = i;
      }
}

// ------------------------------------------------------------- scan -----
constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void scan_reduce_kernel(int n, const int* __restrict__ in, long long* __restrict__ sums) {
  long long v[1] = {0};
  const int base = blockIdx.x * kScanTile;
  for (int t = threadIdx.x; t < kScanTile; t += kScanThreads) {
    const int i = base + t;
    if (i < n) v[0] += in[i];
  }
  double d[1] = {(double)v[0]};
  block_sum<1>(d);
  if (threadIdx.x == 0) sums[blockIdx.x] = (long long)llrint(d[0]);
}

// exclusive scan of the tile sums by one CTA; total at sums[nb]
__global__ void scan_sums_kernel(int nb, long long* __restrict__ sums) {
  __shared__ long long s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += blockDim.x) {
    const int i = base + threadIdx.x;
    long long v = i < nb ? sums[i] : 0;
    // inclusive warp scan
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    __shared__ long long s_w[32];
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    if (w == 0) {
      long long t = lane < (int)(blockDim.x >> 5) ? s_w[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      s_w[lane] = t;
    }
    __syncthreads();
    const long long incl = x + (w > 0 ? s_w[w - 1] : 0) + s_carry;
    if (i < nb) sums[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[nb] = s_carry;
}

__global__ void scan_apply_kernel(int n, const int* __restrict__ in, const long long* __restrict__ sums,
                                  int* __restrict__ out) {
  __shared__ long long s_w[kScanThreads / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  long long loc[kScanItems];
  long long t = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const int i = base + j;
    loc[j] = t;
    t += (i < n) ? in[i] : 0;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[w] = x;
  __syncthreads();
  long long wp = 0;
  for (int q = 0; q < w; ++q) wp += s_w[q];
  const long long excl = sums[blockIdx.x] + wp + x - t;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const int i = base + j;
    if (i < n) {
      const long long v = excl + loc[j];
      out[i] = v > INT_MAX ? INT_MAX : (int)v;
    }
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = (int)min(sums[gridDim.x], (long long)INT_MAX);
}

// ------------------------------------------------------ per-cell sort ----
__global__ void flags_kernel(int n, const int* __restrict__ count, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = count[i] > 0 ? 1 : 0;
}

__global__ void compact_kernel(int n, const int* __restrict__ count, const int* __restrict__ pos,
                               int* __restrict__ valid) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && count[i] > 0) valid[pos[i]] = i;
}

constexpr int kSortMax = 16384;

// Bitonic sort of each occupied cell's list in shared memory (one CTA per
// cell).  A cell longer than kSortMax is appended to big[] (count in
// *big_n) for sort_big_cells_kernel.
__global__ void sort_cells_kernel(int nvalid, const int* __restrict__ valid, const int* __restrict__ off,
                                  int* __restrict__ lists, int* __restrict__ big_n, int* __restrict__ big) {
  extern __shared__ int s_keys[];
  const int v = blockIdx.x;
  if (v >= nvalid) return;
  const int c = valid[v];
  const int b = off[c], L = off[c + 1] - b;
  if (L <= 1) return;
  if (L > kSortMax) {
    if (threadIdx.x == 0) big[atomicAdd(big_n, 1)] = v;
    return;
  }
  int P2 = 1;
  while (P2 < L) P2 <<= 1;
  for (int t = threadIdx.x; t < P2; t += blockDim.x) s_keys[t] = t < L ? lists[b + t] : INT_MAX;
  __syncthreads();
  for (int k = 2; k <= P2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < P2; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const int a = s_keys[t], bb = s_keys[u];
          const bool up = (t & k) == 0;
          if ((a > bb) == up) {
            s_keys[t] = bb;
            s_keys[u] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int t = threadIdx.x; t < L; t += blockDim.x) lists[b + t] = s_keys[t];
}

// Lengths of the cells sort_cells_kernel set aside.
__global__ void big_cell_sizes_kernel(int nbig, const int* __restrict__ big, const int* __restrict__ valid,
                                      const int* __restrict__ off, int* __restrict__ sizes) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nbig) return;
  const int c = valid[big[k]];
  sizes[k] = off[c + 1] - off[c];
}

// The long cells, one CTA each: chunk sorts and merges (cta_sort_distinct)
// through the cell's part of scratch (at scratch_off[k], the cell's length).
__global__ void __launch_bounds__(1024) sort_big_cells_kernel(int nbig, const int* __restrict__ big,
                                                              const int* __restrict__ valid,
                                                              const int* __restrict__ off, int* lists,
                                                              int* scratch, const long long* __restrict__ scratch_off) {
  extern __shared__ int s_keys[];
  const int k = blockIdx.x;
  if (k >= nbig) return;
  const int c = valid[big[k]];
  const int b = off[c], L = off[c + 1] - b;
  cta_sort_distinct<int, kSortMax>(lists + b, scratch + scratch_off[k], L, INT_MAX, s_keys);
}

// Cell of each Gaussian centre (GaussianView.cpp:3918-3928) and per-cell counts.
__global__ void center_cell_kernel(int N, const float* __restrict__ pos, const GridParams* __restrict__ Pg,
                                   int* __restrict__ cell, int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const GridParams P = *Pg;
  int c3[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    c3[c] = min(max((int)floorf((pos[3 * (size_t)i + c] - P.mn[c]) / P.step), 0), P.g - 1);
  const int id = (c3[0] * P.g + c3[1]) * P.g + c3[2];
  cell[i] = id;
  atomicAdd(count + id, 1);
}

__global__ void center_fill_kernel(int N, const int* __restrict__ cell, const int* __restrict__ off,
                                   int* __restrict__ cursor, int* __restrict__ lists) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int c = cell[i];
  lists[off[c] + atomicAdd(cursor + c, 1)] = i;
}

// 64 samples per occupied cell (GaussianView.cpp:4104-4133).
__global__ void samples_kernel(int nvalid, const int* __restrict__ valid, const GridParams* __restrict__ Pg,
                               float* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nvalid * 64) return;
  const GridParams P = *Pg;
  const int v = t >> 6, s = t & 63;
  const int c = valid[v];
  const int g = P.g;
  const int ci[3] = {c / (g * g), (c % (g * g)) / g, c % g};
  const int si[3] = {s / 16, (s % 16) / 4, s % 4};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    // float32 multiply and add kept separate, as the reference's host code
    const float base = (float)((double)__fadd_rn(P.mn[d], __fmul_rn((float)ci[d], P.step)) + 0.5 * (double)P.interval);
    out[3 * (size_t)t + d] = __fadd_rn(base, __fmul_rn((float)si[d], P.interval));
  }
}

// GetAdaLpfRatio: M = P Q^T (Q Q^T)^-1 with Q the unit-cube corners and P
// the corner samples' offsets / 3; out = lpf * M M^T (row-major 3x3).
__global__ void ada_lpf_kernel(int nvalid, const float* __restrict__ samples, float lpf, float* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvalid) return;
  const float* S = samples + (size_t)v * 64 * 3;
  float PQ[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};  // [coord][axis]
#pragma unroll
  for (int cidx = 1; cidx < 8; ++cidx) {
    const int bx = cidx & 1, by = (cidx >> 1) & 1, bz = (cidx >> 2) & 1;
    const int idx = bx * 48 + by * 12 + bz * 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float pd = (S[3 * idx + d] - S[d]) / 3.0f;
      if (bx) PQ[d][0] += pd;
      if (by) PQ[d][1] += pd;
      if (bz) PQ[d][2] += pd;
    }
  }
  // (Q Q^T)^-1 = 0.5 I - 0.125 * ones
  float M[3][3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float s = PQ[d][0] + PQ[d][1] + PQ[d][2];
#pragma unroll
    for (int j = 0; j < 3; ++j) M[d][j] = 0.5f * PQ[d][j] - 0.125f * s;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      out[(size_t)v * 9 + a * 3 + b] = lpf * (M[a][0] * M[b][0] + M[a][1] * M[b][1] + M[a][2] * M[b][2]);
}

// Density sampling: one CTA of 64 threads per occupied cell, one thread per
// sample; the cell's Gaussians are staged in shared memory in chunks with
// their inverse filtered covariance (S_i + L)^-1.
constexpr int kDensChunk = 64;

__global__ void __launch_bounds__(64) density_kernel(
    int nvalid, const int* __restrict__ valid, const int* __restrict__ off, const int* __restrict__ lists,
    const float* __restrict__ pos, const float* __restrict__ rot, const float* __restrict__ scale,
    const float* __restrict__ opacity, const float* __restrict__ shs, const float* __restrict__ samples,
    const float* __restrict__ ada, float lpf, float* __restrict__ sigma, float* __restrict__ feat) {
  __shared__ float s_mu[kDensChunk][3];
  __shared__ float s_A[kDensChunk][6];
  __shared__ float s_a[kDensChunk];
  __shared__ float s_sh[kDensChunk][48];
  const int v = blockIdx.x;
  if (v >= nvalid) return;
  const int c = valid[v];
  const int b = off[c], L = off[c + 1] - b;
  float Lm[6];
  if (ada) {
    const float* m = ada + (size_t)v * 9;
    Lm[0] = m[0]; Lm[1] = m[1]; Lm[2] = m[2]; Lm[3] = m[4]; Lm[4] = m[5]; Lm[5] = m[8];
  } else {
    Lm[0] = lpf; Lm[1] = 0.f; Lm[2] = 0.f; Lm[3] = lpf; Lm[4] = 0.f; Lm[5] = lpf;
  }
  const int s = threadIdx.x;
  const size_t sid = (size_t)v * 64 + s;
  const float x = samples[3 * sid], y = samples[3 * sid + 1], z = samples[3 * sid + 2];
  float acc = 0.f;
  float F[48];
#pragma unroll
  for (int t = 0; t < 48; ++t) F[t] = 0.f;
  for (int c0 = 0; c0 < L; c0 += kDensChunk) {
    const int cnt = min(kDensChunk, L - c0);
    __syncthreads();
    if (s < cnt) {
      const int gi = lists[b + c0 + s];
      float R[9];
      quat_to_rowmajor(quat_normalize(__ldg(reinterpret_cast<const float4*>(rot) + gi)), R);
      const float s2[3] = {scale[3 * (size_t)gi] * scale[3 * (size_t)gi],
                           scale[3 * (size_t)gi + 1] * scale[3 * (size_t)gi + 1],
                           scale[3 * (size_t)gi + 2] * scale[3 * (size_t)gi + 2]};
      float C6[6];
      int o = 0;
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = r; q < 3; ++q)
          C6[o++] = R[r * 3] * s2[0] * R[q * 3] + R[r * 3 + 1] * s2[1] * R[q * 3 + 1] + R[r * 3 + 2] * s2[2] * R[q * 3 + 2];
#pragma unroll
      for (int t = 0; t < 6; ++t) C6[t] += Lm[t];
      // inverse of the symmetric 3x3 (a b c; b d e; c e f)
      const float a = C6[0], bb = C6[1], cc = C6[2], d = C6[3], e = C6[4], f = C6[5];
      const float A0 = d * f - e * e, A1 = cc * e - bb * f, A2 = bb * e - cc * d;
      const float det = a * A0 + bb * A1 + cc * A2;
      const float id = 1.0f / det;
      s_A[s][0] = A0 * id;
      s_A[s][1] = A1 * id;
      s_A[s][2] = A2 * id;
      s_A[s][3] = (a * f - cc * cc) * id;
      s_A[s][4] = (bb * cc - a * e) * id;
      s_A[s][5] = (a * d - bb * bb) * id;
      s_mu[s][0] = pos[3 * (size_t)gi];
      s_mu[s][1] = pos[3 * (size_t)gi + 1];
      s_mu[s][2] = pos[3 * (size_t)gi + 2];
      s_a[s] = opacity[gi];
    }
    // stage SH cooperatively: cnt * 48 floats
    for (int t = s; t < cnt * 12; t += 64) {
      const int gq = t / 12, q4 = t % 12;
      const int gi = lists[b + c0 + gq];
      const float4 u = __ldg(reinterpret_cast<const float4*>(shs + 48 * (size_t)gi) + q4);
      s_sh[gq][4 * q4] = u.x;
      s_sh[gq][4 * q4 + 1] = u.y;
      s_sh[gq][4 * q4 + 2] = u.z;
      s_sh[gq][4 * q4 + 3] = u.w;
    }
    __syncthreads();
    for (int q = 0; q < cnt; ++q) {
      const float dx = x - s_mu[q][0], dy = y - s_mu[q][1], dz = z - s_mu[q][2];
      const float* A = s_A[q];
      const float m = A[0] * dx * dx + A[3] * dy * dy + A[5] * dz * dz +
                      2.f * (A[1] * dx * dy + A[2] * dx * dz + A[4] * dy * dz);
      const float gw = s_a[q] * __expf(-0.5f * m);
      acc += gw;
#pragma unroll
      for (int t = 0; t < 48; ++t) F[t] = fmaf(gw, s_sh[q][t], F[t]);
    }
  }
  sigma[sid] = acc;
  float4* fo = reinterpret_cast<float4*>(feat + 48 * sid);
#pragma unroll
  for (int t = 0; t < 12; ++t) fo[t] = make_float4(F[4 * t], F[4 * t + 1], F[4 * t + 2], F[4 * t + 3]);
}

// ------------------------------------------------- Stage-II alignment ----
// The library's definition of the step the viewer runs through the
// un-vendored rasteriser (L1loss3d + backward3d_grid + update3d): an L1 loss
// between the field of the current Gaussians and the target field at the
// grid samples, its gradient to the raw attributes (mean, quaternion,
// log-scale, logit opacity, SH) and an Adam step.
//
// stage2_pair_kernel: one CTA of 64 threads per occupied cell.  Pass 1: one
// thread per sample forms sigma and F as density_kernel does (from the raw
// attributes) and the sample's dL/dsigma and dL/dF.  Pass 2: one thread per
// Gaussian of the cell's list walks the 64 samples and sums that pair's
// contribution, so no reduction across threads is needed; it writes 58
// floats per pair (dL/dSH 48 | dL/dalpha | dL/dmu 3 | dL/dSigma 6, the upper
// triangle of the symmetric matrix) into planes [58][npairs] at the pair's
// CSR position.  stage2_gather_kernel then sums each Gaussian's pairs in
// ascending cell order (deterministic) and applies the chain rule.
constexpr int kS2Floats = 58;
constexpr int kS2Params = 59;  // per Gaussian: opacity 1 | SH 48 | mean 3 | quaternion 4 | log-scale 3

__device__ __forceinline__ float sign0(float v) { return (v > 0.f) ? 1.f : ((v < 0.f) ? -1.f : 0.f); }

__device__ __forceinline__ void stage2_stage(int cnt, int base, const int* __restrict__ lists,
                                             const float* __restrict__ pos, const float* __restrict__ rot,
                                             const float* __restrict__ log_scale, const float* __restrict__ logit_op,
                                             const float* __restrict__ shs, const float* Lm,
                                             float (*s_mu)[3], float (*s_A)[6], float* s_a, float (*s_sh)[48]) {
  const int s = threadIdx.x;
  if (s < cnt) {
    const int gi = lists[base + s];
    float R[9];
    quat_to_rowmajor(quat_normalize(__ldg(reinterpret_cast<const float4*>(rot) + gi)), R);
    float s2[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float sc = __expf(log_scale[3 * (size_t)gi + d]);
      s2[d] = sc * sc;
    }
    float C6[6];
    int o = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int q = r; q < 3; ++q)
        C6[o++] = R[r * 3] * s2[0] * R[q * 3] + R[r * 3 + 1] * s2[1] * R[q * 3 + 1] + R[r * 3 + 2] * s2[2] * R[q * 3 + 2];
#pragma unroll
    for (int t = 0; t < 6; ++t) C6[t] += Lm[t];
    const float a = C6[0], bb = C6[1], cc = C6[2], d = C6[3], e = C6[4], f = C6[5];
    const float A0 = d * f - e * e, A1 = cc * e - bb * f, A2 = bb * e - cc * d;
    const float id = 1.0f / (a * A0 + bb * A1 + cc * A2);
    s_A[s][0] = A0 * id;
    s_A[s][1] = A1 * id;
    s_A[s][2] = A2 * id;
    s_A[s][3] = (a * f - cc * cc) * id;
    s_A[s][4] = (bb * cc - a * e) * id;
    s_A[s][5] = (a * d - bb * bb) * id;
    s_mu[s][0] = pos[3 * (size_t)gi];
    s_mu[s][1] = pos[3 * (size_t)gi + 1];
    s_mu[s][2] = pos[3 * (size_t)gi + 2];
    s_a[s] = 1.0f / (1.0f + __expf(-logit_op[gi]));
  }
  for (int t = s; t < cnt * 12; t += 64) {
    const int gq = t / 12, q4 = t % 12;
    const int gi = lists[base + gq];
    const float4 u = __ldg(reinterpret_cast<const float4*>(shs + 48 * (size_t)gi) + q4);
    s_sh[gq][4 * q4] = u.x;
    s_sh[gq][4 * q4 + 1] = u.y;
    s_sh[gq][4 * q4 + 2] = u.z;
    s_sh[gq][4 * q4 + 3] = u.w;
  }
}

__global__ void __launch_bounds__(64) stage2_pair_kernel(
    int nvalid, const int* __restrict__ valid, const int* __restrict__ off, const int* __restrict__ lists,
    long long npairs, const float* __restrict__ pos, const float* __restrict__ rot,
    const float* __restrict__ log_scale, const float* __restrict__ logit_op, const float* __restrict__ shs,
    const float* __restrict__ samples, const float* __restrict__ ada, float lpf,
    const float* __restrict__ aim_sigma, const float* __restrict__ aim_feat,
    const uint8_t* __restrict__ cell_active, float wf, float* __restrict__ part, float* __restrict__ loss_cta) {
  __shared__ float s_mu[kDensChunk][3];
  __shared__ float s_A[kDensChunk][6];
  __shared__ float s_a[kDensChunk];
  __shared__ float s_sh[kDensChunk][48];
  __shared__ float s_x[64][3];
  __shared__ float s_ds[64];
  __shared__ float s_df[64][48];
  __shared__ float s_red[2][2];
  const int v = blockIdx.x;
  if (v >= nvalid) return;
  const int c = valid[v];
  const int b = off[c], L = off[c + 1] - b;
  const bool act = cell_active == nullptr || cell_active[v] != 0;
  float Lm[6];
  if (ada) {
    const float* m = ada + (size_t)v * 9;
    Lm[0] = m[0]; Lm[1] = m[1]; Lm[2] = m[2]; Lm[3] = m[4]; Lm[4] = m[5]; Lm[5] = m[8];
  } else {
    Lm[0] = lpf; Lm[1] = 0.f; Lm[2] = 0.f; Lm[3] = lpf; Lm[4] = 0.f; Lm[5] = lpf;
  }
  const int s = threadIdx.x;
  const size_t sid = (size_t)v * 64 + s;
  const float x = samples[3 * sid], y = samples[3 * sid + 1], z = samples[3 * sid + 2];
  s_x[s][0] = x;
  s_x[s][1] = y;
  s_x[s][2] = z;
  // pass 1: the sample's sigma and F
  float acc = 0.f;
  float F[48];
#pragma unroll
  for (int t = 0; t < 48; ++t) F[t] = 0.f;
  for (int c0 = 0; c0 < L; c0 += kDensChunk) {
    const int cnt = min(kDensChunk, L - c0);
    __syncthreads();
    stage2_stage(cnt, b + c0, lists, pos, rot, log_scale, logit_op, shs, Lm, s_mu, s_A, s_a, s_sh);
    __syncthreads();
    for (int q = 0; q < cnt; ++q) {
      const float dx = x - s_mu[q][0], dy = y - s_mu[q][1], dz = z - s_mu[q][2];
      const float* A = s_A[q];
      const float m = A[0] * dx * dx + A[3] * dy * dy + A[5] * dz * dz +
                      2.f * (A[1] * dx * dy + A[2] * dx * dz + A[4] * dy * dz);
      const float gw = s_a[q] * __expf(-0.5f * m);
      acc += gw;
#pragma unroll
      for (int t = 0; t < 48; ++t) F[t] = fmaf(gw, s_sh[q][t], F[t]);
    }
  }
  // dL/dsigma and dL/dF of the sample, and its loss terms
  float ls = 0.f, lf = 0.f;
  {
    const float ts = aim_sigma[sid];
    ls = act ? fabsf(acc - ts) : 0.f;
    s_ds[s] = act ? sign0(acc - ts) : 0.f;
    const float4* tf = reinterpret_cast<const float4*>(aim_feat + 48 * sid);
#pragma unroll
    for (int t = 0; t < 12; ++t) {
      const float4 u = tf[t];
      const float tv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const float dv = F[4 * t + h] - tv[h];
        lf += act ? fabsf(dv) : 0.f;
        s_df[s][4 * t + h] = act ? wf * sign0(dv) : 0.f;
      }
    }
    lf *= wf;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ls += __shfl_xor_sync(0xffffffffu, ls, o);
    lf += __shfl_xor_sync(0xffffffffu, lf, o);
  }
  if ((s & 31) == 0) {
    s_red[s >> 5][0] = ls;
    s_red[s >> 5][1] = lf;
  }
  // pass 2: one thread per Gaussian of the chunk over the cell's 64 samples
  for (int c0 = 0; c0 < L; c0 += kDensChunk) {
    const int cnt = min(kDensChunk, L - c0);
    __syncthreads();
    stage2_stage(cnt, b + c0, lists, pos, rot, log_scale, logit_op, shs, Lm, s_mu, s_A, s_a, s_sh);
    __syncthreads();
    if (s < cnt) {
      const float mx = s_mu[s][0], my = s_mu[s][1], mz = s_mu[s][2];
      float A[6];
#pragma unroll
      for (int t = 0; t < 6; ++t) A[t] = s_A[s][t];
      const float al = s_a[s];
      float sh[48];
#pragma unroll
      for (int h = 0; h < 48; ++h) sh[h] = s_sh[s][h];
      float gsh[48];
#pragma unroll
      for (int t = 0; t < 48; ++t) gsh[t] = 0.f;
      float ga = 0.f, gm[3] = {0.f, 0.f, 0.f}, gS[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (act) {
        for (int t = 0; t < 64; ++t) {
          const float dx = s_x[t][0] - mx, dy = s_x[t][1] - my, dz = s_x[t][2] - mz;
          const float ax = A[0] * dx + A[1] * dy + A[2] * dz;
          const float ay = A[1] * dx + A[3] * dy + A[4] * dz;
          const float az = A[2] * dx + A[4] * dy + A[5] * dz;
          const float G = __expf(-0.5f * (dx * ax + dy * ay + dz * az));
          const float gw = al * G;
          float cc = s_ds[t];
#pragma unroll
          for (int h = 0; h < 48; ++h) {
            const float dfv = s_df[t][h];
            cc = fmaf(dfv, sh[h], cc);
            gsh[h] = fmaf(gw, dfv, gsh[h]);
          }
          ga = fmaf(cc, G, ga);
          const float de = cc * gw;
          gm[0] = fmaf(de, ax, gm[0]);
          gm[1] = fmaf(de, ay, gm[1]);
          gm[2] = fmaf(de, az, gm[2]);
          const float hd = 0.5f * de;
          gS[0] = fmaf(hd * ax, ax, gS[0]);
          gS[1] = fmaf(hd * ax, ay, gS[1]);
          gS[2] = fmaf(hd * ax, az, gS[2]);
          gS[3] = fmaf(hd * ay, ay, gS[3]);
          gS[4] = fmaf(hd * ay, az, gS[4]);
          gS[5] = fmaf(hd * az, az, gS[5]);
        }
      }
      const size_t p = (size_t)b + c0 + s;
      const size_t np = (size_t)npairs;
#pragma unroll
      for (int h = 0; h < 48; ++h) part[h * np + p] = gsh[h];
      part[48 * np + p] = ga;
#pragma unroll
      for (int h = 0; h < 3; ++h) part[(49 + h) * np + p] = gm[h];
#pragma unroll
      for (int h = 0; h < 6; ++h) part[(52 + h) * np + p] = gS[h];
    }
  }
  __syncthreads();
  if (s == 0) {
    loss_cta[2 * (size_t)v] = s_red[0][0] + s_red[1][0];
    loss_cta[2 * (size_t)v + 1] = s_red[0][1] + s_red[1][1];
  }
}

__global__ void stage2_gather_kernel(int N, int g, const int* __restrict__ ranges, const int* __restrict__ off,
                                     const int* __restrict__ lists, long long npairs,
                                     const float* __restrict__ part, const float* __restrict__ rot,
                                     const float* __restrict__ log_scale, const float* __restrict__ logit_op,
                                     float* __restrict__ g_pos, float* __restrict__ g_rot,
                                     float* __restrict__ g_ls, float* __restrict__ g_lo,
                                     float* __restrict__ g_shs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  float acc[kS2Floats];
#pragma unroll
  for (int h = 0; h < kS2Floats; ++h) acc[h] = 0.f;
  const int* r = ranges + 6 * (size_t)i;
  const size_t np = (size_t)npairs;
  for (int x = r[0]; x <= r[1]; ++x)
    for (int y = r[2]; y <= r[3]; ++y)
      for (int z = r[4]; z <= r[5]; ++z) {
        const size_t c = ((size_t)x * g + y) * g + z;
        int lo = off[c], hi = off[c + 1];
        const int end = hi;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (lists[mid] < i) lo = mid + 1; else hi = mid;
        }
        if (lo < end && lists[lo] == i) {
#pragma unroll
          for (int h = 0; h < kS2Floats; ++h) acc[h] += part[h * np + lo];
        }
      }
  float4* gs = reinterpret_cast<float4*>(g_shs + 48 * (size_t)i);
#pragma unroll
  for (int t = 0; t < 12; ++t) gs[t] = make_float4(acc[4 * t], acc[4 * t + 1], acc[4 * t + 2], acc[4 * t + 3]);
  const float al = 1.0f / (1.0f + __expf(-logit_op[i]));
  g_lo[i] = acc[48] * al * (1.0f - al);
#pragma unroll
  for (int h = 0; h < 3; ++h) g_pos[3 * (size_t)i + h] = acc[49 + h];
  // dL/dSigma as the full symmetric matrix
  const float G[9] = {acc[52], acc[53], acc[54], acc[53], acc[55], acc[56], acc[54], acc[56], acc[57]};
  const float4 q = __ldg(reinterpret_cast<const float4*>(rot) + i);
  const float nq = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  const float4 qn = make_float4(q.x / nq, q.y / nq, q.z / nq, q.w / nq);
  float R[9];
  quat_to_rowmajor(qn, R);
  float sc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) sc[k] = __expf(log_scale[3 * (size_t)i + k]);
  float M[9];  // G R
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int k = 0; k < 3; ++k) M[a * 3 + k] = G[a * 3] * R[k] + G[a * 3 + 1] * R[3 + k] + G[a * 3 + 2] * R[6 + k];
  float dR[9];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float rtgr = R[k] * M[k] + R[3 + k] * M[3 + k] + R[6 + k] * M[6 + k];
    g_ls[3 * (size_t)i + k] = 2.0f * sc[k] * rtgr * sc[k];
#pragma unroll
    for (int a = 0; a < 3; ++a) dR[a * 3 + k] = 2.0f * M[a * 3 + k] * sc[k] * sc[k];
  }
  const float w = qn.x, x = qn.y, y = qn.z, z = qn.w;
  const float dw = 2.f * (-z * dR[1] + y * dR[2] + z * dR[3] - x * dR[5] - y * dR[6] + x * dR[7]);
  const float dx = 2.f * (y * dR[1] + z * dR[2] + y * dR[3] - 2.f * x * dR[4] - w * dR[5] + z * dR[6] +
                          w * dR[7] - 2.f * x * dR[8]);
  const float dy = 2.f * (-2.f * y * dR[0] + x * dR[1] + w * dR[2] + x * dR[3] + z * dR[5] - w * dR[6] +
                          z * dR[7] - 2.f * y * dR[8]);
  const float dz = 2.f * (-2.f * z * dR[0] - w * dR[1] + x * dR[2] + w * dR[3] - 2.f * z * dR[4] + y * dR[5] +
                          x * dR[6] + y * dR[7]);
  const float dot = w * dw + x * dx + y * dy + z * dz;
  reinterpret_cast<float4*>(g_rot)[i] =
      make_float4((dw - w * dot) / nq, (dx - x * dot) / nq, (dy - y * dot) / nq, (dz - z * dot) / nq);
}

// Adam over the 59 attributes of each moved Gaussian; m and v are [N][59] in
// the order opacity | SH | mean | quaternion | log-scale.
struct Stage2Adam {
  float* p[5];
  const float* g[5];
  float lr[5];
};

__global__ void stage2_adam_kernel(int N, Stage2Adam A, const uint8_t* __restrict__ moved, float* __restrict__ m,
                                   float* __restrict__ v, float b1, float b2, float eps, float bc1, float bc2) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)N * kS2Params) return;
  const int i = (int)(e / kS2Params);
  const int r = (int)(e % kS2Params);
  if (moved && !moved[i]) return;
  int a, k, width;
  if (r < 1) { a = 0; k = r; width = 1; }
  else if (r < 49) { a = 1; k = r - 1; width = 48; }
  else if (r < 52) { a = 2; k = r - 49; width = 3; }
  else if (r < 56) { a = 3; k = r - 52; width = 4; }
  else { a = 4; k = r - 56; width = 3; }
  const size_t idx = (size_t)i * width + k;
  const float gv = A.g[a][idx];
  const float mm = b1 * m[e] + (1.0f - b1) * gv;
  const float vv = b2 * v[e] + (1.0f - b2) * gv * gv;
  m[e] = mm;
  v[e] = vv;
  A.p[a][idx] -= A.lr[a] * (mm / bc1) / (sqrtf(vv / bc2) + eps);
}

// JudgeEmptyGrid (GaussianView.cpp:4272-4316) and ExpandOpRange
// (GaussianView.cpp:4319-4360) over the occupied cells: a cell marks itself
// and its six face neighbours (clamped to the grid) in a g^3 byte map.
__device__ __forceinline__ void mark_with_neighbours(int c, int g, uint8_t* __restrict__ map) {
  const int x = c / (g * g), y = (c / g) % g, z = c % g;
  map[c] = 1;
  map[(size_t)max(x - 1, 0) * g * g + y * g + z] = 1;
  map[(size_t)min(x + 1, g - 1) * g * g + y * g + z] = 1;
  map[(size_t)x * g * g + max(y - 1, 0) * g + z] = 1;
  map[(size_t)x * g * g + min(y + 1, g - 1) * g + z] = 1;
  map[(size_t)x * g * g + y * g + max(z - 1, 0)] = 1;
  map[(size_t)x * g * g + y * g + min(z + 1, g - 1)] = 1;
}

// mode 0: cells whose 64 aim opacities, summed in order in float, exceed 1e-6
// mark; mode 1: cells not converged mark.
__global__ void cell_mark_kernel(int nvalid, const int* __restrict__ valid, int g, int mode,
                                 const float* __restrict__ aim_opacity, const uint8_t* __restrict__ converged,
                                 uint8_t* __restrict__ map) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvalid) return;
  bool mark;
  if (mode == 0) {
    float tot = 0.f;
    for (int j = 0; j < 64; ++j) tot = __fadd_rn(tot, aim_opacity[(size_t)v * 64 + j]);
    mark = (double)tot > 1e-6;
  } else {
    mark = converged[v] == 0;
  }
  if (mark) mark_with_neighbours(valid[v], g, map);
}

// mode 0: empty_out[v] = 1 for an unmarked cell; mode 1: converged_io[v] = 0
// for a marked cell.
__global__ void cell_flag_kernel(int nvalid, const int* __restrict__ valid, int mode,
                                 const uint8_t* __restrict__ map, uint8_t* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvalid) return;
  const bool m = map[valid[v]] != 0;
  if (mode == 0) out[v] = m ? 0 : 1;
  else if (m) out[v] = 0;
}

}  // namespace arap

// ------------------------------------------------------------------ host --
using namespace arap;

struct arap_grid {
  int N = 0, g = 0, padding = 1, nvalid = 0;
  long long npairs = 0;
  GridParams* params = nullptr;  // device
  int* status = nullptr;         // device status word of the grid's kernels
  int* off = nullptr;            // [g^3 + 1]
  int* lists = nullptr;          // [npairs]
  int* valid = nullptr;          // [nvalid]
  int* ranges = nullptr;         // [N*6]
  GridParams host{};
  // Stage-II scratch: pair partials [58][npairs] then the per-cell losses
  // [nvalid][2]; allocated by the first arap_stage2_loss_grad call
  mutable float* stage2_scratch = nullptr;
  mutable size_t stage2_floats = 0;
};

static int scan_exclusive(const int* in, int* out, int n, long long* sums, cudaStream_t st) {
  const int nb = (n + kScanTile - 1) / kScanTile;
  scan_reduce_kernel<<<nb, kScanThreads, 0, st>>>(n, in, sums);
  scan_sums_kernel<<<1, 1024, 0, st>>>(nb, sums);
  scan_apply_kernel<<<nb, kScanThreads, 0, st>>>(n, in, sums, out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

// Sort every occupied cell's list ascending: one CTA per cell in shared
// memory, then the cells longer than kSortMax (the reference's serial fill
// has no limit, GaussianView.cpp:4077-4100) by sort_big_cells_kernel.
// big_n [1], big and sizes [nvalid] are free device ints of the caller's;
// alloc(bytes) gives the long cells' scratch (device memory, 8-byte aligned)
// or nullptr when there is no room, and the call then returns no_room.
template <typename Alloc>
static int sort_cell_lists(int nvalid, const int* valid, const int* off, int* lists, int* big_n, int* big,
                           int* sizes, Alloc alloc, int no_room, cudaStream_t st) {
  if (nvalid <= 0) return ARAP_OK;
  if (cudaMemsetAsync(big_n, 0, sizeof(int), st) != cudaSuccess ||
      cudaFuncSetAttribute(sort_cells_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kSortMax * (int)sizeof(int)) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  sort_cells_kernel<<<nvalid, 256, kSortMax * sizeof(int), st>>>(nvalid, valid, off, lists, big_n, big);
  int nbig = 0;
  if (cudaPeekAtLastError() != cudaSuccess ||
      cudaMemcpyAsync(&nbig, big_n, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  if (nbig == 0) return ARAP_OK;
  big_cell_sizes_kernel<<<grid_for(nbig, 128), 128, 0, st>>>(nbig, big, valid, off, sizes);
  std::vector<int> hs(nbig);
  if (cudaPeekAtLastError() != cudaSuccess ||
      cudaMemcpyAsync(hs.data(), sizes, sizeof(int) * (size_t)nbig, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  std::vector<long long> so((size_t)nbig + 1, 0);
  for (int k = 0; k < nbig; ++k) so[k + 1] = so[k] + hs[k];
  const size_t b_off = sizeof(long long) * ((size_t)nbig + 1);
  char* scr = static_cast<char*>(alloc(b_off + sizeof(int) * (size_t)so[nbig]));
  if (!scr) return no_room;
  long long* d_so = reinterpret_cast<long long*>(scr);
  int* d_keys = reinterpret_cast<int*>(scr + b_off);
  if (cudaMemcpyAsync(d_so, so.data(), b_off, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaFuncSetAttribute(sort_big_cells_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kSortMax * (int)sizeof(int)) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  sort_big_cells_kernel<<<nbig, 1024, kSortMax * sizeof(int), st>>>(nbig, big, valid, off, lists, d_keys, d_so);
  if (cudaPeekAtLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  return ARAP_OK;
}

extern "C" void arap_grid_destroy(arap_grid* G) {
  if (!G) return;
  cudaFree(G->params);
  cudaFree(G->status);
  cudaFree(G->off);
  cudaFree(G->lists);
  cudaFree(G->valid);
  cudaFree(G->ranges);
  cudaFree(G->stage2_scratch);
  delete G;
}

extern "C" int arap_grid_build(arap_grid** out, int N, const float* pos, const float* rot, const float* scale,
                               const float* opacity, int grid_num, int padding, arap_grid_info* info_host,
                               arap_stream_t stream) {
  if (!out) return ARAP_EBADINPUT;
  *out = nullptr;
  if (N < 1 || !pos || !rot || !scale || !opacity || grid_num < 1 || grid_num > 1024 || padding < 0)
    return ARAP_EBADINPUT;
  if (reinterpret_cast<uintptr_t>(rot) & 15) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  const long long cells = (long long)grid_num * grid_num * grid_num;
  if (cells >= INT_MAX) return ARAP_EUNSUPPORTED;
  const int C = (int)cells;
  auto* G = new (std::nothrow) arap_grid();
  if (!G) return ARAP_ENOMEM;
  G->N = N;
  G->g = grid_num;
  G->padding = padding;
  int* count = nullptr;
  int* cursor = nullptr;
  int* flagpos = nullptr;
  long long* sums = nullptr;
  unsigned int* mm = nullptr;
  int rc = ARAP_OK;
  const int nbs = (C + 1 + kScanTile - 1) / kScanTile + 1;
  auto fail = [&](int code) {
    cudaFree(count);
    cudaFree(cursor);
    cudaFree(flagpos);
    cudaFree(sums);
    cudaFree(mm);
    arap_grid_destroy(G);
    return code;
  };
  if (cudaMalloc(&G->params, sizeof(GridParams)) || cudaMalloc(&G->status, sizeof(int)) ||
      cudaMalloc(&G->off, sizeof(int) * ((size_t)C + 1)) ||
      cudaMalloc(&G->ranges, sizeof(int) * 6 * (size_t)N) || cudaMalloc(&count, sizeof(int) * (size_t)C) ||
      cudaMalloc(&cursor, sizeof(int) * (size_t)C) || cudaMalloc(&flagpos, sizeof(int) * ((size_t)C + 1)) ||
      cudaMalloc(&sums, sizeof(long long) * (nbs + 1)) || cudaMalloc(&mm, sizeof(unsigned int) * 6)) {
    (void)cudaGetLastError();
    return fail(ARAP_ENOMEM);
  }
  const unsigned int init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  if (cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, st) ||
      cudaMemsetAsync(G->status, 0, sizeof(int), st) ||
      cudaMemsetAsync(count, 0, sizeof(int) * (size_t)C, st) || cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)C, st))
    return fail(ARAP_ECUDA);
  minmax_kernel<<<std::min(grid_for(N, 256), 1184), 256, 0, st>>>(N, pos, mm);
  params_kernel<<<1, 32, 0, st>>>(mm, grid_num, padding, G->params);
  ranges_kernel<<<grid_for(N, 128), 128, 0, st>>>(N, pos, rot, scale, opacity, G->params, G->ranges, count);
  if (cudaPeekAtLastError() != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(ARAP_ECUDA);
  }
  if ((rc = scan_exclusive(count, G->off, C, sums, st)) != ARAP_OK) return fail(rc);
  long long total = 0;
  if (cudaMemcpyAsync(&total, sums + (C + kScanTile - 1) / kScanTile, sizeof(long long), cudaMemcpyDeviceToHost, st) ||
      cudaMemcpyAsync(&G->host, G->params, sizeof(GridParams), cudaMemcpyDeviceToHost, st) ||
      cudaStreamSynchronize(st))
    return fail(ARAP_ECUDA);
  if (total >= INT_MAX) return fail(ARAP_EUNSUPPORTED);
  G->npairs = total;
  if (cudaMalloc(&G->lists, sizeof(int) * (size_t)std::max(total, 1ll))) {
    (void)cudaGetLastError();
    return fail(ARAP_ENOMEM);
  }
  fill_kernel<<<grid_for(N, 128), 128, 0, st>>>(N, G->ranges, G->params, G->off, cursor, G->lists);
  flags_kernel<<<grid_for(C, 256), 256, 0, st>>>(C, count, cursor);
  if ((rc = scan_exclusive(cursor, flagpos, C, sums, st)) != ARAP_OK) return fail(rc);
  int nvalid = 0;
  if (cudaMemcpyAsync(&nvalid, flagpos + C, sizeof(int), cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
    return fail(ARAP_ECUDA);
  G->nvalid = nvalid;
  if (cudaMalloc(&G->valid, sizeof(int) * (size_t)std::max(nvalid, 1))) {
    (void)cudaGetLastError();
    return fail(ARAP_ENOMEM);
  }
  compact_kernel<<<grid_for(C, 256), 256, 0, st>>>(C, count, flagpos, G->valid);
  {
    // count, cursor and flagpos are free now: the long-cell list and lengths
    void* big_scratch = nullptr;
    auto alloc = [&](size_t bytes) -> void* {
      if (cudaMallocAsync(&big_scratch, bytes, st) != cudaSuccess) {
        (void)cudaGetLastError();
        big_scratch = nullptr;
      }
      return big_scratch;
    };
    rc = sort_cell_lists(nvalid, G->valid, G->off, G->lists, flagpos, count, cursor, alloc, ARAP_ENOMEM, st);
    if (big_scratch) cudaFreeAsync(big_scratch, st);
    if (rc != ARAP_OK) return fail(rc);
  }
  if (cudaPeekAtLastError() != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(ARAP_ECUDA);
  }
  if (cudaStreamSynchronize(st)) return fail(ARAP_ECUDA);
  cudaFree(count);
  cudaFree(cursor);
  cudaFree(flagpos);
  cudaFree(sums);
  cudaFree(mm);
  if (info_host) {
    for (int c = 0; c < 3; ++c) {
      info_host->min_xyz[c] = G->host.mn[c];
      info_host->max_xyz[c] = G->host.mx[c];
    }
    info_host->step = G->host.step;
    info_host->interval = G->host.interval;
    info_host->grid_num = grid_num;
    info_host->n_valid = nvalid;
    info_host->n_pairs = total;
  }
  const int gs = status_read_clear(G->status, st);
  if (gs != ARAP_OK) {
    arap_grid_destroy(G);
    return gs;
  }
  *out = G;
  return ARAP_OK;
}

extern "C" int arap_grid_center_order(const arap_grid* G, int N, const float* pos, int32_t* order_out,
                                      arap_stream_t stream) {
  if (!G || !pos || !order_out || N < 1) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  const long long cells = (long long)G->g * G->g * G->g;
  const int C = (int)cells;
  int *cell = nullptr, *count = nullptr, *cursor = nullptr, *off = nullptr, *flagpos = nullptr, *valid = nullptr;
  long long* sums = nullptr;
  const int nbs = (C + 1 + kScanTile - 1) / kScanTile + 1;
  int rc = ARAP_OK;
  auto done = [&](int code) {
    cudaFree(cell); cudaFree(count); cudaFree(cursor); cudaFree(off); cudaFree(flagpos); cudaFree(valid);
    cudaFree(sums);
    return code;
  };
  if (cudaMalloc(&cell, sizeof(int) * (size_t)N) || cudaMalloc(&count, sizeof(int) * (size_t)C) ||
      cudaMalloc(&cursor, sizeof(int) * (size_t)C) || cudaMalloc(&off, sizeof(int) * ((size_t)C + 1)) ||
      cudaMalloc(&flagpos, sizeof(int) * ((size_t)C + 1)) || cudaMalloc(&sums, sizeof(long long) * (nbs + 1))) {
    (void)cudaGetLastError();
    return done(ARAP_ENOMEM);
  }
  if (cudaMemsetAsync(count, 0, sizeof(int) * (size_t)C, st) || cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)C, st))
    return done(ARAP_ECUDA);
  center_cell_kernel<<<grid_for(N, 256), 256, 0, st>>>(N, pos, G->params, cell, count);
  if ((rc = scan_exclusive(count, off, C, sums, st)) != ARAP_OK) return done(rc);
  center_fill_kernel<<<grid_for(N, 256), 256, 0, st>>>(N, cell, off, cursor, order_out);
  flags_kernel<<<grid_for(C, 256), 256, 0, st>>>(C, count, cursor);
  if ((rc = scan_exclusive(cursor, flagpos, C, sums, st)) != ARAP_OK) return done(rc);
  int nvalid = 0;
  if (cudaMemcpyAsync(&nvalid, flagpos + C, sizeof(int), cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
    return done(ARAP_ECUDA);
  if (nvalid > 0) {
    if (cudaMalloc(&valid, sizeof(int) * (size_t)nvalid)) {
      (void)cudaGetLastError();
      return done(ARAP_ENOMEM);
    }
    compact_kernel<<<grid_for(C, 256), 256, 0, st>>>(C, count, flagpos, valid);
    void* big_scratch = nullptr;
    auto alloc = [&](size_t bytes) -> void* {
      if (cudaMallocAsync(&big_scratch, bytes, st) != cudaSuccess) {
        (void)cudaGetLastError();
        big_scratch = nullptr;
      }
      return big_scratch;
    };
    rc = sort_cell_lists(nvalid, valid, off, order_out, flagpos, count, cursor, alloc, ARAP_ENOMEM, st);
    if (big_scratch) cudaFreeAsync(big_scratch, st);
    if (rc != ARAP_OK) return done(rc);
  }
  if (cudaPeekAtLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
    (void)cudaGetLastError();
    return done(ARAP_ECUDA);
  }
  return done(ARAP_OK);
}

extern "C" int arap_grid_status(arap_grid* G, arap_stream_t stream) {
  if (!G) return ARAP_EBADINPUT;
  return status_read_clear(G->status, (cudaStream_t)stream);
}

extern "C" int arap_grid_arrays(const arap_grid* G, const int32_t** cell_offsets, const int32_t** cell_lists,
                                const int32_t** valid_cells) {
  if (!G) return ARAP_EBADINPUT;
  if (cell_offsets) *cell_offsets = G->off;
  if (cell_lists) *cell_lists = G->lists;
  if (valid_cells) *valid_cells = G->valid;
  return ARAP_OK;
}

extern "C" int arap_grid_samples(const arap_grid* G, float* samples_out, arap_stream_t stream) {
  if (!G || !samples_out) return ARAP_EBADINPUT;
  if (G->nvalid == 0) return ARAP_OK;
  samples_kernel<<<grid_for((long long)G->nvalid * 64, 256), 256, 0, (cudaStream_t)stream>>>(
      G->nvalid, G->valid, G->params, samples_out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_grid_ada_lpf(const arap_grid* G, const float* samples, float lpf, float* out,
                                 arap_stream_t stream) {
  if (!G || !samples || !out) return ARAP_EBADINPUT;
  if (G->nvalid == 0) return ARAP_OK;
  ada_lpf_kernel<<<grid_for(G->nvalid, 128), 128, 0, (cudaStream_t)stream>>>(G->nvalid, samples, lpf, out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_grid_density(const arap_grid* G, const float* pos, const float* rot, const float* scale,
                                 const float* opacity, const float* shs, const float* samples, const float* ada,
                                 float lpf, float* sigma_out, float* feature_out, arap_stream_t stream) {
  if (!G || !pos || !rot || !scale || !opacity || !shs || !samples || !sigma_out || !feature_out)
    return ARAP_EBADINPUT;
  if ((reinterpret_cast<uintptr_t>(rot) | reinterpret_cast<uintptr_t>(shs) |
       reinterpret_cast<uintptr_t>(feature_out)) & 15)
    return ARAP_EBADINPUT;
  if (G->nvalid == 0) return ARAP_OK;
  density_kernel<<<G->nvalid, 64, 0, (cudaStream_t)stream>>>(G->nvalid, G->valid, G->off, G->lists, pos, rot,
                                                              scale, opacity, shs, samples, ada, lpf, sigma_out,
                                                              feature_out);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_stage2_loss_grad(const arap_grid* G, const float* pos, const float* rot, const float* log_scale,
                                     const float* logit_opacity, const float* shs, const float* samples,
                                     const float* ada, float lpf, const float* aim_sigma, const float* aim_feature,
                                     const uint8_t* cell_active, float feature_weight, float* grad_pos,
                                     float* grad_rot, float* grad_log_scale, float* grad_logit_opacity,
                                     float* grad_shs, double* loss_host, arap_stream_t stream) {
  if (!G || !pos || !rot || !log_scale || !logit_opacity || !shs || !samples || !aim_sigma || !aim_feature ||
      !grad_pos || !grad_rot || !grad_log_scale || !grad_logit_opacity || !grad_shs)
    return ARAP_EBADINPUT;
  if ((reinterpret_cast<uintptr_t>(rot) | reinterpret_cast<uintptr_t>(shs) |
       reinterpret_cast<uintptr_t>(aim_feature) | reinterpret_cast<uintptr_t>(grad_rot) |
       reinterpret_cast<uintptr_t>(grad_shs)) & 15)
    return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  if (loss_host) loss_host[0] = loss_host[1] = 0.0;
  if (G->N == 0) return ARAP_OK;
  const size_t need = (size_t)kS2Floats * (size_t)G->npairs + 2 * (size_t)G->nvalid;
  if (need > G->stage2_floats) {
    cudaFree(G->stage2_scratch);
    G->stage2_scratch = nullptr;
    G->stage2_floats = 0;
    ARAP_CUDA_TRY(cudaMalloc(&G->stage2_scratch, need * sizeof(float)));
    G->stage2_floats = need;
  }
  float* part = G->stage2_scratch;
  float* loss_cta = part + (size_t)kS2Floats * (size_t)G->npairs;
  if (G->nvalid > 0)
    stage2_pair_kernel<<<G->nvalid, 64, 0, st>>>(G->nvalid, G->valid, G->off, G->lists, G->npairs, pos, rot,
                                                 log_scale, logit_opacity, shs, samples, ada, lpf, aim_sigma,
                                                 aim_feature, cell_active, feature_weight, part, loss_cta);
  stage2_gather_kernel<<<grid_for(G->N, 128), 128, 0, st>>>(G->N, G->g, G->ranges, G->off, G->lists, G->npairs,
                                                            part, rot, log_scale, logit_opacity, grad_pos, grad_rot,
                                                            grad_log_scale, grad_logit_opacity, grad_shs);
  ARAP_LAUNCH_CHECK();
  if (loss_host && G->nvalid > 0) {
    std::vector<float> h(2 * (size_t)G->nvalid);
    ARAP_CUDA_TRY(cudaMemcpyAsync(h.data(), loss_cta, h.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
    ARAP_CUDA_TRY(cudaStreamSynchronize(st));
    for (int v = 0; v < G->nvalid; ++v) {
      loss_host[0] += h[2 * (size_t)v];
      loss_host[1] += h[2 * (size_t)v + 1];
    }
  }
  return ARAP_OK;
}

extern "C" int arap_stage2_adam(int N, int step, const float* lr_host, const uint8_t* moved, float* logit_opacity,
                                float* shs, float* pos, float* rot, float* log_scale, const float* g_opacity,
                                const float* g_shs, const float* g_pos, const float* g_rot,
                                const float* g_log_scale, float* m, float* v, arap_stream_t stream) {
  if (N < 0 || step < 1 || !lr_host || !logit_opacity || !shs || !pos || !rot || !log_scale || !g_opacity ||
      !g_shs || !g_pos || !g_rot || !g_log_scale || !m || !v)
    return ARAP_EBADINPUT;
  if (N == 0) return ARAP_OK;
  Stage2Adam A;
  A.p[0] = logit_opacity; A.p[1] = shs; A.p[2] = pos; A.p[3] = rot; A.p[4] = log_scale;
  A.g[0] = g_opacity; A.g[1] = g_shs; A.g[2] = g_pos; A.g[3] = g_rot; A.g[4] = g_log_scale;
  for (int a = 0; a < 5; ++a) A.lr[a] = lr_host[a];
  const double b1 = 0.9, b2 = 0.999;
  const float bc1 = (float)(1.0 - std::pow(b1, step)), bc2 = (float)(1.0 - std::pow(b2, step));
  const long long total = (long long)N * kS2Params;
  stage2_adam_kernel<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(N, A, moved, m, v, (float)b1, (float)b2,
                                                                               1e-8f, bc1, bc2);
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

extern "C" int arap_stage2_cell_flags(const arap_grid* G, const float* aim_opacity, uint8_t* empty_out,
                                      uint8_t* converged_io, arap_stream_t stream) {
  if (!G || (!empty_out && !converged_io) || (empty_out && !aim_opacity)) return ARAP_EBADINPUT;
  if (G->nvalid == 0) return ARAP_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t cells = (size_t)G->g * G->g * G->g;
  uint8_t* map = nullptr;
  ARAP_CUDA_TRY(cudaMallocAsync(&map, cells, st));
  int rc = ARAP_OK;
  for (int mode = 0; mode < 2 && rc == ARAP_OK; ++mode) {
    uint8_t* out = mode == 0 ? empty_out : converged_io;
    if (!out) continue;
    if (cudaMemsetAsync(map, 0, cells, st) != cudaSuccess) {
      rc = ARAP_ECUDA;
      break;
    }
    cell_mark_kernel<<<grid_for(G->nvalid, 256), 256, 0, st>>>(G->nvalid, G->valid, G->g, mode, aim_opacity,
                                                                 converged_io, map);
    cell_flag_kernel<<<grid_for(G->nvalid, 256), 256, 0, st>>>(G->nvalid, G->valid, mode, map, out);
    if (cudaPeekAtLastError() != cudaSuccess) rc = ARAP_ECUDA;
  }
  cudaFreeAsync(map, st);
  return rc;
}

// ------------------------------------------- allocation-free centre order ----
// arap_grid_center_order_noalloc: the same kernel sequence as
// arap_grid_center_order with its scratch carved from one static device array
// of ARAP_CENTER_SCRATCH_BYTES instead of cudaMalloc/cudaFree.  Host code
// cannot use the array's name as a device address, so every call looks the
// address up with cudaGetSymbolAddress on the current device (a host-side
// query; the first one on a device loads the module there, so that first call
// should come before any stream capture).  Calls that overlap on the GPU
// share the array and race.
static __device__ __align__(256) unsigned char g_center_scratch[ARAP_CENTER_SCRATCH_BYTES];

namespace {
int center_scratch_base(unsigned char** out) {
  unsigned char* ptr = nullptr;
  if (cudaGetSymbolAddress((void**)&ptr, g_center_scratch) != cudaSuccess || !ptr) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  *out = ptr;
  return ARAP_OK;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
}  // namespace

extern "C" int arap_grid_center_order_noalloc(const arap_grid* G, int N, const float* pos, int32_t* order_out,
                                              arap_stream_t stream) {
  if (!G || !pos || !order_out || N < 1) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  const int C = G->g * G->g * G->g;
  const int nbs = (C + 1 + kScanTile - 1) / kScanTile + 1;
  // scratch: cell [N], count [C], cursor [C], off [C+1], flagpos [C+1],
  // valid [C], sums [nbs+1] (long long), each 256-byte aligned
  const size_t b_cell = align256(sizeof(int) * (size_t)N), b_cnt = align256(sizeof(int) * (size_t)C),
               b_off = align256(sizeof(int) * ((size_t)C + 1)), b_sums = align256(sizeof(long long) * (nbs + 1));
  const size_t need = b_cell + 3 * b_cnt + 2 * b_off + b_sums;
  if (need > (size_t)ARAP_CENTER_SCRATCH_BYTES) return ARAP_EUNSUPPORTED;
  unsigned char* base = nullptr;
  int rc = center_scratch_base(&base);
  if (rc != ARAP_OK) return rc;
  int* cell = reinterpret_cast<int*>(base);
  int* count = reinterpret_cast<int*>(base + b_cell);
  int* cursor = reinterpret_cast<int*>(base + b_cell + b_cnt);
  int* valid = reinterpret_cast<int*>(base + b_cell + 2 * b_cnt);
  int* off = reinterpret_cast<int*>(base + b_cell + 3 * b_cnt);
  int* flagpos = reinterpret_cast<int*>(base + b_cell + 3 * b_cnt + b_off);
  long long* sums = reinterpret_cast<long long*>(base + b_cell + 3 * b_cnt + 2 * b_off);
  // the per-cell counters start at zero; every other region is written
  // before it is read
  if (cudaMemsetAsync(count, 0, sizeof(int) * (size_t)C, st) || cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)C, st)) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  center_cell_kernel<<<grid_for(N, 256), 256, 0, st>>>(N, pos, G->params, cell, count);
  if ((rc = scan_exclusive(count, off, C, sums, st)) != ARAP_OK) return rc;
  center_fill_kernel<<<grid_for(N, 256), 256, 0, st>>>(N, cell, off, cursor, order_out);
  flags_kernel<<<grid_for(C, 256), 256, 0, st>>>(C, count, cursor);
  if ((rc = scan_exclusive(cursor, flagpos, C, sums, st)) != ARAP_OK) return rc;
  int nvalid = 0;
  if (cudaMemcpyAsync(&nvalid, flagpos + C, sizeof(int), cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st)) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  if (nvalid > 0) {
    compact_kernel<<<grid_for(C, 256), 256, 0, st>>>(C, count, flagpos, valid);
    // cells longer than the shared-memory sort take their merge scratch from
    // the rest of the static array
    auto alloc = [&](size_t bytes) -> void* {
      return need + bytes <= (size_t)ARAP_CENTER_SCRATCH_BYTES ? static_cast<void*>(base + need) : nullptr;
    };
    rc = sort_cell_lists(nvalid, valid, off, order_out, flagpos, count, cursor, alloc, ARAP_EUNSUPPORTED, st);
    if (rc != ARAP_OK) return rc;
  }
  if (cudaPeekAtLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ECUDA;
  }
  return ARAP_OK;
}
