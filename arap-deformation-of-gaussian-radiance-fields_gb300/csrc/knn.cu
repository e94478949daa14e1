// Brute-force kNN of points against the deformation nodes (sm_103a).
//
// Replaces DeformGraph::findNearestNodes / computeWeights (Deform.hpp:153-208)
// and the OpenMP loops of GaussianView::setupWeights* (GaussianView.cpp:
// 2818-2918).  One thread owns one point and keeps its K+1 best candidates in
// registers; the CTA streams the node set through shared memory in tiles.
// Distances are float32 sqrt((dx*dx+dy*dy)+dz*dz) rounded exactly as the
// reference's Pos arithmetic; the order is (distance, node index), which is the
// reference's order except for exactly equal distances.
#include "arap_common.cuh"

namespace arap {

constexpr int kKnnThreads = 256;  // default CTA size; 128 and 512 are built too
constexpr int kKnnTile = 2048;    // nodes per shared-memory tile (32 KB)

template <int KP1, int NT>
__global__ void __launch_bounds__(NT) knn_kernel(const float* __restrict__ pts, int P,
                                                          const float* __restrict__ nodes, int n,
                                                          int skip_first, int kout,
                                                          int32_t* __restrict__ idx_out,
                                                          float* __restrict__ w_out, int planes,
                                                          int* __restrict__ status) {
  __shared__ float4 s_nodes[kKnnTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < P;
  float px = 0.f, py = 0.f, pz = 0.f;
  if (active) {
    px = pts[3 * (size_t)i + 0];
    py = pts[3 * (size_t)i + 1];
    pz = pts[3 * (size_t)i + 2];
  }
  float bd2[KP1], bd[KP1];
  int bi[KP1];
#pragma unroll
  for (int j = 0; j < KP1; ++j) {
    bd2[j] = __int_as_float(0x7f800000);
    bd[j] = __int_as_float(0x7f800000);
    bi[j] = 0x7fffffff;
  }
  for (int base = 0; base < n; base += kKnnTile) {
    const int cnt = min(kKnnTile, n - base);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      const size_t g = 3 * (size_t)(base + t);
      s_nodes[t] = make_float4(nodes[g], nodes[g + 1], nodes[g + 2], 0.f);
    }
    __syncthreads();
    if (!active) continue;
    for (int t = 0; t < cnt; ++t) {
      const float4 q = s_nodes[t];
      const float d2 = dist2_rn(__fsub_rn(px, q.x), __fsub_rn(py, q.y), __fsub_rn(pz, q.z));
      if (d2 < bd2[KP1 - 1]) {
        const float d = __fsqrt_rn(d2);
        if (d < bd[KP1 - 1]) {
          // insert after every entry with distance <= d (their indices are lower)
          const int id = base + t;
#pragma unroll
          for (int j = KP1 - 1; j > 0; --j) {
            const bool shift = bd[j - 1] > d;
            const bool here = !shift && bd[j] > d;
            if (shift) {
              bd[j] = bd[j - 1];
              bd2[j] = bd2[j - 1];
              bi[j] = bi[j - 1];
            } else if (here) {
              bd[j] = d;
              bd2[j] = d2;
              bi[j] = id;
            }
          }
          if (bd[0] > d) {
            bd[0] = d;
            bd2[0] = d2;
            bi[0] = id;
          }
        }
      }
    }
  }
  if (!active) return;
  if (w_out == nullptr) {
    // graph: drop the first (self) entry, node-major rows
    for (int j = 0; j < kout; ++j) idx_out[(size_t)i * kout + j] = bi[j + skip_first];
    return;
  }
  // weights (Deform.hpp:196-207): w_j = (1 - d_j / d_k)^2, normalised, in float64
  const double dmax = (double)bd[KP1 - 1];
  double w[KP1 - 1];
  double sum = 0.0;
#pragma unroll
  for (int j = 0; j < KP1 - 1; ++j) {
    const double r = 1.0 - (double)bd[j] / dmax;
    w[j] = r * r;
    sum += w[j];
  }
  const bool bad = !(dmax > 0.0) || !(sum > 0.0);
  if (bad) raise_status(status, ARAP_ENONFINITE);
#pragma unroll
  for (int j = 0; j < KP1 - 1; ++j) {
    const double wj = (KP1 - 1 == 1) ? 1.0 : w[j] / sum;
    const size_t o = planes ? (size_t)j * P + i : (size_t)i * (KP1 - 1) + j;
    idx_out[o] = bi[j];
    w_out[o] = (float)wj;
  }
}

template <int KP1>
static int launch_knn(const float* pts, int P, const float* nodes, int n, int skip, int kout,
                      int32_t* idx, float* w, int planes, int* status, int threads, cudaStream_t st) {
  switch (threads) {
    case 128:
      knn_kernel<KP1, 128><<<grid_for(P, 128), 128, 0, st>>>(pts, P, nodes, n, skip, kout, idx, w, planes, status);
      break;
    case 512:
      knn_kernel<KP1, 512><<<grid_for(P, 512), 512, 0, st>>>(pts, P, nodes, n, skip, kout, idx, w, planes, status);
      break;
    default:
      knn_kernel<KP1, 256><<<grid_for(P, 256), 256, 0, st>>>(pts, P, nodes, n, skip, kout, idx, w, planes, status);
  }
  ARAP_LAUNCH_CHECK();
  return ARAP_OK;
}

static int dispatch_knn(int kp1, const float* pts, int P, const float* nodes, int n, int skip,
                        int kout, int32_t* idx, float* w, int planes, int* status, int threads,
                        cudaStream_t st) {
  switch (kp1) {
#define ARAP_KNN_CASE(K) \
  case K:                \
    return launch_knn<K>(pts, P, nodes, n, skip, kout, idx, w, planes, status, threads, st);
    ARAP_KNN_CASE(2)
    ARAP_KNN_CASE(3)
    ARAP_KNN_CASE(4)
    ARAP_KNN_CASE(5)
    ARAP_KNN_CASE(6)
    ARAP_KNN_CASE(7)
    ARAP_KNN_CASE(8)
    ARAP_KNN_CASE(9)
    ARAP_KNN_CASE(10)
    ARAP_KNN_CASE(11)
    ARAP_KNN_CASE(12)
    ARAP_KNN_CASE(13)
#undef ARAP_KNN_CASE
    default:
      return ARAP_EUNSUPPORTED;
  }
}

}  // namespace arap

using namespace arap;

extern "C" int arap_build_graph(const float* nodes_xyz, int n, int k, int32_t* neighbors_out,
                                arap_stream_t stream) {
  if (!nodes_xyz || !neighbors_out || k < 1 || n < k + 1) return ARAP_EBADINPUT;
  if (k > ARAP_KNN_MAX) return ARAP_EUNSUPPORTED;
  return dispatch_knn(k + 1, nodes_xyz, n, nodes_xyz, n, 1, k, neighbors_out, nullptr, 0, nullptr, kKnnThreads,
                      (cudaStream_t)stream);
}

extern "C" int arap_compute_weights_ex(const float* points_xyz, int P, const float* nodes_xyz, int n, int k,
                                       int threads, int32_t* idx_out, float* w_out, int32_t* status,
                                       arap_stream_t stream) {
  if (P == 0) return ARAP_OK;
  if (!points_xyz || !nodes_xyz || !idx_out || !w_out || P < 0 || k < 1 || n < k + 1)
    return ARAP_EBADINPUT;
  if (threads != 0 && threads != 128 && threads != 256 && threads != 512) return ARAP_EBADINPUT;
  if (k > ARAP_KNN_MAX) return ARAP_EUNSUPPORTED;
  return dispatch_knn(k + 1, points_xyz, P, nodes_xyz, n, 0, k, idx_out, w_out, 1, status,
                      threads ? threads : kKnnThreads, (cudaStream_t)stream);
}

extern "C" int arap_compute_weights(const float* points_xyz, int P, const float* nodes_xyz, int n,
                                    int k, int32_t* idx_out, float* w_out, int32_t* status,
                                    arap_stream_t stream) {
  return arap_compute_weights_ex(points_xyz, P, nodes_xyz, n, k, 0, idx_out, w_out, status, stream);
}

extern "C" int arap_knn_autotune(const float* points_xyz, int P, const float* nodes_xyz, int n, int k,
                                 int* threads_out, float* ms_out, arap_stream_t stream) {
  if (!threads_out || !points_xyz || !nodes_xyz || P < 1 || k < 1 || n < k + 1) return ARAP_EBADINPUT;
  if (k > ARAP_KNN_MAX) return ARAP_EUNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  // a bounded sample: the first points (the work per point is the same)
  const int S = P < (1 << 18) ? P : (1 << 18);
  void* buf = nullptr;
  if (cudaMalloc(&buf, (size_t)S * k * 8 + sizeof(int)) != cudaSuccess) {
    (void)cudaGetLastError();
    return ARAP_ENOMEM;
  }
  int32_t* idx = static_cast<int32_t*>(buf);
  float* w = reinterpret_cast<float*>(idx + (size_t)S * k);
  int* word = reinterpret_cast<int*>(w + (size_t)S * k);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = cudaMemsetAsync(word, 0, sizeof(int), st) == cudaSuccess ? ARAP_OK : ARAP_ECUDA;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = ARAP_ECUDA;
  const int cand[3] = {128, 256, 512};
  float best = 0.f;
  *threads_out = kKnnThreads;
  for (int c = 0; c < 3 && rc == ARAP_OK; ++c) {
    float ms = 0.f;
    for (int rep = 0; rep < 2 && rc == ARAP_OK; ++rep) {  // the first run warms up
      if (cudaEventRecord(e0, st) != cudaSuccess) rc = ARAP_ECUDA;
      if (rc == ARAP_OK)
        rc = dispatch_knn(k + 1, points_xyz, S, nodes_xyz, n, 0, k, idx, w, 1, word, cand[c], st);
      if (rc == ARAP_OK && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = ARAP_ECUDA;
    }
    if (rc != ARAP_OK) break;
    if (ms_out) ms_out[c] = ms;
    if (c == 0 || ms < best) {
      best = ms;
      *threads_out = cand[c];
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc != ARAP_OK) (void)cudaGetLastError();
  cudaFree(buf);
  return rc;
}
