// Headless rasteriser of the deformed Gaussians (sm_103a): the published 3D
// Gaussian splatting forward (Kerbl et al. 2023; EWA splatting, Zwicker et
// al. 2002) into a device image, standing in for the un-vendored
// CudaRasterizer::forward the viewer draws with (GaussianView.cpp:1066-1127).
// The window and the GL interop are replaced by the image array.
//
// Per Gaussian (raster_preprocess_kernel):
// - culled when its camera depth is at most 0.2;
// - 2D covariance J W Sigma W^T J^T + 0.3 I, with x/z and y/z clamped to
//   1.3 tan(fov/2) before J is formed;
// - radius ceil(3 sqrt(largest eigenvalue)), discriminant floored at 0.1;
// - colour = SH value in direction (mu - campos)/|mu - campos| + 0.5,
//   clamped at 0;
// - the 16x16 tiles of its radius square.
// Tile lists: a count per tile, a scan, an atomic fill.  raster_tile_kernel,
// one CTA of 256 threads per tile (one per pixel): the tile's list, keyed by
// (depth bits, Gaussian index), is bitonic-sorted in shared memory, so the
// order is deterministic; a list longer than kMaxTileList is sorted before by
// raster_sort_long_kernel (chunk sorts and merges through global scratch) and
// read from global memory.  Then the Gaussians are composited front to back
// in batches staged in shared memory:
// - alpha = min(0.99, o exp(power)); a term with power > 0 or alpha < 1/255
//   is skipped;
// - compositing stops before T would drop below 1e-4;
// - out = sum c alpha T + T bg.
// The SH basis is the real basis with the Condon-Shortley phase, which
// matches the SH rotation of the skinning kernels.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "arap_common.cuh"

namespace arap {

constexpr int kTile = 16;
constexpr int kMaxTileList = 16384;  // sort keys per tile held in shared memory (128 KB)

// Tiles with more than kMaxTileList entries, one CTA each: their key runs
// sorted in place (keys are distinct: the Gaussian index is in the low bits).
__global__ void __launch_bounds__(1024) raster_sort_long_kernel(int nlong, const int* __restrict__ long_tiles,
                                                                const int* __restrict__ tile_off,
                                                                const int* __restrict__ tile_count,
                                                                unsigned long long* keys,
                                                                unsigned long long* scratch,
                                                                const long long* __restrict__ scratch_off) {
  extern __shared__ unsigned long long s_sort[];
  const int k = blockIdx.x;
  if (k >= nlong) return;
  const int t = long_tiles[k];
  cta_sort_distinct<unsigned long long, kMaxTileList>(keys + tile_off[t], scratch + scratch_off[k], tile_count[t],
                                                      ~0ull, s_sort);
}

struct RasterCam {
  float view[16];  // row-major, world -> camera
  float proj[16];  // row-major, world -> clip
  float campos[3];
  float tanx, tany, fx, fy;
  int width, height, gx, gy;
  float scale_modifier;
  int sh_degree;
};

// Real SH with the Condon-Shortley phase, degree <= 3, at unit direction
// (x, y, z); the constants are the normalisations sqrt((2l+1)/(4 pi) *
// (l-|m|)!/(l+|m|)!) (times sqrt(2) for m != 0) of the Cartesian forms.
__device__ __forceinline__ void sh_basis16(float x, float y, float z, int degree, float* B) {
  const float pi = 3.14159265358979323846f;
  B[0] = 0.5f * sqrtf(1.0f / pi);
  if (degree < 1) return;
  const float c1 = sqrtf(3.0f / (4.0f * pi));
  B[1] = -c1 * y;
  B[2] = c1 * z;
  B[3] = -c1 * x;
  if (degree < 2) return;
  const float c2 = 0.5f * sqrtf(15.0f / pi), c20 = 0.25f * sqrtf(5.0f / pi);
  B[4] = c2 * x * y;
  B[5] = -c2 * y * z;
  B[6] = c20 * (2.f * z * z - x * x - y * y);
  B[7] = -c2 * x * z;
  B[8] = 0.5f * c2 * (x * x - y * y);
  if (degree < 3) return;
  const float c33 = 0.25f * sqrtf(35.0f / (2.0f * pi)), c32 = 0.5f * sqrtf(105.0f / pi);
  const float c31 = 0.25f * sqrtf(21.0f / (2.0f * pi)), c30 = 0.25f * sqrtf(7.0f / pi);
  const float xx = x * x, yy = y * y, zz = z * z;
  B[9] = -c33 * y * (3.f * xx - yy);
  B[10] = c32 * x * y * z;
  B[11] = -c31 * y * (4.f * zz - xx - yy);
  B[12] = c30 * z * (2.f * zz - 3.f * xx - 3.f * yy);
  B[13] = -c31 * x * (4.f * zz - xx - yy);
  B[14] = 0.5f * c32 * z * (xx - yy);
  B[15] = -c33 * x * (xx - 3.f * yy);
}

__global__ void raster_preprocess_kernel(int N, const float* __restrict__ pos, const float* __restrict__ shs,
                                         const float* __restrict__ opacity, const float* __restrict__ scale,
                                         const float* __restrict__ rot, RasterCam cam, float* __restrict__ xy,
                                         float* __restrict__ conic_op, float* __restrict__ color,
                                         float* __restrict__ depth, int* __restrict__ rect,
                                         int* __restrict__ tile_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  rect[4 * (size_t)i] = rect[4 * (size_t)i + 1] = rect[4 * (size_t)i + 2] = rect[4 * (size_t)i + 3] = 0;
  const float px = pos[3 * (size_t)i], py = pos[3 * (size_t)i + 1], pz = pos[3 * (size_t)i + 2];
  const float* V = cam.view;
  const float vx = V[0] * px + V[1] * py + V[2] * pz + V[3];
  const float vy = V[4] * px + V[5] * py + V[6] * pz + V[7];
  const float vz = V[8] * px + V[9] * py + V[10] * pz + V[11];
  depth[i] = vz;
  if (!(vz > 0.2f)) return;
  const float* Pm = cam.proj;
  const float cx = Pm[0] * px + Pm[1] * py + Pm[2] * pz + Pm[3];
  const float cy = Pm[4] * px + Pm[5] * py + Pm[6] * pz + Pm[7];
  const float cw = Pm[12] * px + Pm[13] * py + Pm[14] * pz + Pm[15];
  const float iw = 1.0f / (cw + 1e-7f);
  const float nx = cx * iw, ny = cy * iw;
  // 3D covariance
  float R[9];
  quat_to_rowmajor(quat_normalize(__ldg(reinterpret_cast<const float4*>(rot) + i)), R);
  float s2[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float sv = cam.scale_modifier * scale[3 * (size_t)i + d];
    s2[d] = sv * sv;
  }
  float S[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q)
      S[r * 3 + q] = R[r * 3] * s2[0] * R[q * 3] + R[r * 3 + 1] * s2[1] * R[q * 3 + 1] + R[r * 3 + 2] * s2[2] * R[q * 3 + 2];
  // EWA projection
  const float limx = 1.3f * cam.tanx, limy = 1.3f * cam.tany;
  const float tx = fminf(limx, fmaxf(-limx, vx / vz)) * vz;
  const float ty = fminf(limy, fmaxf(-limy, vy / vz)) * vz;
  const float j00 = cam.fx / vz, j02 = -cam.fx * tx / (vz * vz);
  const float j11 = cam.fy / vz, j12 = -cam.fy * ty / (vz * vz);
  float T[6];  // rows 0, 1 of J W
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T[k] = j00 * V[k] + j02 * V[8 + k];
    T[3 + k] = j11 * V[4 + k] + j12 * V[8 + k];
  }
  float TS[6];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      TS[r * 3 + k] = T[r * 3] * S[k] + T[r * 3 + 1] * S[3 + k] + T[r * 3 + 2] * S[6 + k];
  const float a = TS[0] * T[0] + TS[1] * T[1] + TS[2] * T[2] + 0.3f;
  const float b = TS[0] * T[3] + TS[1] * T[4] + TS[2] * T[5];
  const float c = TS[3] * T[3] + TS[4] * T[4] + TS[5] * T[5] + 0.3f;
  const float det = a * c - b * b;
  if (det == 0.f) return;
  const float idet = 1.0f / det;
  const float mid = 0.5f * (a + c);
  const float root = sqrtf(fmaxf(0.1f, mid * mid - det));
  const float radius = ceilf(3.0f * sqrtf(fmaxf(mid + root, mid - root)));
  const float mx = ((nx + 1.0f) * cam.width - 1.0f) * 0.5f;
  const float my = ((ny + 1.0f) * cam.height - 1.0f) * 0.5f;
  const int x0 = min(cam.gx, max(0, (int)((mx - radius) / kTile)));
  const int y0 = min(cam.gy, max(0, (int)((my - radius) / kTile)));
  const int x1 = min(cam.gx, max(0, (int)((mx + radius + kTile - 1) / kTile)));
  const int y1 = min(cam.gy, max(0, (int)((my + radius + kTile - 1) / kTile)));
  if ((x1 - x0) * (y1 - y0) <= 0) return;
  // colour
  float dx = px - cam.campos[0], dy = py - cam.campos[1], dz = pz - cam.campos[2];
  const float il = rsqrtf(dx * dx + dy * dy + dz * dz);
  dx *= il;
  dy *= il;
  dz *= il;
  float B[16];
  sh_basis16(dx, dy, dz, cam.sh_degree, B);
  const int K = (cam.sh_degree + 1) * (cam.sh_degree + 1);
  const float* sh = shs + 48 * (size_t)i;
  float col[3] = {0.f, 0.f, 0.f};
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) col[ch] = fmaf(B[k], sh[3 * k + ch], col[ch]);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) color[3 * (size_t)i + ch] = fmaxf(col[ch] + 0.5f, 0.f);
  xy[2 * (size_t)i] = mx;
  xy[2 * (size_t)i + 1] = my;
  conic_op[4 * (size_t)i] = c * idet;
  conic_op[4 * (size_t)i + 1] = -b * idet;
  conic_op[4 * (size_t)i + 2] = a * idet;
  conic_op[4 * (size_t)i + 3] = opacity[i];
  rect[4 * (size_t)i] = x0;
  rect[4 * (size_t)i + 1] = y0;
  rect[4 * (size_t)i + 2] = x1;
  rect[4 * (size_t)i + 3] = y1;
  for (int ty2 = y0; ty2 < y1; ++ty2)
    for (int tx2 = x0; tx2 < x1; ++tx2) atomicAdd(tile_count + ty2 * cam.gx + tx2, 1);
}

// Exclusive scan of the tile counts in one CTA of 1024 threads (the tile
// count of an image is small); total_out[0] = the sum.
__global__ void __launch_bounds__(1024) raster_scan_kernel(int n, const int* __restrict__ in,
                                                           int* __restrict__ out, int* __restrict__ total_out) {
  __shared__ int s_warp[32];
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    int x = v;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = s_warp[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      s_warp[lane] = t;
    }
    __syncthreads();
    const int incl = x + (w > 0 ? s_warp[w - 1] : 0);
    if (i < n) out[i] = s_carry + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry += incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) total_out[0] = s_carry;
}

__global__ void raster_fill_kernel(int N, const int* __restrict__ rect, const float* __restrict__ depth, int gx,
                                   const int* __restrict__ tile_off, int* __restrict__ cursor,
                                   unsigned long long* __restrict__ keys) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int* r = rect + 4 * (size_t)i;
  if ((r[2] - r[0]) * (r[3] - r[1]) <= 0) return;
  const unsigned long long key =
      ((unsigned long long)__float_as_uint(depth[i]) << 32) | (unsigned long long)(unsigned int)i;
  for (int ty = r[1]; ty < r[3]; ++ty)
    for (int tx = r[0]; tx < r[2]; ++tx) {
      const int t = ty * gx + tx;
      const int slot = atomicAdd(cursor + t, 1);
      keys[(size_t)tile_off[t] + slot] = key;
    }
}

__global__ void __launch_bounds__(256) raster_tile_kernel(
    RasterCam cam, const int* __restrict__ tile_off, const int* __restrict__ tile_count,
    const unsigned long long* __restrict__ keys, const float* __restrict__ xy, const float* __restrict__ conic_op,
    const float* __restrict__ color, float bg0, float bg1, float bg2, float* __restrict__ image,
    float* __restrict__ final_t, int* __restrict__ n_contrib) {
  extern __shared__ unsigned long long s_keys[];
  __shared__ float s_xy[256][2];
  __shared__ float s_co[256][4];
  __shared__ float s_col[256][3];
  const int tile = blockIdx.x;
  const int tx = tile % cam.gx, ty = tile / cam.gx;
  const int n = tile_count[tile];
  const int off = tile_off[tile];
  // a long list was sorted in global memory before; a short one is
  // bitonic-sorted here, padded to a power of two with ~0
  const bool long_list = n > kMaxTileList;
  const unsigned long long* sorted = long_list ? keys + off : s_keys;
  if (!long_list) {
    int m = 1;
    while (m < n) m <<= 1;
    for (int t = threadIdx.x; t < m; t += 256) s_keys[t] = t < n ? keys[(size_t)off + t] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = threadIdx.x; t < m; t += 256) {
          const int u = t ^ j;
          if (u > t) {
            const unsigned long long a = s_keys[t], b = s_keys[u];
            const bool up = (t & k) == 0;
            if ((a > b) == up) {
              s_keys[t] = b;
              s_keys[u] = a;
            }
          }
        }
        __syncthreads();
      }
  }
  // front-to-back compositing, one thread per pixel
  const int px = tx * kTile + (threadIdx.x % kTile), py = ty * kTile + (threadIdx.x / kTile);
  const bool inside = px < cam.width && py < cam.height;
  bool done = !inside;
  float T = 1.f, C0 = 0.f, C1 = 0.f, C2 = 0.f;
  int contrib = 0;
  for (int base = 0; base < n; base += 256) {
    if (__syncthreads_and(done)) break;
    const int q = base + threadIdx.x;
    if (q < n) {
      const int gi = (int)(unsigned int)(sorted[q] & 0xffffffffull);
      s_xy[threadIdx.x][0] = xy[2 * (size_t)gi];
      s_xy[threadIdx.x][1] = xy[2 * (size_t)gi + 1];
#pragma unroll
      for (int h = 0; h < 4; ++h) s_co[threadIdx.x][h] = conic_op[4 * (size_t)gi + h];
#pragma unroll
      for (int h = 0; h < 3; ++h) s_col[threadIdx.x][h] = color[3 * (size_t)gi + h];
    }
    __syncthreads();
    const int cnt = min(256, n - base);
    for (int j = 0; j < cnt && !done; ++j) {
      const float dx = s_xy[j][0] - (float)px, dy = s_xy[j][1] - (float)py;
      const float power = -0.5f * (s_co[j][0] * dx * dx + s_co[j][2] * dy * dy) - s_co[j][1] * dx * dy;
      if (power > 0.f) continue;
      const float alpha = fminf(0.99f, s_co[j][3] * __expf(power));
      if (alpha < 1.0f / 255.0f) continue;
      const float tn = T * (1.f - alpha);
      if (tn < 1e-4f) {
        done = true;
        break;
      }
      C0 = fmaf(s_col[j][0], alpha * T, C0);
      C1 = fmaf(s_col[j][1], alpha * T, C1);
      C2 = fmaf(s_col[j][2], alpha * T, C2);
      T = tn;
      ++contrib;
    }
  }
  if (inside) {
    const size_t pix = (size_t)py * cam.width + px, hw = (size_t)cam.width * cam.height;
    image[pix] = C0 + T * bg0;
    image[hw + pix] = C1 + T * bg1;
    image[2 * hw + pix] = C2 + T * bg2;
    if (final_t) final_t[pix] = T;
    if (n_contrib) n_contrib[pix] = contrib;
  }
}

}  // namespace arap

using namespace arap;

extern "C" int arap_render(int N, const float* pos, const float* shs, const float* opacity, const float* scale,
                           const float* rot, float scale_modifier, int sh_degree, const float* view_host,
                           const float* proj_host, const float* campos_host, float tan_fovx, float tan_fovy,
                           int width, int height, const float* background_host, float* image_out,
                           float* final_t_out, int32_t* n_contrib_out, arap_stream_t stream) {
  if (N < 0 || width <= 0 || height <= 0 || sh_degree < 0 || sh_degree > 3 || !view_host || !proj_host ||
      !campos_host || !background_host || !image_out || !(tan_fovx > 0.f) || !(tan_fovy > 0.f))
    return ARAP_EBADINPUT;
  if (N > 0 && (!pos || !shs || !opacity || !scale || !rot)) return ARAP_EBADINPUT;
  if (reinterpret_cast<uintptr_t>(rot) & 15) return ARAP_EBADINPUT;
  cudaStream_t st = (cudaStream_t)stream;
  RasterCam cam;
  for (int k = 0; k < 16; ++k) {
    cam.view[k] = view_host[k];
    cam.proj[k] = proj_host[k];
  }
  for (int k = 0; k < 3; ++k) cam.campos[k] = campos_host[k];
  cam.tanx = tan_fovx;
  cam.tany = tan_fovy;
  cam.fx = width / (2.0f * tan_fovx);
  cam.fy = height / (2.0f * tan_fovy);
  cam.width = width;
  cam.height = height;
  cam.gx = (width + kTile - 1) / kTile;
  cam.gy = (height + kTile - 1) / kTile;
  cam.scale_modifier = scale_modifier;
  cam.sh_degree = sh_degree;
  const int tiles = cam.gx * cam.gy;
  const size_t n = (size_t)std::max(N, 1);
  // scratch: xy 2 | conic+opacity 4 | colour 3 | depth 1 floats and rect 4 ints
  // per Gaussian; count, offset, cursor per tile; the total
  char* scratch = nullptr;
  const size_t bytes_g = n * (10 * sizeof(float) + 4 * sizeof(int));
  const size_t bytes_t = (size_t)tiles * 3 * sizeof(int) + sizeof(int);
  ARAP_CUDA_TRY(cudaMallocAsync(&scratch, bytes_g + bytes_t, st));
  float* xy = reinterpret_cast<float*>(scratch);
  float* co = xy + 2 * n;
  float* col = co + 4 * n;
  float* dep = col + 3 * n;
  int* rect = reinterpret_cast<int*>(dep + n);
  int* tcount = rect + 4 * n;
  int* toff = tcount + tiles;
  int* tcur = toff + tiles;
  int* total = tcur + tiles;
  int rc = ARAP_OK;
  int h_total = 0;
  unsigned long long* keys = nullptr;
  cudaMemsetAsync(tcount, 0, (size_t)tiles * sizeof(int), st);
  cudaMemsetAsync(tcur, 0, (size_t)tiles * sizeof(int), st);
  if (N > 0)
    raster_preprocess_kernel<<<(N + 127) / 128, 128, 0, st>>>(N, pos, shs, opacity, scale, rot, cam, xy, co, col,
                                                              dep, rect, tcount);
  raster_scan_kernel<<<1, 1024, 0, st>>>(tiles, tcount, toff, total);
  if (cudaPeekAtLastError() != cudaSuccess) rc = ARAP_ECUDA;
  if (rc == ARAP_OK && cudaMemcpyAsync(&h_total, total, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    rc = ARAP_ECUDA;
  if (rc == ARAP_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = ARAP_ECUDA;
  if (rc == ARAP_OK && cudaMallocAsync(&keys, sizeof(unsigned long long) * (size_t)std::max(h_total, 1), st) !=
                           cudaSuccess)
    rc = ARAP_ENOMEM;
  // tiles whose lists exceed the shared-memory sort: sorted in global memory
  std::vector<int> long_tiles;
  std::vector<long long> long_off(1, 0);
  const size_t smem = sizeof(unsigned long long) * kMaxTileList;
  if (rc == ARAP_OK && h_total > kMaxTileList) {
    std::vector<int> cnt(tiles);
    if (cudaMemcpyAsync(cnt.data(), tcount, sizeof(int) * (size_t)tiles, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = ARAP_ECUDA;
    for (int t = 0; rc == ARAP_OK && t < tiles; ++t)
      if (cnt[t] > kMaxTileList) {
        long_tiles.push_back(t);
        long_off.push_back(long_off.back() + cnt[t]);
      }
  }
  // set on every call, so that every device the caller renders on has them
  if (rc == ARAP_OK && (cudaFuncSetAttribute(raster_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem) != cudaSuccess ||
                        cudaFuncSetAttribute(raster_sort_long_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem) != cudaSuccess)) {
    (void)cudaGetLastError();
    rc = ARAP_ECUDA;
  }
  char* long_scratch = nullptr;
  if (rc == ARAP_OK) {
    if (N > 0)
      raster_fill_kernel<<<(N + 127) / 128, 128, 0, st>>>(N, rect, dep, cam.gx, toff, tcur, keys);
    if (!long_tiles.empty()) {
      const int nl = (int)long_tiles.size();
      const size_t b_ids = ((sizeof(int) * (size_t)nl) + 15) & ~size_t(15);
      const size_t b_off = sizeof(long long) * ((size_t)nl + 1);
      const size_t bytes = b_ids + b_off + sizeof(unsigned long long) * (size_t)long_off.back();
      if (cudaMallocAsync(&long_scratch, bytes, st) != cudaSuccess) {
        (void)cudaGetLastError();
        long_scratch = nullptr;
        rc = ARAP_ENOMEM;
      } else {
        int* d_ids = reinterpret_cast<int*>(long_scratch);
        long long* d_off = reinterpret_cast<long long*>(long_scratch + b_ids);
        unsigned long long* d_keys = reinterpret_cast<unsigned long long*>(long_scratch + b_ids + b_off);
        if (cudaMemcpyAsync(d_ids, long_tiles.data(), sizeof(int) * (size_t)nl, cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(d_off, long_off.data(), b_off, cudaMemcpyHostToDevice, st) != cudaSuccess)
          rc = ARAP_ECUDA;
        else
          raster_sort_long_kernel<<<nl, 1024, smem, st>>>(nl, d_ids, toff, tcount, keys, d_keys, d_off);
      }
    }
  }
  if (rc == ARAP_OK) {
    const float* bg = background_host;
    raster_tile_kernel<<<tiles, 256, smem, st>>>(cam, toff, tcount, keys, xy, co, col, bg[0], bg[1], bg[2],
                                                image_out, final_t_out, n_contrib_out);
    if (cudaPeekAtLastError() != cudaSuccess) rc = ARAP_ECUDA;
    if (rc == ARAP_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = ARAP_ECUDA;
  }
  if (long_scratch) cudaFreeAsync(long_scratch, st);
  if (keys) cudaFreeAsync(keys, st);
  cudaFreeAsync(scratch, st);
  return rc;
}
