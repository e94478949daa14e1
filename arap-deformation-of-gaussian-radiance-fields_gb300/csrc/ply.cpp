// 3D Gaussian splatting binary PLY files: load into the activated SoA arrays
// the deformation path works on, and save them back (the reference viewer's
// loadPly / loadPly_Origin / savePly, GaussianView.cpp:43-339).  Host code
// only: nothing here touches the device, so it runs without a GPU.
//
// Loading (GaussianView.cpp:43-147, 149-262):
// - the vertex records are read as float properties in header order; the
//   standard 3DGS layout is x y z, nx ny nz, f_dc_0..2, f_rest_0..3*(K-1)-1
//   (channel-major), opacity, scale_0..2, rot_0..3 with K = (D+1)^2 SH
//   coefficients, and optionally `index` (the viewer's "soup" files);
// - the splats are reordered by a 63-bit Morton code of their position in
//   the bounding box (21 bits per axis, x in bit 3i, y in 3i+1, z in 3i+2),
//   ties kept in file order;
// - quaternions are normalised, scales exponentiated, opacities passed
//   through the logistic function; SH coefficients are interleaved per
//   coefficient (rgb) into 48 floats, the bands above D left zero;
// - the file's `index` property, when present, is rounded to an integer.
// The file read, the Morton codes and the per-splat decode run on up to 16
// host threads over fixed contiguous ranges, and the Morton order is a
// stable radix sort, so the result does not depend on the thread count.
// Saving (GaussianView.cpp:264-339): splats outside the box [box_min,
// box_max] or flagged too small are dropped; scales are stored as logs,
// opacities as logits, quaternions as given, normals as zero, SH degree 3.
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/arap_gb300.h"

namespace {

constexpr int kShFloats = 48;  // degree-3 SH, rgb per coefficient

struct PlyLayout {
  long long count = -1;
  std::vector<std::string> props;  // float properties of a vertex, in order
  std::streamoff data_start = 0;
  int sh_degree = -1;
  bool has_index = false;
  int at(const std::string& name) const {
    for (size_t i = 0; i < props.size(); ++i)
      if (props[i] == name) return (int)i;
    return -1;
  }
};

bool little_endian_host() {
  const uint32_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

// Header of a binary little-endian PLY whose only element is `vertex` with
// float properties.  Returns ARAP_OK or ARAP_EBADINPUT.
int read_layout(std::ifstream& in, PlyLayout& L) {
  std::string line;
  if (!std::getline(in, line) || line.rfind("ply", 0) != 0) return ARAP_EBADINPUT;
  bool format_ok = false, in_vertex = false;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ss(line);
    std::string word;
    ss >> word;
    if (word == "end_header") {
      L.data_start = in.tellg();
      break;
    }
    if (word == "format") {
      std::string kind;
      ss >> kind;
      format_ok = kind == "binary_little_endian";
    } else if (word == "element") {
      std::string name;
      long long n = -1;
      ss >> name >> n;
      if (name != "vertex" || n < 0 || L.count >= 0) return ARAP_EBADINPUT;
      L.count = n;
      in_vertex = true;
    } else if (word == "property") {
      std::string type, name;
      ss >> type >> name;
      if (!in_vertex || type != "float" || name.empty()) return ARAP_EBADINPUT;
      L.props.push_back(name);
    } else if (word != "comment" && word != "obj_info" && !word.empty()) {
      return ARAP_EBADINPUT;
    }
  }
  if (!format_ok || L.count < 0 || L.data_start <= 0) return ARAP_EBADINPUT;
  // the fields the deformation path needs
  static const char* required[] = {"x", "y", "z", "f_dc_0", "f_dc_1", "f_dc_2", "opacity",
                                   "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"};
  for (const char* r : required)
    if (L.at(r) < 0) return ARAP_EBADINPUT;
  int rest = 0;
  while (L.at("f_rest_" + std::to_string(rest)) >= 0) ++rest;
  switch (rest) {
    case 0: L.sh_degree = 0; break;
    case 9: L.sh_degree = 1; break;
    case 24: L.sh_degree = 2; break;
    case 45: L.sh_degree = 3; break;
    default: return ARAP_EBADINPUT;
  }
  L.has_index = L.at("index") >= 0;
  return ARAP_OK;
}

int open_layout(const char* path, std::ifstream& in, PlyLayout& L) {
  if (!path) return ARAP_EBADINPUT;
  in.open(path, std::ios_base::binary);
  if (!in.good()) return ARAP_EBADINPUT;
  return read_layout(in, L);
}

// Morton code of a position in the box (the viewer's 21-bit quantisation:
// float relative position times 2^21 - 1, truncated).  A flat axis (hi ==
// lo, where the viewer divides by zero) quantises to 0.
uint64_t morton_code(const float* p, const float* lo, const float* hi) {
  uint64_t code = 0;
  uint32_t q[3];
  for (int a = 0; a < 3; ++a) {
    const float rel = hi[a] > lo[a] ? (p[a] - lo[a]) / (hi[a] - lo[a]) : 0.f;
    const float scaled = float((1 << 21) - 1) * rel;
    q[a] = (uint32_t)(int)scaled;
  }
  for (int bit = 0; bit < 21; ++bit)
    for (int a = 0; a < 3; ++a) code |= (uint64_t)((q[a] >> bit) & 1u) << (3 * bit + a);
  return code;
}

// Host threads for the per-splat loops: up to 16, one per 16k splats.
int worker_count(size_t n) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t by_size = n / 16384 + 1;
  return (int)std::min<size_t>(std::min<size_t>(hw, 16), by_size);
}

// Runs f(thread, begin, end) over nt contiguous chunks of [0, n); chunk t
// always covers the same range, so per-thread partial results are
// deterministic.
template <class F>
void parallel_chunks(size_t n, int nt, F f) {
  if (nt <= 1) {
    f(0, 0, n);
    return;
  }
  std::vector<std::thread> pool;
  pool.reserve(nt - 1);
  for (int t = 1; t < nt; ++t)
    pool.emplace_back([&f, t, n, nt] { f(t, n * t / nt, n * (t + 1) / nt); });
  f(0, 0, n / nt);
  for (auto& th : pool) th.join();
}

// Stable LSD radix sort of `order` by `key` (both permuted together), 16-bit
// digits; digits that are equal for every key are skipped.
void radix_sort_stable(std::vector<uint64_t>& key, std::vector<uint32_t>& order) {
  const size_t n = key.size();
  std::vector<uint64_t> k2(n);
  std::vector<uint32_t> o2(n);
  std::vector<size_t> count(65537);
  for (int shift = 0; shift < 64; shift += 16) {
    std::fill(count.begin(), count.end(), 0);
    for (size_t i = 0; i < n; ++i) ++count[((key[i] >> shift) & 0xffffu) + 1];
    if (count[((key[0] >> shift) & 0xffffu) + 1] == n) continue;
    for (size_t d = 1; d < count.size(); ++d) count[d] += count[d - 1];
    for (size_t i = 0; i < n; ++i) {
      const size_t dst = count[(key[i] >> shift) & 0xffffu]++;
      k2[dst] = key[i];
      o2[dst] = order[i];
    }
    key.swap(k2);
    order.swap(o2);
  }
}

// Reads [offset, offset + bytes) of the file into dst with nt threads, each
// issuing pread on its own contiguous range.  A read a signal interrupts
// (EINTR) is retried; false on end of file or any other error.
bool read_parallel(const char* path, size_t offset, char* dst, size_t bytes, int nt) {
  const int fd = ::open(path, O_RDONLY);
  if (fd < 0) return false;
  std::atomic<bool> ok{true};
  parallel_chunks(bytes, nt, [&](int, size_t b, size_t e) {
    size_t done = b;
    while (done < e) {
      const ssize_t r = ::pread(fd, dst + done, e - done, (off_t)(offset + done));
      if (r < 0 && errno == EINTR) continue;
      if (r <= 0) {
        ok = false;
        return;
      }
      done += (size_t)r;
    }
  });
  ::close(fd);
  return ok.load();
}

}  // namespace

extern "C" int arap_ply_info(const char* path, int64_t* count, int* sh_degree, int* has_index) {
  if (!count || !sh_degree || !has_index) return ARAP_EBADINPUT;
  std::ifstream in;
  PlyLayout L;
  const int rc = open_layout(path, in, L);
  if (rc != ARAP_OK) return rc;
  *count = (int64_t)L.count;
  *sh_degree = L.sh_degree;
  *has_index = L.has_index ? 1 : 0;
  return ARAP_OK;
}

extern "C" int arap_ply_load(const char* path, int64_t count, int morton_order, float* pos, float* shs,
                             float* opacity, float* scale, float* rot, float* box_min, float* box_max,
                             int32_t* index) {
  if (!little_endian_host()) return ARAP_EUNSUPPORTED;
  if (!pos || !shs || !opacity || !scale || !rot || count < 0) return ARAP_EBADINPUT;
  std::ifstream in;
  PlyLayout L;
  int rc = open_layout(path, in, L);
  if (rc != ARAP_OK) return rc;
  if (count != (int64_t)L.count || (index && !L.has_index)) return ARAP_EBADINPUT;
  const size_t P = L.props.size(), N = (size_t)L.count;
  if (N > (size_t)UINT32_MAX) return ARAP_EUNSUPPORTED;
  // the records, read by several threads at once (uninitialised buffer: every
  // byte is read or the call fails)
  std::unique_ptr<float[]> rec_buf(new (std::nothrow) float[std::max<size_t>(P * N, 1)]);
  if (!rec_buf) return ARAP_ENOMEM;
  const float* const rec = rec_buf.get();
  in.close();
  if (N > 0 && !read_parallel(path, (size_t)L.data_start, reinterpret_cast<char*>(rec_buf.get()),
                              P * N * sizeof(float), worker_count(N)))
    return ARAP_EBADINPUT;
  const int ix = L.at("x"), iop = L.at("opacity"), isc = L.at("scale_0"), irot = L.at("rot_0");
  const int isx = L.at("scale_1"), isy = L.at("scale_2");
  const int ir1 = L.at("rot_1"), ir2 = L.at("rot_2"), ir3 = L.at("rot_3");
  const int iy = L.at("y"), iz = L.at("z");
  const int idc[3] = {L.at("f_dc_0"), L.at("f_dc_1"), L.at("f_dc_2")};
  const int K = (L.sh_degree + 1) * (L.sh_degree + 1);
  std::vector<int> irest((size_t)3 * (K - 1));
  for (int i = 0; i < 3 * (K - 1); ++i) irest[i] = L.at("f_rest_" + std::to_string(i));
  const int iidx = L.at("index");

  // bounding box: per-thread partial min/max, combined (order-independent)
  const int nt = worker_count(N);
  std::vector<float> part_lo((size_t)nt * 3, INFINITY), part_hi((size_t)nt * 3, -INFINITY);
  const int ipos[3] = {ix, iy, iz};
  parallel_chunks(N, nt, [&](int t, size_t b, size_t e) {
    float* l = part_lo.data() + 3 * t;
    float* h = part_hi.data() + 3 * t;
    for (size_t i = b; i < e; ++i)
      for (int a = 0; a < 3; ++a) {
        const float v = rec[i * P + ipos[a]];
        l[a] = std::min(l[a], v);
        h[a] = std::max(h[a], v);
      }
  });
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int t = 0; t < nt; ++t)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], part_lo[3 * t + a]);
      hi[a] = std::max(hi[a], part_hi[3 * t + a]);
    }
  // the processing order: a stable sort by Morton code keeps ties in file order
  std::vector<uint32_t> order(N);
  for (size_t i = 0; i < N; ++i) order[i] = (uint32_t)i;
  if (morton_order && N > 1) {
    std::vector<uint64_t> code(N);
    parallel_chunks(N, nt, [&](int, size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) {
        const float p3[3] = {rec[i * P + ix], rec[i * P + iy], rec[i * P + iz]};
        code[i] = morton_code(p3, lo, hi);
      }
    });
    radix_sort_stable(code, order);
  }
  parallel_chunks(N, nt, [&](int, size_t kb, size_t ke) {
    const int is3[3] = {isc, isx, isy};
    for (size_t k = kb; k < ke; ++k) {
      const float* r = rec + (size_t)order[k] * P;
      for (int a = 0; a < 3; ++a) pos[3 * k + a] = r[ipos[a]];
      const float q[4] = {r[irot], r[ir1], r[ir2], r[ir3]};
      float len2 = 0.f;
      for (int j = 0; j < 4; ++j) len2 += q[j] * q[j];
      const float len = std::sqrt(len2);
      for (int j = 0; j < 4; ++j) rot[4 * k + j] = q[j] / len;
      for (int a = 0; a < 3; ++a) scale[3 * k + a] = std::exp(r[is3[a]]);
      opacity[k] = 1.0f / (1.0f + std::exp(-r[iop]));
      float* sh = shs + (size_t)kShFloats * k;
      for (int e = 0; e < kShFloats; ++e) sh[e] = 0.f;
      for (int c = 0; c < 3; ++c) sh[c] = r[idc[c]];
      for (int j = 1; j < K; ++j)
        for (int c = 0; c < 3; ++c) sh[3 * j + c] = r[irest[(size_t)c * (K - 1) + (j - 1)]];
      if (index) index[k] = (int32_t)std::lround(r[iidx]);
    }
  });
  if (box_min)
    for (int a = 0; a < 3; ++a) box_min[a] = lo[a];
  if (box_max)
    for (int a = 0; a < 3; ++a) box_max[a] = hi[a];
  return ARAP_OK;
}

extern "C" int arap_ply_save(const char* path, int64_t count, const float* pos, const float* shs,
                             const float* opacity, const float* scale, const float* rot, const float* box_min,
                             const float* box_max, const uint8_t* too_small, int64_t* written) {
  if (!little_endian_host()) return ARAP_EUNSUPPORTED;
  if (!path || count < 0 || (count > 0 && (!pos || !shs || !opacity || !scale || !rot)) || !box_min || !box_max)
    return ARAP_EBADINPUT;
  auto kept = [&](int64_t i) {
    for (int a = 0; a < 3; ++a)
      if (pos[3 * i + a] < box_min[a] || pos[3 * i + a] > box_max[a]) return false;
    return !(too_small && too_small[i]);
  };
  // kept splats per fixed chunk, then each chunk encodes into its own range
  const size_t total = (size_t)count;
  const int nt = worker_count(total);
  std::vector<int64_t> chunk_kept((size_t)nt + 1, 0);
  parallel_chunks(total, nt, [&](int t, size_t b, size_t e) {
    int64_t c = 0;
    for (size_t i = b; i < e; ++i) c += kept((int64_t)i) ? 1 : 0;
    chunk_kept[(size_t)t + 1] = c;
  });
  for (int t = 0; t < nt; ++t) chunk_kept[(size_t)t + 1] += chunk_kept[(size_t)t];
  const int64_t n = chunk_kept[(size_t)nt];
  std::ofstream out(path, std::ios_base::binary);
  if (!out.good()) return ARAP_EBADINPUT;
  out << "ply\nformat binary_little_endian 1.0\nelement vertex " << n << "\n";
  const char* head[] = {"x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"};
  for (const char* h : head) out << "property float " << h << "\n";
  for (int i = 0; i < 45; ++i) out << "property float f_rest_" << i << "\n";
  const char* tail[] = {"opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"};
  for (const char* t : tail) out << "property float " << t << "\n";
  out << "end_header\n";
  constexpr int R = 62;
  std::vector<float> rec((size_t)R * (size_t)n);
  parallel_chunks(total, nt, [&](int t, size_t b, size_t e) {
    int64_t k = chunk_kept[(size_t)t];
    for (size_t ii = b; ii < e; ++ii) {
      const int64_t i = (int64_t)ii;
      if (!kept(i)) continue;
      float* r = rec.data() + (size_t)R * (size_t)k;
      for (int a = 0; a < 3; ++a) r[a] = pos[3 * i + a];
      r[3] = r[4] = r[5] = 0.f;  // normals
      const float* sh = shs + (size_t)kShFloats * i;
      for (int c = 0; c < 3; ++c) r[6 + c] = sh[c];
      for (int j = 1; j < 16; ++j)
        for (int c = 0; c < 3; ++c) r[9 + c * 15 + (j - 1)] = sh[3 * j + c];
      const float o = opacity[i];
      r[54] = std::log(o / (1.0f - o));
      for (int a = 0; a < 3; ++a) r[55 + a] = std::log(scale[3 * i + a]);
      for (int j = 0; j < 4; ++j) r[58 + j] = rot[4 * i + j];
      ++k;
    }
  });
  if (n > 0) out.write(reinterpret_cast<const char*>(rec.data()), (std::streamsize)(rec.size() * sizeof(float)));
  if (!out.good()) return ARAP_EBADINPUT;
  if (written) *written = n;
  return ARAP_OK;
}
