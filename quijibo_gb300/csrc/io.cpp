// File formats of the path's outputs, written from host or device buffers:
//  * FIELD_3D's binary stream (FIELD_3D::write/read, src/geometry/FIELD_3D.cpp:4371-4450):
//    int xRes, yRes, zRes; double center[3]; double lengths[3]; double data[X*Y*Z].
//  * TRIANGLE_MESH's raw stream (TRIANGLE_MESH::write, TRIANGLE_MESH.cpp:4502-4522):
//    int V, int T; V x 3 doubles; T x 3 int vertex indices.
//  * OBJ as TRIANGLE_MESH::writeOBJ prints it (TRIANGLE_MESH.cpp:2762-2800): "v %.16f %.16f
//    %.16f" per vertex, then "f %i %i %i" with 1-based indices.
// Device buffers are copied out in chunks through a host staging buffer;
// OBJ lines are formatted by several host threads, chunk by chunk, and
// written in order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/quijibo_gpu.h"

namespace {

bool on_device(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // a host pointer on a machine without a device
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Calls fn(host_ptr, first, count) over [0, n) elements of `src` (host or
// device) in chunks of at most `chunk` elements.
template <class T, class Fn>
int for_chunks(const T* src, int64_t n, int64_t chunk, Fn fn) {
  if (!on_device(src)) {
    for (int64_t i = 0; i < n; i += chunk)
      if (int rc = fn(src + i, i, std::min(chunk, n - i))) return rc;
    return QJG_OK;
  }
  std::vector<T> host((size_t)std::min(chunk, std::max<int64_t>(n, 1)));
  for (int64_t i = 0; i < n; i += chunk) {
    const int64_t c = std::min(chunk, n - i);
    if (cudaMemcpy(host.data(), src + i, (size_t)c * sizeof(T), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
      return QJG_ERR_CUDA;
    if (int rc = fn(host.data(), i, c)) return rc;
  }
  return QJG_OK;
}

struct File {
  FILE* f = nullptr;
  explicit File(const char* path, const char* mode) : f(path ? std::fopen(path, mode) : nullptr) {}
  ~File() {
    if (f) std::fclose(f);
  }
  bool put(const void* p, size_t bytes) { return std::fwrite(p, 1, bytes, f) == bytes; }
};

constexpr int64_t kChunk = 1 << 20;  // elements per staged chunk

// printf-style append (a line of three %.16f of huge values can exceed any
// fixed buffer)
template <class... A>
void appendf(std::string& s, const char* fmt, A... a) {
  char buf[128];
  const int len = std::snprintf(buf, sizeof buf, fmt, a...);
  if (len < 0) return;
  if ((size_t)len < sizeof buf) {
    s.append(buf, (size_t)len);
    return;
  }
  const size_t at = s.size();
  s.resize(at + (size_t)len + 1);
  std::snprintf(&s[at], (size_t)len + 1, fmt, a...);
  s.resize(at + (size_t)len);
}

// Formats lines [0, count) with `line(i, str)` (appending to str) on several
// threads and writes them in order.
template <class LineFn>
bool write_lines(File& out, int64_t count, LineFn line) {
  const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const int64_t per = (count + nt - 1) / nt;
  std::vector<std::string> parts((size_t)nt);
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++) {
    th.emplace_back([&, t] {
      const int64_t a = t * per, b = std::min(count, a + per);
      std::string& s = parts[(size_t)t];
      s.reserve((size_t)std::max<int64_t>(b - a, 0) * 64);
      for (int64_t i = a; i < b; i++) line(i, s);
    });
  }
  for (auto& x : th) x.join();
  for (auto& s : parts)
    if (!s.empty() && !out.put(s.data(), s.size())) return false;
  return true;
}

}  // namespace

extern "C" {

int qjg_field3d_write(const char* path, const int32_t res[3], const double center[3],
                      const double lengths[3], const double* field) {
  if (!path || !res || !center || !lengths) return QJG_ERR_ARG;
  const int64_t n = (int64_t)res[0] * res[1] * res[2];
  if (res[0] < 0 || res[1] < 0 || res[2] < 0 || (n > 0 && !field)) return QJG_ERR_ARG;
  File out(path, "wb");
  if (!out.f) return QJG_ERR_ARG;
  const int32_t r[3] = {res[0], res[1], res[2]};
  if (!out.put(r, sizeof r) || !out.put(center, 3 * sizeof(double)) ||
      !out.put(lengths, 3 * sizeof(double)))
    return QJG_ERR_ARG;
  if (n <= 0) return QJG_OK;
  return for_chunks(field, n, kChunk, [&](const double* p, int64_t, int64_t c) {
    return out.put(p, (size_t)c * sizeof(double)) ? QJG_OK : QJG_ERR_ARG;
  });
}

int qjg_field3d_read_header(const char* path, int32_t res[3], double center[3],
                            double lengths[3]) {
  if (!path || !res || !center || !lengths) return QJG_ERR_ARG;
  File in(path, "rb");
  if (!in.f) return QJG_ERR_ARG;
  if (std::fread(res, sizeof(int32_t), 3, in.f) != 3 ||
      std::fread(center, sizeof(double), 3, in.f) != 3 ||
      std::fread(lengths, sizeof(double), 3, in.f) != 3)
    return QJG_ERR_ARG;
  return QJG_OK;
}

int qjg_field3d_read(const char* path, double* field, int64_t capacity) {
  int32_t res[3];
  double c[3], l[3];
  if (int rc = qjg_field3d_read_header(path, res, c, l)) return rc;
  if (res[0] < 0 || res[1] < 0 || res[2] < 0) return QJG_ERR_ARG;
  const int64_t n = (int64_t)res[0] * res[1] * res[2];
  if (n > capacity) return QJG_ERR_CAPACITY;
  if (n == 0) return QJG_OK;
  if (!field) return QJG_ERR_ARG;
  File in(path, "rb");
  if (!in.f || std::fseek(in.f, 3 * 4 + 6 * 8, SEEK_SET) != 0) return QJG_ERR_ARG;
  if (!on_device(field))
    return std::fread(field, sizeof(double), (size_t)n, in.f) == (size_t)n ? QJG_OK : QJG_ERR_ARG;
  std::vector<double> host((size_t)std::min<int64_t>(n, kChunk));
  for (int64_t i = 0; i < n; i += kChunk) {
    const int64_t cnt = std::min<int64_t>(kChunk, n - i);
    if (std::fread(host.data(), sizeof(double), (size_t)cnt, in.f) != (size_t)cnt)
      return QJG_ERR_ARG;
    if (cudaMemcpy(field + i, host.data(), (size_t)cnt * sizeof(double),
                   cudaMemcpyHostToDevice) != cudaSuccess)
      return QJG_ERR_CUDA;
  }
  return QJG_OK;
}

int qjg_mesh_write_raw(const char* path, const double* verts, int64_t n_verts,
                       const int32_t* tris, int64_t n_tris) {
  if (!path || n_verts < 0 || n_tris < 0 || n_verts > INT32_MAX || n_tris > INT32_MAX ||
      (n_verts && !verts) || (n_tris && !tris))
    return QJG_ERR_ARG;
  File out(path, "wb");
  if (!out.f) return QJG_ERR_ARG;
  const int32_t counts[2] = {(int32_t)n_verts, (int32_t)n_tris};
  if (!out.put(counts, sizeof counts)) return QJG_ERR_ARG;
  int rc = for_chunks(verts, 3 * n_verts, 3 * kChunk, [&](const double* p, int64_t, int64_t c) {
    return out.put(p, (size_t)c * sizeof(double)) ? QJG_OK : QJG_ERR_ARG;
  });
  if (rc) return rc;
  return for_chunks(tris, 3 * n_tris, 3 * kChunk, [&](const int32_t* p, int64_t, int64_t c) {
    return out.put(p, (size_t)c * sizeof(int32_t)) ? QJG_OK : QJG_ERR_ARG;
  });
}

int qjg_mesh_write_obj(const char* path, const double* verts64, const float* verts32,
                       int64_t n_verts, const int32_t* tris, int64_t n_tris) {
  if (!path || n_verts < 0 || n_tris < 0 || (verts64 && verts32) ||
      (n_verts && !verts64 && !verts32) || (n_tris && !tris))
    return QJG_ERR_ARG;
  File out(path, "w");
  if (!out.f) return QJG_ERR_ARG;
  int rc;
  if (verts64)
    rc = for_chunks(verts64, 3 * n_verts, 3 * kChunk, [&](const double* p, int64_t, int64_t c) {
      return write_lines(out, c / 3, [&](int64_t i, std::string& str) {
               appendf(str, "v %.16f %.16f %.16f\n", p[3 * i], p[3 * i + 1], p[3 * i + 2]);
             })
                 ? QJG_OK
                 : QJG_ERR_ARG;
    });
  else
    rc = for_chunks(verts32, 3 * n_verts, 3 * kChunk, [&](const float* p, int64_t, int64_t c) {
      return write_lines(out, c / 3, [&](int64_t i, std::string& str) {
               appendf(str, "v %.16f %.16f %.16f\n", (double)p[3 * i], (double)p[3 * i + 1],
                       (double)p[3 * i + 2]);
             })
                 ? QJG_OK
                 : QJG_ERR_ARG;
    });
  if (rc) return rc;
  return for_chunks(tris, 3 * n_tris, 3 * kChunk, [&](const int32_t* p, int64_t, int64_t c) {
    return write_lines(out, c / 3, [&](int64_t i, std::string& str) {
             appendf(str, "f %i %i %i\n", p[3 * i] + 1, p[3 * i + 1] + 1, p[3 * i + 2] + 1);
           })
               ? QJG_OK
               : QJG_ERR_ARG;
  });
}

}  // extern "C"

// ---------------------------------------------------------------- .o3d
// OPTIMIZE_3D::write / read (src/solvers/OPTIMIZE_3D.cpp:3253-3360): int
// xRes, yRes, zRes; VEC3 center, lengths; top and bottom POLYNOMIAL_4D
// (POLYNOMIAL_4D.cpp:650-727: int totalRoots; coefficient, derivative and
// second-derivative quaternion lists, each an int count then 4 doubles w x y
// z per entry; the roots likewise; an int count then totalRoots doubles of
// powers; the power scalar); double expScaling; int history count; then the
// fractal, distance and curvature FIELD_3D streams.

namespace {

constexpr int32_t kMaxRoots = 1 << 20;
constexpr int32_t kMaxList = 1 << 28;

struct Reader {
  FILE* f;
  bool ok = true;
  template <class T>
  T get() {
    T v{};
    if (ok && std::fread(&v, sizeof v, 1, f) != 1) ok = false;
    return v;
  }
  void get_n(double* dst, int64_t n) {
    if (!ok || n <= 0) return;
    if (dst) {
      if (std::fread(dst, sizeof(double), (size_t)n, f) != (size_t)n) ok = false;
    } else if (std::fseek(f, (long)(n * (int64_t)sizeof(double)), SEEK_CUR) != 0) {
      ok = false;
    }
  }
};

// One polynomial; roots (n x 4) and powers (n) are copied when not null.
bool read_poly(Reader& r, int32_t* n, double* sigma, double* roots, double* powers) {
  const int32_t total = r.get<int32_t>();
  if (!r.ok || total < 0 || total > kMaxRoots) return false;
  for (int list = 0; list < 3; list++) {  // coefficients, derivatives, second derivatives
    const int32_t c = r.get<int32_t>();
    if (!r.ok || c < 0 || c > kMaxList) return false;
    r.get_n(nullptr, 4ll * c);
  }
  const int32_t nr = r.get<int32_t>();
  if (!r.ok || nr < 0 || nr > kMaxRoots) return false;
  r.get_n(nr == total ? roots : nullptr, 4ll * nr);
  if (nr != total && roots) return false;
  r.get<int32_t>();  // the powers' count; the reader takes totalRoots of them
  r.get_n(powers, total);
  const double ps = r.get<double>();
  if (n) *n = total;
  if (sigma) *sigma = ps;
  return r.ok;
}

bool read_field_header(Reader& r, int32_t res[3], double c[3], double l[3]) {
  for (int k = 0; k < 3; k++) res[k] = r.get<int32_t>();
  for (int k = 0; k < 3; k++) c[k] = r.get<double>();
  for (int k = 0; k < 3; k++) l[k] = r.get<double>();
  return r.ok;
}

int64_t cells(const int32_t res[3]) {
  return (res[0] > 0 && res[1] > 0 && res[2] > 0) ? (int64_t)res[0] * res[1] * res[2] : 0;
}

int read_o3d(const char* path, qjg_o3d_info* info, double* top_roots, double* top_powers,
             double* bot_roots, double* bot_powers, double* fields[3]) {
  if (!path || !info) return QJG_ERR_ARG;
  File in(path, "rb");
  if (!in.f) return QJG_ERR_ARG;
  Reader r{in.f};
  for (int k = 0; k < 3; k++) info->res[k] = r.get<int32_t>();
  for (int k = 0; k < 3; k++) info->center[k] = r.get<double>();
  for (int k = 0; k < 3; k++) info->lengths[k] = r.get<double>();
  if (!r.ok) return QJG_ERR_ARG;
  if (!read_poly(r, &info->n_top, &info->sigma_top, top_roots, top_powers) ||
      !read_poly(r, &info->n_bot, &info->sigma_bot, bot_roots, bot_powers))
    return QJG_ERR_ARG;
  info->exp_scaling = r.get<double>();
  info->history = r.get<int32_t>();
  for (int k = 0; k < 3; k++) {
    if (!read_field_header(r, info->field_res[k], info->field_center[k], info->field_lengths[k]))
      return QJG_ERR_ARG;
    r.get_n(fields ? fields[k] : nullptr, cells(info->field_res[k]));
  }
  return r.ok ? QJG_OK : QJG_ERR_ARG;
}

bool write_poly(File& out, int32_t n, const double* roots, const double* powers, double sigma) {
  const int32_t zero = 0;
  bool ok = out.put(&n, 4);
  for (int list = 0; list < 3; list++) ok = ok && out.put(&zero, 4);
  ok = ok && out.put(&n, 4) && (n == 0 || out.put(roots, (size_t)n * 32));
  ok = ok && out.put(&n, 4) && (n == 0 || out.put(powers, (size_t)n * 8));
  return ok && out.put(&sigma, 8);
}

}  // namespace

extern "C" {

int qjg_o3d_read_info(const char* path, qjg_o3d_info* info) {
  return read_o3d(path, info, nullptr, nullptr, nullptr, nullptr, nullptr);
}

int qjg_o3d_read(const char* path, double* top_roots, double* top_powers, double* bot_roots,
                 double* bot_powers, double* fractal, double* distance, double* curvature) {
  qjg_o3d_info info;
  double* fields[3] = {fractal, distance, curvature};
  return read_o3d(path, &info, top_roots, top_powers, bot_roots, bot_powers, fields);
}

int qjg_o3d_write(const char* path, const qjg_o3d_info* info, const double* top_roots,
                  const double* top_powers, const double* bot_roots, const double* bot_powers,
                  const double* fractal, const double* distance, const double* curvature) {
  if (!path || !info || info->n_top < 0 || info->n_bot < 0 ||
      (info->n_top && (!top_roots || !top_powers)) || (info->n_bot && (!bot_roots || !bot_powers)))
    return QJG_ERR_ARG;
  const double* fields[3] = {fractal, distance, curvature};
  for (int k = 0; k < 3; k++)
    if (cells(info->field_res[k]) > 0 && !fields[k]) return QJG_ERR_ARG;
  File out(path, "wb");
  if (!out.f) return QJG_ERR_ARG;
  bool ok = out.put(info->res, 12) && out.put(info->center, 24) && out.put(info->lengths, 24);
  ok = ok && write_poly(out, info->n_top, top_roots, top_powers, info->sigma_top);
  ok = ok && write_poly(out, info->n_bot, bot_roots, bot_powers, info->sigma_bot);
  ok = ok && out.put(&info->exp_scaling, 8) && out.put(&info->history, 4);
  for (int k = 0; k < 3 && ok; k++) {
    ok = out.put(info->field_res[k], 12) && out.put(info->field_center[k], 24) &&
         out.put(info->field_lengths[k], 24);
    const int64_t n = cells(info->field_res[k]);
    if (ok && n > 0) ok = out.put(fields[k], (size_t)n * 8);
  }
  return ok ? QJG_OK : QJG_ERR_ARG;
}

}  // extern "C"
