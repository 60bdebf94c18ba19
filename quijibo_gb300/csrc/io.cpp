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
