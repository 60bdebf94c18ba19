// GPU backing for the reference's own C++ surface, linked into the
// reference drivers (projects/*MarchingCubes3D, projects/toothOptimizer)
// with GNU ld's --wrap, so the drivers run unchanged on the GB300 path:
//
//   g++ ... driver.o <reference objects> quijibo_gpu_adapter.o \
//       -L<lib dir> -lquijibo_gpu -Wl,--wrap=<symbol> ...
//
// (the symbols are listed by `make -C quijibo_gb300/adapter wrap-flags`).
// Each wrapped function keeps its reference signature and semantics:
//   OPTIMIZE_3D::computeLogScaledPowerRationalMap(top, bottom, fractal, verbose)
//       src/solvers/OPTIMIZE_3D.cpp:1272-1370        -> qjg_field_host
//   TRIANGLE_MESH(const FIELD_3D&)                   TRIANGLE_MESH.cpp:48-57  -> qjg_mesh_field, linear
//   TRIANGLE_MESH(field, top, bottom, s, maxIt, slice, iso)      :62-76      -> qjg_mesh_field, bisection
//   TRIANGLE_MESH(center, lengths, res, top, bottom, s, maxIt, slice, iso, rotation, cacheFile)
//       :84-101                                      -> qjg_mesh_stream
//   OPTIMIZE_3D::computeScoreAP and the five gradient methods toothOptimizer
//       calls (OPTIMIZE_3D.cpp:3563-3625, 8905-10602) -> one qjg_tanh_score_grad
//       per state, cached for the gradient calls that follow it.
// The reference's escape radius (2000 for the map and the meshers, 20 for the
// AP score) is kept.  QJG_PRECISION=fp32refine selects the precision form
// for the field and the streaming mesher (default: the plain FP64 form).
// The constructed meshes are filled through TRIANGLE_MESH::read (the
// reference's raw format, TRIANGLE_MESH.cpp:4527-4553), so writeOBJ and the
// rest of the class work on them unchanged.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <unistd.h>

#include "OPTIMIZE_3D.h"
#include "TRIANGLE_MESH.h"
#include "quijibo_gpu.h"

#if defined(USING_DOUBLE_NLS)
#define QJA_R "d"
#define QJA_V "TVEC3IdE"
#else
#define QJA_R "e"
#define QJA_V "TVEC3IeE"
#endif

#define QJA_MAP "_ZN11OPTIMIZE_3D32computeLogScaledPowerRationalMapERK13POLYNOMIAL_4DS2_R8FIELD_3Db"
#define QJA_MESH_LINEAR "_ZN13TRIANGLE_MESHC1ERK8FIELD_3D"
#define QJA_MESH_FIELD "_ZN13TRIANGLE_MESHC1ERK8FIELD_3DRK13POLYNOMIAL_4DS5_" QJA_R "i" QJA_R QJA_R
#define QJA_MESH_STREAM                                                                      \
  "_ZN13TRIANGLE_MESHC1ERK5" QJA_V "S3_RKS0_IiERK13POLYNOMIAL_4DS9_" QJA_R "i" QJA_R QJA_R \
  "RK10QUATERNIONRKNSt7__cxx1112basic_stringIcSt11char_traitsIcESaIcEEE"
#define QJA_MESH_LAGRANGE \
  "_ZN13TRIANGLE_MESHC1ERK5" QJA_V "S3_RKS0_IiERK13POLYNOMIAL_4DS9_" QJA_R "i" QJA_R QJA_R \
  "RK10QUATERNION"
#define QJA_SCORE "_ZN11OPTIMIZE_3D14computeScoreAPEv"
#define QJA_EXPG "_ZN11OPTIMIZE_3D20computeExpGradientAPEv"
#define QJA_TOPG "_ZN11OPTIMIZE_3D20computeTopGradientAPEi"
#define QJA_BOTG "_ZN11OPTIMIZE_3D23computeBottomGradientAPEi"
#define QJA_TOPBULK "_ZN11OPTIMIZE_3D30computeTopBulkScalarGradientAPEv"
#define QJA_BOTBULK "_ZN11OPTIMIZE_3D33computeBottomBulkScalarGradientAPEv"

namespace {

void die(const char* what, qjg_ctx* ctx, int rc) {
  std::fprintf(stderr, "quijibo_gpu adapter: %s failed (%d): %s\n", what, rc,
               ctx ? qjg_last_error(ctx) : "");
  std::exit(1);  // the reference's own convention on failure
}

qjg_ctx* gpu() {
  static qjg_ctx* ctx = nullptr;
  if (!ctx) {
    const int rc = qjg_create(0, &ctx);
    if (rc) die("qjg_create", nullptr, rc);
  }
  return ctx;
}

int precision() {
  const char* p = std::getenv("QJG_PRECISION");
  return (p && std::string(p) == "fp32refine") ? QJG_FP32_REFINE : QJG_FP64;
}

qjg_rootset upload(const POLYNOMIAL_4D& top, const POLYNOMIAL_4D& bottom, Real s) {
  std::vector<double> tr, tp, br, bp;
  for (int i = 0; i < top.totalRoots(); i++) {
    for (int c = 0; c < 4; c++) tr.push_back((double)top.roots()[i][c]);
    tp.push_back((double)top.powers()[i]);
  }
  for (int i = 0; i < bottom.totalRoots(); i++) {
    for (int c = 0; c < 4; c++) br.push_back((double)bottom.roots()[i][c]);
    bp.push_back((double)bottom.powers()[i]);
  }
  qjg_rootset h;
  const int rc = qjg_rootset_upload(gpu(), top.totalRoots(), tr.data(), tp.data(),
                                    (double)top.powerScalar(), bottom.totalRoots(),
                                    br.empty() ? nullptr : br.data(), bp.empty() ? nullptr : bp.data(),
                                    bottom.totalRoots() ? (double)bottom.powerScalar() : 1.0,
                                    (double)s, &h);
  if (rc) die("qjg_rootset_upload", gpu(), rc);
  return h;
}

qjg_grid grid_of(const VEC3I& res, const VEC3F& center, const VEC3F& lengths,
                 const QUATERNION& rot, Real slice) {
  qjg_grid g;
  for (int c = 0; c < 3; c++) {
    g.res[c] = res[c];
    g.center[c] = (double)center[c];
    g.lengths[c] = (double)lengths[c];
  }
  for (int c = 0; c < 4; c++) g.rot[c] = (double)rot[c];
  g.slice = (double)slice;
  return g;
}

qjg_iter iter_of(int max_it, double escape, int prec) {
  qjg_iter it = {};
  it.max_it = max_it;
  it.precision = prec;
  it.refine_pow = QJG_REFINE_POW;
  it.want_de = 0;
  it.escape = escape;
  it.band_h = 2.0;
  it.field_tol = 1e-3;
  it.rel_tol = prec == QJG_FP32_REFINE ? 1e-6 : 0.0;
  return it;
}

// Device outputs of a mesher call, read back into the raw format of
// TRIANGLE_MESH::read: int V, int T, V x 3 doubles, T x 3 ints.
struct MeshOut {
  double* v = nullptr;
  int32_t* t = nullptr;
  int64_t vcap = 0, tcap = 0;
  void alloc(int64_t nv, int64_t nt) {
    release();
    vcap = nv;
    tcap = nt;
    if (cudaMalloc(&v, sizeof(double) * 3 * std::max<int64_t>(nv, 1)) ||
        cudaMalloc(&t, sizeof(int32_t) * 3 * std::max<int64_t>(nt, 1)))
      die("cudaMalloc", nullptr, QJG_ERR_NOMEM);
  }
  void release() {
    if (v) cudaFree(v);
    if (t) cudaFree(t);
    v = nullptr;
    t = nullptr;
  }
  ~MeshOut() { release(); }
};

void fill_mesh(TRIANGLE_MESH* self, const MeshOut& out, const qjg_mesh_stats& st) {
  const int V = (int)st.n_verts, T = (int)st.n_tris;
  std::vector<char> raw(2 * sizeof(int) + (size_t)V * 3 * sizeof(double) + (size_t)T * 3 * sizeof(int));
  std::memcpy(raw.data(), &V, sizeof V);
  std::memcpy(raw.data() + sizeof V, &T, sizeof T);
  char* p = raw.data() + 2 * sizeof(int);
  cudaMemcpy(p, out.v, (size_t)V * 3 * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(p + (size_t)V * 3 * sizeof(double), out.t, (size_t)T * 3 * sizeof(int),
             cudaMemcpyDeviceToHost);
  FILE* f = fmemopen(raw.data(), raw.size(), "rb");
  if (!f) die("fmemopen", nullptr, QJG_ERR_NOMEM);
  self->read(f);
  std::fclose(f);
}

template <class Call>
void run_mesher(TRIANGLE_MESH* self, int64_t n_vox, Call call) {
  MeshOut out;
  qjg_mesh_stats st;
  out.alloc(n_vox / 4 + 1024, n_vox / 2 + 1024);
  int rc = call(out, &st);
  if (rc == QJG_ERR_CAPACITY) {  // retry with the counts the mesher reported
    out.alloc(st.n_verts, st.n_tris + st.n_degenerate);
    rc = call(out, &st);
  }
  if (rc) die("mesher", gpu(), rc);
  new (self) TRIANGLE_MESH();
  fill_mesh(self, out, st);
}

// The streaming mesher's edge cache (TRIANGLE_MESH.cpp:681-768): the
// reference writes it after classifying when the file is absent
// (writeEdgeCacheHuge, :535-586), and when it exists takes its cube flags and
// edges instead of classifying again (readEdgeCacheHuge, :431-482).  Here the
// grid is always classified on the GPU (it costs milliseconds); an absent
// file is written with the same bytes, an existing one is compared with the
// lists just computed and reported when it does not match them (a cache left
// by another map or grid, which the reference would mesh from).
std::vector<char> file_bytes(const std::string& path, bool* ok) {
  std::vector<char> b;
  *ok = false;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return b;
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + n);
  std::fclose(f);
  *ok = true;
  return b;
}

void edge_cache(const std::string& path) {
  bool exists;
  const std::vector<char> old = file_bytes(path, &exists);
  if (!exists) {
    const int rc = qjg_mesh_edge_cache_write(gpu(), path.c_str());
    if (rc) std::printf(" FAILED TO CACHE OUT EDGES: %s\n", path.c_str());
    return;
  }
  char tmp[] = "/tmp/qja_edgecacheXXXXXX";
  const int fd = mkstemp(tmp);
  if (fd < 0) return;
  close(fd);
  bool ok = qjg_mesh_edge_cache_write(gpu(), tmp) == 0;
  const std::vector<char> now = ok ? file_bytes(tmp, &ok) : std::vector<char>();
  unlink(tmp);
  if (ok && now != old)
    std::printf(" Cache file %s does not match this grid and map; the mesh is the recomputed one\n",
                path.c_str());
}

// The state of the last GPU score, for the gradient calls that follow it.
struct ScoreCache {
  std::vector<double> grad;  // [log s, bottom, top, sigma_t, sigma_b]
  bool valid = false;
};
std::map<const OPTIMIZE_3D*, ScoreCache> g_scores;

}  // namespace

// ---------------------------------------------------------------- wrappers

void qja_map(OPTIMIZE_3D* self, const POLYNOMIAL_4D& top, const POLYNOMIAL_4D& bottom,
             FIELD_3D& fractal, bool verbose) __asm__("__wrap_" QJA_MAP);
void qja_map(OPTIMIZE_3D* self, const POLYNOMIAL_4D& top, const POLYNOMIAL_4D& bottom,
             FIELD_3D& fractal, bool verbose) {
  (void)verbose;
  const qjg_rootset h = upload(top, bottom, self->expScaling());
  const qjg_grid g = grid_of(fractal.res(), fractal.center(), fractal.lengths(), fractal.rotation(),
                             self->slice());
  const qjg_iter it = iter_of(self->maxIterations(), 2000.0, precision());
  std::vector<double> out((size_t)fractal.totalCells());
  const int rc = qjg_field_host(gpu(), h, &g, &it, out.data(), nullptr, nullptr);
  if (rc) die("qjg_field_host", gpu(), rc);
  for (int i = 0; i < fractal.totalCells(); i++) fractal[i] = (Real)out[i];
  qjg_rootset_free(gpu(), h);
}

void qja_mesh_linear(TRIANGLE_MESH* self, const FIELD_3D& field) __asm__("__wrap_" QJA_MESH_LINEAR);
void qja_mesh_linear(TRIANGLE_MESH* self, const FIELD_3D& field) {
  const qjg_grid g = grid_of(field.res(), field.center(), field.lengths(), field.rotation(), 0);
  const int64_t n = field.totalCells();
  std::vector<double> host(n);
  for (int64_t i = 0; i < n; i++) host[i] = (double)field[i];
  double* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(double))) die("cudaMalloc", nullptr, QJG_ERR_NOMEM);
  cudaMemcpy(d, host.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  run_mesher(self, n, [&](MeshOut& o, qjg_mesh_stats* st) {
    return qjg_mesh_field(gpu(), -1, &g, nullptr, d, QJG_EDGE_LINEAR, 0.0, 0, o.v, nullptr, o.vcap,
                          o.t, o.tcap, st, nullptr);
  });
  cudaFree(d);
}

void qja_mesh_field(TRIANGLE_MESH* self, const FIELD_3D& field, const POLYNOMIAL_4D& top,
                    const POLYNOMIAL_4D& bottom, Real expScaling, int maxIterations, Real slice,
                    Real isosurface) __asm__("__wrap_" QJA_MESH_FIELD);
void qja_mesh_field(TRIANGLE_MESH* self, const FIELD_3D& field, const POLYNOMIAL_4D& top,
                    const POLYNOMIAL_4D& bottom, Real expScaling, int maxIterations, Real slice,
                    Real isosurface) {
  const qjg_rootset h = upload(top, bottom, expScaling);
  const qjg_grid g = grid_of(field.res(), field.center(), field.lengths(), field.rotation(), slice);
  const qjg_iter it = iter_of(maxIterations, 2000.0, QJG_FP64);
  const int64_t n = field.totalCells();
  std::vector<double> host(n);
  for (int64_t i = 0; i < n; i++) host[i] = (double)field[i];
  double* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(double))) die("cudaMalloc", nullptr, QJG_ERR_NOMEM);
  cudaMemcpy(d, host.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  run_mesher(self, n, [&](MeshOut& o, qjg_mesh_stats* st) {
    return qjg_mesh_field(gpu(), h, &g, &it, d, QJG_EDGE_BISECT, (double)isosurface, 0, o.v, nullptr,
                          o.vcap, o.t, o.tcap, st, nullptr);
  });
  cudaFree(d);
  qjg_rootset_free(gpu(), h);
}

void qja_mesh_stream(TRIANGLE_MESH* self, const VEC3F& center, const VEC3F& lengths,
                     const VEC3I& res, const POLYNOMIAL_4D& top, const POLYNOMIAL_4D& bottom,
                     Real expScaling, int maxIterations, Real slice, Real isosurface,
                     const QUATERNION& rotation, const std::string& cacheFilename)
    __asm__("__wrap_" QJA_MESH_STREAM);
void qja_mesh_stream(TRIANGLE_MESH* self, const VEC3F& center, const VEC3F& lengths,
                     const VEC3I& res, const POLYNOMIAL_4D& top, const POLYNOMIAL_4D& bottom,
                     Real expScaling, int maxIterations, Real slice, Real isosurface,
                     const QUATERNION& rotation, const std::string& cacheFilename) {
  const qjg_rootset h = upload(top, bottom, expScaling);
  const qjg_grid g = grid_of(res, center, lengths, rotation, slice);
  const qjg_iter it = iter_of(maxIterations, 2000.0, precision());
  const bool cache = !cacheFilename.empty();
  if (cache) qjg_mesh_capture(gpu(), 1);
  run_mesher(self, (int64_t)res[0] * res[1] * 8, [&](MeshOut& o, qjg_mesh_stats* st) {
    return qjg_mesh_stream(gpu(), h, &g, &it, (double)isosurface, 0, o.v, nullptr, o.vcap, o.t,
                           o.tcap, st, nullptr);
  });
  qjg_rootset_free(gpu(), h);
  if (cache) {
    edge_cache(cacheFilename);
    qjg_mesh_capture(gpu(), 0);
  }
}

// TRIANGLE_MESH(center, lengths, res, top, bottom, expScaling, maxIterations,
// slice, isosurface, rotation): the Lagrange streaming mesher
// (TRIANGLE_MESH.cpp:106-123), in the form QJG_PRECISION selects.
void qja_mesh_lagrange(TRIANGLE_MESH* self, const VEC3F& center, const VEC3F& lengths,
                       const VEC3I& res, const POLYNOMIAL_4D& top, const POLYNOMIAL_4D& bottom,
                       Real expScaling, int maxIterations, Real slice, Real isosurface,
                       const QUATERNION& rotation) __asm__("__wrap_" QJA_MESH_LAGRANGE);
void qja_mesh_lagrange(TRIANGLE_MESH* self, const VEC3F& center, const VEC3F& lengths,
                       const VEC3I& res, const POLYNOMIAL_4D& top, const POLYNOMIAL_4D& bottom,
                       Real expScaling, int maxIterations, Real slice, Real isosurface,
                       const QUATERNION& rotation) {
  const qjg_rootset h = upload(top, bottom, expScaling);
  const qjg_grid g = grid_of(res, center, lengths, rotation, slice);
  qjg_iter it = iter_of(maxIterations, 2000.0, precision());
  it.form = QJG_FORM_LAGRANGE;
  run_mesher(self, (int64_t)res[0] * res[1] * 8, [&](MeshOut& o, qjg_mesh_stats* st) {
    return qjg_mesh_stream(gpu(), h, &g, &it, (double)isosurface, 0, o.v, nullptr, o.vcap, o.t,
                           o.tcap, st, nullptr);
  });
  qjg_rootset_free(gpu(), h);
}

Real qja_score(OPTIMIZE_3D* self) __asm__("__wrap_" QJA_SCORE);
Real qja_score(OPTIMIZE_3D* self) {
  const qjg_rootset h = upload(self->top(), self->bottom(), self->expScaling());
  FIELD_3D& f = self->fractal();
  FIELD_3D& w = self->weightField();
  const qjg_grid g = grid_of(f.res(), f.center(), f.lengths(), f.rotation(), self->slice());
  const qjg_grid wg = grid_of(w.res(), w.center(), w.lengths(), w.rotation(), 0);
  const int64_t nw = w.totalCells(), nf = f.totalCells();
  std::vector<double> hw(nw);
  for (int64_t i = 0; i < nw; i++) hw[i] = (double)w[i];
  double *dw = nullptr, *df = nullptr;
  if (cudaMalloc(&dw, nw * sizeof(double)) || cudaMalloc(&df, nf * sizeof(double)))
    die("cudaMalloc", nullptr, QJG_ERR_NOMEM);
  cudaMemcpy(dw, hw.data(), nw * sizeof(double), cudaMemcpyHostToDevice);
  ScoreCache& c = g_scores[self];
  c.grad.assign(3 + self->top().totalRoots() + self->bottom().totalRoots(), 0.0);
  double score = 0;
  // _tanhAlpha and _tanhThreshold keep the values the constructors give them (10, 0)
  const int rc = qjg_tanh_score_grad(gpu(), h, &g, self->maxIterations(), &wg, dw, 10.0, 0.0,
                                     &score, c.grad.data(), df, nullptr, nullptr);
  if (rc) die("qjg_tanh_score_grad", gpu(), rc);
  std::vector<double> hf(nf);
  cudaMemcpy(hf.data(), df, nf * sizeof(double), cudaMemcpyDeviceToHost);
  for (int64_t i = 0; i < nf; i++) f[i] = (Real)hf[i];
  cudaFree(dw);
  cudaFree(df);
  qjg_rootset_free(gpu(), h);
  c.valid = true;
  return (Real)score;
}

static const ScoreCache& cached(OPTIMIZE_3D* self) {
  auto it = g_scores.find(self);
  if (it == g_scores.end() || !it->second.valid) qja_score(self);
  return g_scores[self];
}

Real qja_expg(OPTIMIZE_3D* self) __asm__("__wrap_" QJA_EXPG);
Real qja_expg(OPTIMIZE_3D* self) { return (Real)cached(self).grad[0]; }

Real qja_botg(OPTIMIZE_3D* self, int i) __asm__("__wrap_" QJA_BOTG);
Real qja_botg(OPTIMIZE_3D* self, int i) { return (Real)cached(self).grad[1 + i]; }

Real qja_topg(OPTIMIZE_3D* self, int i) __asm__("__wrap_" QJA_TOPG);
Real qja_topg(OPTIMIZE_3D* self, int i) {
  return (Real)cached(self).grad[1 + self->bottom().totalRoots() + i];
}

Real qja_topbulk(OPTIMIZE_3D* self) __asm__("__wrap_" QJA_TOPBULK);
Real qja_topbulk(OPTIMIZE_3D* self) {
  return (Real)cached(self).grad[1 + self->bottom().totalRoots() + self->top().totalRoots()];
}

Real qja_botbulk(OPTIMIZE_3D* self) __asm__("__wrap_" QJA_BOTBULK);
Real qja_botbulk(OPTIMIZE_3D* self) {
  return (Real)cached(self).grad[2 + self->bottom().totalRoots() + self->top().totalRoots()];
}
