// Harness that runs the reference QUIJIBO implementation, compiled from its
// own sources, behind a small C ABI.  TEST INFRASTRUCTURE ONLY: it is built
// (by oracle/Makefile) only where the reference sources are present, into
// oracle/_ref/, and is used to pin the C restatement in qj_oracle.c and to
// generate the golden fixtures in tests/golden/.
//
// Everything here calls the reference's own classes; the one loop written
// here is the escape-time loop with the escape radius as a parameter
// (the reference hard-codes 2000), restated from OPTIMIZE_3D.cpp:1317-1362
// around the reference's POLYNOMIAL_4D / QUATERNION / FIELD_3D calls.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>
#include <vector>

#include "FIELD_3D.h"
#include "MERSENNETWISTER.h"
#include "OPTIMIZE_3D.h"
#include "POLYNOMIAL_4D.h"
#include "QUATERNION.h"
#include "RATIONAL_4D.h"
#include "TAO_SOLVER.h"
#include "TRIANGLE_MESH.h"

namespace {

POLYNOMIAL_4D make_poly(int n, const double* roots, const double* pows, double sigma) {
  if (n == 0) return POLYNOMIAL_4D();
  std::vector<QUATERNION> r;
  std::vector<Real> p;
  for (int i = 0; i < n; i++) {
    r.push_back(QUATERNION(roots[4 * i], roots[4 * i + 1], roots[4 * i + 2], roots[4 * i + 3]));
    p.push_back(pows[i]);
  }
  POLYNOMIAL_4D poly(r, p);
  poly.powerScalar() = sigma;
  return poly;
}

struct MapArgs {
  int nt;
  const double* troots;
  const double* tpows;
  double tsig;
  int nb;
  const double* broots;
  const double* bpows;
  double bsig;
  double s;
};

int export_mesh(TRIANGLE_MESH& mesh, double* verts, int max_v, int* tris, int max_t, int* nv,
                int* nt) {
  const int V = (int)mesh.vertices().size();
  const int T = (int)mesh.triangles().size();
  *nv = V;
  *nt = T;
  if (V > max_v || T > max_t) return -1;
  for (int i = 0; i < V; i++)
    for (int c = 0; c < 3; c++) verts[3 * i + c] = (double)mesh.vertices()[i][c];
  for (int t = 0; t < T; t++)
    for (int j = 0; j < 3; j++) tris[3 * t + j] = mesh.vertexIndex(t, j);
  return 0;
}

// ---- the BLMVM callbacks -------------------------------------------------
// TAO_SOLVER takes a plain function pointer with no user data, so the
// objective of the current solve is held here.
typedef void (*ref_objective)(int n, const double* x, double* f, double* g);
ref_objective g_objective = nullptr;

void objective_trampoline(const VECTOR& x, Real& f, VECTOR& g) {
  const int n = (int)x.size();
  std::vector<double> xx(n), gg(n);
  for (int i = 0; i < n; i++) xx[i] = (double)x[i];
  double ff = 0;
  g_objective(n, xx.data(), &ff, gg.data());
  f = ff;
  g.resize(n);
  for (int i = 0; i < n; i++) g[i] = gg[i];
}

// toothOptimizer's two objectives over a global OPTIMIZE_3D, restated from
// FormScaledFunctionGradient / FormScaledOnlyFunctionGradient
// (projects/toothOptimizer/toothOptimizer.cpp:65-130); every evaluation's
// value and state are appended to the history.
OPTIMIZE_3D* g_opt = nullptr;
std::vector<double>* g_hist = nullptr;

void record(const VECTOR& state, Real f) {
  g_hist->push_back((double)f);
  for (int i = 0; i < state.size(); i++) g_hist->push_back((double)state[i]);
}

void scaled_fg(const VECTOR& state, Real& function, VECTOR& gradient) {
  OPTIMIZE_3D& o = *g_opt;
  const int nt = o.top().totalRoots(), nb = o.bottom().totalRoots();
  const int k = 1 + nt + nb;
  o.expScaling() = exp(state[0]);
  int xi = 1;
  for (int i = 0; i < nb; i++, xi++) o.bottom().powersMutable()[i] = state[xi];
  for (int i = 0; i < nt; i++, xi++) o.top().powersMutable()[i] = state[xi];
  o.top().powerScalar() = state[k];
  o.bottom().powerScalar() = state[k + 1];
  function = o.computeScoreAP();
  gradient.resize(k + 2);
  gradient[0] = o.computeExpGradientAP();
  for (int i = 0; i < nb; i++) gradient[i + 1] = o.computeBottomGradientAP(i);
  for (int i = 0; i < nt; i++) gradient[i + 1 + nb] = o.computeTopGradientAP(i);
  gradient[k] = o.computeTopBulkScalarGradientAP();
  gradient[k + 1] = o.computeBottomBulkScalarGradientAP();
  record(state, function);
}

void scaled_only_fg(const VECTOR& state, Real& function, VECTOR& gradient) {
  OPTIMIZE_3D& o = *g_opt;
  o.expScaling() = exp(state[0]);
  o.top().powerScalar() = state[1];
  o.bottom().powerScalar() = state[2];
  function = o.computeScoreAP();
  gradient.resize(3);
  gradient[0] = o.computeExpGradientAP();
  gradient[1] = o.computeTopBulkScalarGradientAP();
  gradient[2] = o.computeBottomBulkScalarGradientAP();
  record(state, function);
}

}  // namespace

extern "C" {

// TAO_SOLVER::optimizeBLMVM (src/TOUPEE/TAO_SOLVER.cpp:72-341) with the
// tolerances toothOptimizer sets, on an objective given as a C callback.
void ref_blmvm(int n, double* x, const double* lower, const double* upper, ref_objective fg) {
  g_objective = fg;
  VECTOR sol(n), lo(n), hi(n);
  for (int i = 0; i < n; i++) {
    sol[i] = x[i];
    lo[i] = lower[i];
    hi[i] = upper[i];
  }
  TAO_SOLVER tao;
  tao.SetTolerances(1e-8, 1e-8, 1e-8, 1e-8, 0);
  tao.optimizeBLMVM(sol, hi, lo, objective_trampoline);
  for (int i = 0; i < n; i++) x[i] = (double)sol[i];
  g_objective = nullptr;
}

// toothOptimizer's main (projects/toothOptimizer/toothOptimizer.cpp:462-530)
// and optimizeSpecificResolution (:385-457) around the reference's classes,
// for the levels given and without the reweighted solve (it needs the
// external sdfGen): read, frame change, amp, then per level the conformal
// scan (first level), scaled-only, scaled and unweighted scaled solves.
// out gets per level [bottom powers, top powers, sigma_t, sigma_b, scale,
// score at the level's end (computeScoreAP)],
// evals per level the evaluations of the three solves; roots_out the final
// roots (top then bottom, 4 each).
void ref_tooth_run(const char* path, double radius, double amp, int nlev, const int* levels,
                   double* out, int* evals, double* roots_out) {
  OPTIMIZE_3D opt;
  opt.read(std::string(path));
  if (opt.lengths()[0] < 0.95 * radius) {
    opt.translateEverythingExceptFirst(VEC3F(-0.5, -0.5, -0.5));
    opt.scaleEverything(radius);
  }
  POLYNOMIAL_4D& top = opt.top();
  POLYNOMIAL_4D& bottom = opt.bottom();
  for (int x = 1; x < top.totalRoots(); x++) top.powersMutable()[x] *= amp;
  for (int x = 1; x < bottom.totalRoots(); x++) bottom.powersMutable()[x] *= amp;
  top.powerScalar() = 1;
  bottom.powerScalar() = 1;
  const int nt = top.totalRoots(), nb = bottom.totalRoots();
  std::vector<double> hv;
  g_opt = &opt;
  g_hist = &hv;
  for (int l = 0; l < nlev; l++) {
    const int res = levels[l];
    VEC3F center = opt.fractal().center();
    VEC3F lengths = opt.fractal().lengths();
    opt.fractal() = FIELD_3D(res, res, res, center, lengths);
    opt.auxiliary() = FIELD_3D(res, res, res, center, lengths);
    opt.maxIterations() = 1;
    if (l == 0) opt.estimateConformalRadius();
    for (int mode = 0; mode < 3; mode++) {
      const int n = mode == 0 ? 3 : 3 + nt + nb;
      VECTOR sol(n);
      sol[0] = log(opt.expScaling());
      if (mode == 0) {
        sol[1] = opt.top().powerScalar();
        sol[2] = opt.bottom().powerScalar();
      } else {
        int xi = 1;
        for (int i = 0; i < nb; i++, xi++) sol[xi] = opt.bottom().powersMutable()[i];
        for (int i = 0; i < nt; i++, xi++) sol[xi] = opt.top().powersMutable()[i];
        sol[n - 2] = opt.top().powerScalar();
        sol[n - 1] = opt.bottom().powerScalar();
      }
      VECTOR hi = VECTOR::Constant(n, FLT_MAX);
      VECTOR lo = VECTOR::Zero(n);
      lo[0] = -FLT_MAX;
      hv.clear();
      TAO_SOLVER tao;
      tao.SetTolerances(1e-8, 1e-8, 1e-8, 1e-8, 0);
      tao.maxScore() = opt.computeMaximumScaledPowerRationalScore();
      tao.optimizeBLMVM(sol, hi, lo, mode == 0 ? scaled_only_fg : scaled_fg);
      evals[3 * l + mode] = (int)(hv.size() / (n + 1));
      opt.expScaling() = exp(sol[0]);
      if (mode == 0) {
        opt.top().powerScalar() = sol[1];
        opt.bottom().powerScalar() = sol[2];
      } else {
        int xi = 1;
        for (int i = 0; i < nb; i++, xi++) opt.bottom().powersMutable()[i] = sol[xi];
        for (int i = 0; i < nt; i++, xi++) opt.top().powersMutable()[i] = sol[xi];
        opt.top().powerScalar() = sol[n - 2];
        opt.bottom().powerScalar() = sol[n - 1];
      }
    }
    double* o = out + (size_t)l * (nt + nb + 4);
    int k = 0;
    for (int i = 0; i < nb; i++) o[k++] = (double)opt.bottom().powersMutable()[i];
    for (int i = 0; i < nt; i++) o[k++] = (double)opt.top().powersMutable()[i];
    o[k++] = (double)opt.top().powerScalar();
    o[k++] = (double)opt.bottom().powerScalar();
    o[k++] = (double)opt.expScaling();
    o[k++] = (double)opt.computeScoreAP();
  }
  int k = 0;
  for (int i = 0; i < nt; i++)
    for (int c = 0; c < 4; c++) roots_out[k++] = (double)opt.top().roots()[i][c];
  for (int i = 0; i < nb; i++)
    for (int c = 0; c < 4; c++) roots_out[k++] = (double)opt.bottom().roots()[i][c];
  g_opt = nullptr;
  g_hist = nullptr;
}

// callConstrainedScaledOnlyTao (mode 0) or callConstrainedScaledTao (mode 1)
// of toothOptimizer (toothOptimizer.cpp:136-229) on the map `a`, grid and
// weight field, with maxIterations max_it.  out gets the final bottom powers,
// top powers, sigma_top, sigma_bottom and expScaling; hist (capacity
// hist_cap doubles) every evaluation as {f, state...}.  Returns the number
// of evaluations.
int ref_tanh_fit(int mode, const MapArgs* a, const int* res, const double* center,
                 const double* lengths, double slice, int max_it, const int* wres,
                 const double* wcenter, const double* wlengths, const double* weights,
                 double* out, double* hist, int hist_cap) {
  OPTIMIZE_3D opt(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                  VEC3F(lengths[0], lengths[1], lengths[2]));
  opt.top() = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  opt.bottom() = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  opt.maxIterations() = max_it;
  opt.expScaling() = a->s;
  opt.slice() = slice;
  FIELD_3D w(wres[0], wres[1], wres[2], VEC3F(wcenter[0], wcenter[1], wcenter[2]),
             VEC3F(wlengths[0], wlengths[1], wlengths[2]));
  for (int i = 0; i < w.totalCells(); i++) w[i] = weights[i];
  opt.weightField() = w;
  std::vector<double> hv;
  g_opt = &opt;
  g_hist = &hv;
  const int nt = a->nt, nb = a->nb;
  const int n = mode == 0 ? 3 : 3 + nt + nb;
  VECTOR sol(n);
  sol[0] = log(opt.expScaling());
  if (mode == 0) {
    sol[1] = opt.top().powerScalar();
    sol[2] = opt.bottom().powerScalar();
  } else {
    int xi = 1;
    for (int i = 0; i < nb; i++, xi++) sol[xi] = opt.bottom().powersMutable()[i];
    for (int i = 0; i < nt; i++, xi++) sol[xi] = opt.top().powersMutable()[i];
    sol[n - 2] = opt.top().powerScalar();
    sol[n - 1] = opt.bottom().powerScalar();
  }
  VECTOR hi = VECTOR::Constant(n, FLT_MAX);
  VECTOR lo = VECTOR::Zero(n);
  lo[0] = -FLT_MAX;
  TAO_SOLVER tao;
  tao.SetTolerances(1e-8, 1e-8, 1e-8, 1e-8, 0);
  tao.optimizeBLMVM(sol, hi, lo, mode == 0 ? scaled_only_fg : scaled_fg);
  // the caller's copy-back
  opt.expScaling() = exp(sol[0]);
  if (mode == 0) {
    opt.top().powerScalar() = sol[1];
    opt.bottom().powerScalar() = sol[2];
  } else {
    int xi = 1;
    for (int i = 0; i < nb; i++, xi++) opt.bottom().powersMutable()[i] = sol[xi];
    for (int i = 0; i < nt; i++, xi++) opt.top().powersMutable()[i] = sol[xi];
    opt.top().powerScalar() = sol[n - 2];
    opt.bottom().powerScalar() = sol[n - 1];
  }
  int k = 0;
  for (int i = 0; i < nb; i++) out[k++] = (double)opt.bottom().powersMutable()[i];
  for (int i = 0; i < nt; i++) out[k++] = (double)opt.top().powersMutable()[i];
  out[k++] = (double)opt.top().powerScalar();
  out[k++] = (double)opt.bottom().powerScalar();
  out[k++] = (double)opt.expScaling();
  const int evals = (int)(hv.size() / (n + 1));
  for (size_t i = 0; i < hv.size() && (int)i < hist_cap; i++) hist[i] = hv[i];
  g_opt = nullptr;
  g_hist = nullptr;
  return evals;
}

int ref_sizeof_real() { return (int)sizeof(Real); }

void ref_mt_rand(unsigned seed, int n, double* out) {
  MERSENNETWISTER mt(seed);
  for (int i = 0; i < n; i++) out[i] = mt.rand();
}

void ref_quat_pow(const double* q, double e, double* out) {
  QUATERNION r = QUATERNION(q[0], q[1], q[2], q[3]).pow(e);
  for (int c = 0; c < 4; c++) out[c] = (double)r[c];
}

// Escape-time field with a parameterised escape radius.
void ref_field_escape(const MapArgs* a, const int* res, const double* center,
                      const double* lengths, const double* rot, double slice, int max_it,
                      double escape, double* out) {
  POLYNOMIAL_4D top = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  POLYNOMIAL_4D bottom = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  FIELD_3D grid(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                VEC3F(lengths[0], lengths[1], lengths[2]));
  grid.rotation() = QUATERNION(rot[0], rot[1], rot[2], rot[3]);
  const Real s = a->s;
#pragma omp parallel for schedule(dynamic)
  for (int z = 0; z < res[2]; z++)
    for (int y = 0; y < res[1]; y++)
      for (int x = 0; x < res[0]; x++) {
        VEC3F point = grid.cellCenter(x, y, z);
        QUATERNION iterate(point[0], point[1], point[2], (Real)slice);
        Real magnitude = iterate.magnitude();
        int totalIterations = 0;
        while (magnitude < escape && totalIterations < max_it) {
          QUATERNION topEval = top.evaluateScaledPowerFactored(iterate);
          if (bottom.totalRoots() > 0) {
            QUATERNION bottomEval = bottom.evaluateScaledPowerFactored(iterate);
            iterate = (topEval / bottomEval);
          } else
            iterate = topEval;
          iterate *= s;
          magnitude = iterate.magnitude();
          totalIterations++;
          if (magnitude < 10.0 * REAL_MIN) totalIterations = max_it;
        }
        out[(size_t)z * res[0] * res[1] + (size_t)y * res[0] + x] = (double)log(magnitude);
      }
}

// The unmodified OPTIMIZE_3D::computeLogScaledPowerRationalMap (escape 2000).
void ref_field_map(const MapArgs* a, const int* res, const double* center, const double* lengths,
                   double slice, int max_it, double* out) {
  OPTIMIZE_3D opt(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                  VEC3F(lengths[0], lengths[1], lengths[2]));
  opt.top() = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  opt.bottom() = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  opt.maxIterations() = max_it;
  opt.expScaling() = a->s;
  opt.slice() = slice;
  opt.computeLogScaledPowerRationalMap(false);
  FIELD_3D& f = opt.fractal();
  for (int i = 0; i < f.totalCells(); i++) out[i] = (double)f[i];
}

// Streaming nonlinear marching cubes: TRIANGLE_MESH's 11-argument
// constructor (TRIANGLE_MESH.cpp:84-101).
int ref_mesh_stream(const MapArgs* a, const int* res, const double* center, const double* lengths,
                    const double* rot, double slice, int max_it, double iso, double* verts,
                    int max_v, int* tris, int max_t, int* nv, int* nt) {
  char path[] = "/tmp/qjref_edgecacheXXXXXX";
  int fd = mkstemp(path);
  if (fd < 0) return -2;
  close(fd);
  unlink(path);  // the constructor must not find a cache
  int rc;
  {
    TRIANGLE_MESH mesh(VEC3F(center[0], center[1], center[2]),
                       VEC3F(lengths[0], lengths[1], lengths[2]), VEC3I(res[0], res[1], res[2]),
                       make_poly(a->nt, a->troots, a->tpows, a->tsig),
                       make_poly(a->nb, a->broots, a->bpows, a->bsig), a->s, max_it, slice, iso,
                       QUATERNION(rot[0], rot[1], rot[2], rot[3]), std::string(path));
    rc = export_mesh(mesh, verts, max_v, tris, max_t, nv, nt);
  }
  unlink(path);
  return rc;
}

// Nonlinear marching cubes on a stored field (TRIANGLE_MESH.cpp:62-76).
int ref_mesh_field_nonlinear(const MapArgs* a, const int* res, const double* center,
                             const double* lengths, const double* field, double slice, int max_it,
                             double iso, double* verts, int max_v, int* tris, int max_t, int* nv,
                             int* nt) {
  FIELD_3D f(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
             VEC3F(lengths[0], lengths[1], lengths[2]));
  for (int i = 0; i < f.totalCells(); i++) f[i] = field[i];
  TRIANGLE_MESH mesh(f, make_poly(a->nt, a->troots, a->tpows, a->tsig),
                     make_poly(a->nb, a->broots, a->bpows, a->bsig), a->s, max_it, slice, iso);
  return export_mesh(mesh, verts, max_v, tris, max_t, nv, nt);
}

// Linear marching cubes on a stored field (TRIANGLE_MESH.cpp:48-57).
int ref_mesh_linear(const int* res, const double* center, const double* lengths,
                    const double* field, double* verts, int max_v, int* tris, int max_t, int* nv,
                    int* nt) {
  FIELD_3D f(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
             VEC3F(lengths[0], lengths[1], lengths[2]));
  for (int i = 0; i < f.totalCells(); i++) f[i] = field[i];
  TRIANGLE_MESH mesh(f);
  return export_mesh(mesh, verts, max_v, tris, max_t, nv, nt);
}

// Tanh-weighted score and its analytic gradients through the reference's
// OPTIMIZE_3D: computeScoreAP, computeExpGradientAP, computeBottomGradientAP,
// computeTopGradientAP and the two bulk scalar gradients, in the gradient
// layout of toothOptimizer's FormScaledFunctionGradient
// (projects/toothOptimizer/toothOptimizer.cpp:65-109).
double ref_tanh_score_grad(const MapArgs* a, const int* res, const double* center,
                           const double* lengths, double slice, int max_it, const int* wres,
                           const double* wcenter, const double* wlengths, const double* weights,
                           double* grad, double* field) {
  OPTIMIZE_3D opt(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                  VEC3F(lengths[0], lengths[1], lengths[2]));
  opt.top() = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  opt.bottom() = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  opt.maxIterations() = max_it;
  opt.expScaling() = a->s;
  opt.slice() = slice;
  FIELD_3D w(wres[0], wres[1], wres[2], VEC3F(wcenter[0], wcenter[1], wcenter[2]),
             VEC3F(wlengths[0], wlengths[1], wlengths[2]));
  for (int i = 0; i < w.totalCells(); i++) w[i] = weights[i];
  opt.weightField() = w;
  const double score = (double)opt.computeScoreAP();
  int k = 0;
  grad[k++] = (double)opt.computeExpGradientAP();
  for (int i = 0; i < a->nb; i++) grad[k++] = (double)opt.computeBottomGradientAP(i);
  for (int i = 0; i < a->nt; i++) grad[k++] = (double)opt.computeTopGradientAP(i);
  grad[k++] = (double)opt.computeTopBulkScalarGradientAP();
  grad[k++] = (double)opt.computeBottomBulkScalarGradientAP();
  FIELD_3D& f = opt.fractal();
  for (int i = 0; i < f.totalCells(); i++) field[i] = (double)f[i];
  return score;
}

// The escape loop of TRIANGLE_MESH::computeLagrangeNonlinearSlice
// (TRIANGLE_MESH.cpp:281-322) over a whole grid, escape as a parameter:
// RATIONAL_4D::evaluateLagrange, then the scale.
void ref_field_lagrange(const MapArgs* a, const int* res, const double* center,
                        const double* lengths, const double* rot, double slice, int max_it,
                        double escape, double* out) {
  POLYNOMIAL_4D top = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  POLYNOMIAL_4D bottom = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  FIELD_3D grid(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                VEC3F(lengths[0], lengths[1], lengths[2]));
  grid.rotation() = QUATERNION(rot[0], rot[1], rot[2], rot[3]);
  const Real s = a->s;
#pragma omp parallel for schedule(dynamic)
  for (int z = 0; z < res[2]; z++) {
    RATIONAL_4D rational(top, bottom);
    for (int y = 0; y < res[1]; y++)
      for (int x = 0; x < res[0]; x++) {
        VEC3F point = grid.cellCenter(x, y, z);
        QUATERNION iterate(point[0], point[1], point[2], (Real)slice);
        Real magnitude = iterate.magnitude();
        int totalIterations = 0;
        while (magnitude < escape && totalIterations < max_it) {
          iterate = rational.evaluateLagrange(iterate);
          iterate *= s;
          magnitude = iterate.magnitude();
          totalIterations++;
          if (magnitude < 10.0 * REAL_MIN) totalIterations = max_it;
        }
        out[(size_t)z * res[0] * res[1] + (size_t)y * res[0] + x] = (double)log(magnitude);
      }
  }
}

// The Lagrange streaming mesher: TRIANGLE_MESH's 10-argument constructor
// (TRIANGLE_MESH.cpp:106-123, computeLagrangeNonlinearMarchingCubesLowMemoryHuge).
int ref_mesh_lagrange(const MapArgs* a, const int* res, const double* center,
                      const double* lengths, const double* rot, double slice, int max_it,
                      double iso, double* verts, int max_v, int* tris, int max_t, int* nv,
                      int* nt) {
  TRIANGLE_MESH mesh(VEC3F(center[0], center[1], center[2]),
                     VEC3F(lengths[0], lengths[1], lengths[2]), VEC3I(res[0], res[1], res[2]),
                     make_poly(a->nt, a->troots, a->tpows, a->tsig),
                     make_poly(a->nb, a->broots, a->bpows, a->bsig), a->s, max_it, slice, iso,
                     QUATERNION(rot[0], rot[1], rot[2], rot[3]));
  return export_mesh(mesh, verts, max_v, tris, max_t, nv, nt);
}

// OPTIMIZE_3D's central-difference root gradients, unmodified: kind 0
// computeLogRationalCenteredGradient (OPTIMIZE_3D.cpp:2872-2951), 1
// computeLogRationalBottomCenteredGradient (:2956-3008), 2
// computeCenteredGradient (:2761-2812).  The distance and curvature fields
// share the fractal's grid, as setScoreFields makes them; *score gets the
// unmoved map's score (computeLogRationalScore / ...BottomScore / computeScore).
void ref_centered_gradient(const MapArgs* a, const int* res, const double* center,
                           const double* lengths, double slice, int max_it, int kind,
                           const double* dist, const double* curv, double* grad, double* score) {
  OPTIMIZE_3D opt(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                  VEC3F(lengths[0], lengths[1], lengths[2]));
  opt.top() = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  opt.bottom() = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  opt.maxIterations() = max_it;
  opt.expScaling() = a->s;
  opt.slice() = slice;
  FIELD_3D d(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
             VEC3F(lengths[0], lengths[1], lengths[2]));
  for (int i = 0; i < d.totalCells(); i++) d[i] = dist[i];
  opt.distanceField() = d;
  FIELD_3D c = d;
  if (curv)
    for (int i = 0; i < c.totalCells(); i++) c[i] = curv[i];
  opt.curvatureField() = c;
  VECTOR g = kind == 0   ? opt.computeLogRationalCenteredGradient()
             : kind == 1 ? opt.computeLogRationalBottomCenteredGradient()
                         : opt.computeCenteredGradient();
  for (int i = 0; i < (int)g.size(); i++) grad[i] = (double)g[i];
  FIELD_3D f = opt.fractal();
  *score = (double)(kind == 0   ? opt.computeLogRationalScore(opt.top(), opt.bottom(), f)
                    : kind == 1 ? opt.computeLogRationalBottomScore(opt.bottom(), f)
                                : opt.computeScore(opt.top(), f));
}

// FIELD_3D::invertedDistance / invertedDistanceNormalized (FIELD_3D.cpp:5241-5352).
void ref_inverted_distance(const int* res, const double* center, const double* lengths,
                           const double* dist, int normalized, double* out) {
  FIELD_3D d(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
             VEC3F(lengths[0], lengths[1], lengths[2]));
  for (int i = 0; i < d.totalCells(); i++) d[i] = dist[i];
  FIELD_3D w = normalized ? d.invertedDistanceNormalized() : d.invertedDistance();
  for (int i = 0; i < w.totalCells(); i++) out[i] = (double)w[i];
}

// OPTIMIZE_3D::estimateConformalRadius (OPTIMIZE_3D.cpp:4693-4772): returns
// the lowest score; *exp_scaling = the _expScaling it leaves behind.
double ref_conformal_radius(const MapArgs* a, const int* res, const double* center,
                            const double* lengths, double slice, const int* dres,
                            const double* dcenter, const double* dlengths, const double* dist,
                            double* exp_scaling) {
  OPTIMIZE_3D opt(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                  VEC3F(lengths[0], lengths[1], lengths[2]));
  opt.top() = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  opt.bottom() = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  opt.expScaling() = a->s;
  opt.maxIterations() = 7;
  opt.slice() = slice;
  FIELD_3D d(dres[0], dres[1], dres[2], VEC3F(dcenter[0], dcenter[1], dcenter[2]),
             VEC3F(dlengths[0], dlengths[1], dlengths[2]));
  for (int i = 0; i < d.totalCells(); i++) d[i] = dist[i];
  opt.distanceField() = d;
  const double score = (double)opt.estimateConformalRadius();
  *exp_scaling = (double)opt.expScaling();
  return score;
}

// OPTIMIZE_3D::write (OPTIMIZE_3D.cpp:3253-3297) of a state: the map, the
// fractal on (res, center, lengths), distance and curvature on (dres, ...).
void ref_o3d_write(const char* path, const MapArgs* a, const int* res, const double* center,
                   const double* lengths, const double* fractal, const int* dres,
                   const double* dcenter, const double* dlengths, const double* dist,
                   const double* curv) {
  OPTIMIZE_3D opt(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
                  VEC3F(lengths[0], lengths[1], lengths[2]));
  opt.top() = make_poly(a->nt, a->troots, a->tpows, a->tsig);
  opt.bottom() = make_poly(a->nb, a->broots, a->bpows, a->bsig);
  opt.expScaling() = a->s;
  for (int i = 0; i < opt.fractal().totalCells(); i++) opt.fractal()[i] = fractal[i];
  FIELD_3D d(dres[0], dres[1], dres[2], VEC3F(dcenter[0], dcenter[1], dcenter[2]),
             VEC3F(dlengths[0], dlengths[1], dlengths[2]));
  FIELD_3D c = d;
  for (int i = 0; i < d.totalCells(); i++) {
    d[i] = dist[i];
    c[i] = curv[i];
  }
  opt.distanceField() = d;
  opt.curvatureField() = c;
  opt.write(std::string(path));
}

// OPTIMIZE_3D::read (OPTIMIZE_3D.cpp:3302-3360) of a state: counts,
// roots (w,x,y,z), powers, power scalars, expScaling; the fractal and the
// distance field data.
void ref_o3d_read(const char* path, int* counts, double* troots, double* tpows, double* broots,
                  double* bpows, double* scalars, double* fractal, double* dist) {
  OPTIMIZE_3D opt;
  opt.read(std::string(path));
  const POLYNOMIAL_4D& t = opt.top();
  const POLYNOMIAL_4D& b = opt.bottom();
  counts[0] = t.totalRoots();
  counts[1] = b.totalRoots();
  for (int i = 0; i < t.totalRoots(); i++) {
    for (int c = 0; c < 4; c++) troots[4 * i + c] = (double)t.roots()[i][c];
    tpows[i] = (double)t.powers()[i];
  }
  for (int i = 0; i < b.totalRoots(); i++) {
    for (int c = 0; c < 4; c++) broots[4 * i + c] = (double)b.roots()[i][c];
    bpows[i] = (double)b.powers()[i];
  }
  scalars[0] = (double)t.powerScalar();
  scalars[1] = (double)b.powerScalar();
  scalars[2] = (double)opt.expScaling();
  for (int i = 0; i < opt.fractal().totalCells(); i++) fractal[i] = (double)opt.fractal()[i];
  for (int i = 0; i < opt.distanceField().totalCells(); i++)
    dist[i] = (double)opt.distanceField()[i];
}

// FIELD_3D::write(string) of a field (FIELD_3D.cpp:280-300, 4371-4393).
void ref_field_write(const char* path, const int* res, const double* center,
                     const double* lengths, const double* data) {
  FIELD_3D f(res[0], res[1], res[2], VEC3F(center[0], center[1], center[2]),
             VEC3F(lengths[0], lengths[1], lengths[2]));
  for (int i = 0; i < f.totalCells(); i++) f[i] = data[i];
  f.write(std::string(path));
}

// A TRIANGLE_MESH loaded through its own raw reader (TRIANGLE_MESH::read,
// TRIANGLE_MESH.cpp:4527-4553), then written by writeOBJ (:2762-2800) and by
// write(FILE*) (:4502-4522).
int ref_mesh_write(const double* verts, int nv, const int* tris, int nt, const char* obj_path,
                   const char* raw_path) {
  std::vector<char> buf(8 + (size_t)nv * 24 + (size_t)nt * 12);
  std::memcpy(buf.data(), &nv, 4);
  std::memcpy(buf.data() + 4, &nt, 4);
  std::memcpy(buf.data() + 8, verts, (size_t)nv * 24);
  std::memcpy(buf.data() + 8 + (size_t)nv * 24, tris, (size_t)nt * 12);
  FILE* in = fmemopen(buf.data(), buf.size(), "rb");
  if (!in) return -1;
  TRIANGLE_MESH mesh;
  mesh.read(in);
  std::fclose(in);
  mesh.writeOBJ(std::string(obj_path));
  FILE* out = std::fopen(raw_path, "wb");
  if (!out) return -2;
  mesh.write(out);
  std::fclose(out);
  return 0;
}

}  // extern "C"
