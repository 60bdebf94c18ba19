// Bound-constrained limited-memory variable metric minimiser (BLMVM, Benson
// and Moré) with the Moré-Thuente line search, as QUIJIBO's TAO port
// (src/TOUPEE) runs it for toothOptimizer:
//
//   TAO_SOLVER::optimizeBLMVM        src/TOUPEE/TAO_SOLVER.cpp:72-341
//   TAO_SOLVER::DefaultConvergenceTest                  :695-790
//   BLMVM (the LMVM matrix)          src/TOUPEE/BLMVM.cpp:34-1055
//   LINE_SEARCH / MORE_THUENTE       src/TOUPEE/LINE_SEARCH.cpp, MORE_THUENTE.cpp
//
// Only the configuration the reference builds is restated: 5 stored pairs,
// Broyden diagonal scaling (phi = 1/8) rescaled by the scalar y's / y'Dy of
// the newest pair, no limiting, and a bounded Moré-Thuente search of at most
// 30 trial points.  The port's behaviour is kept where it differs from TAO:
// the search's step bounds and its last mcstep status carry over from one
// search to the next; its evaluation counters are never advanced (so the
// "too many evaluations" tests never fire); a search that stops on the
// bounded sufficient-decrease test reports no success, which BLMVM treats as
// a failed search; a twice-failed search leaves x at the last trial point.
//
// Rounding follows the reference's double build: every dot product and norm
// sums its terms in the order of Eigen 3.2's two-lane SSE2 reduction (below),
// and the file is compiled without FMA contraction, so given the same
// objective values the iterates are bit-identical to the reference's.
//
// The objective is a callback: for toothOptimizer it is one GPU pass of the
// tanh score and its gradients (tooth_api.cpp).  The solver's own work is
// O(n) host arithmetic on n <= 3 + QJG_MAX_ROOTS variables.
#include "qj_blmvm.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace qj {
namespace {

using Vec = std::vector<double>;

// Sum of c(i), i < n, in the order of Eigen 3.2's vectorised redux for
// dynamic double vectors on SSE2 (two lanes, two packets per trip): lane
// sums over even and odd indices of whole 4-blocks, then one more 2-packet,
// the two lanes added, then the odd tail.
template <class C>
double redux(int n, C c) {
  if (n < 2) return n == 1 ? c(0) : 0.0;
  const int n2 = n & ~1, n4 = n & ~3;
  double a0 = c(0), a1 = c(1);
  if (n2 > 2) {
    double b0 = c(2), b1 = c(3);
    for (int i = 4; i < n4; i += 4) {
      a0 += c(i);
      a1 += c(i + 1);
      b0 += c(i + 2);
      b1 += c(i + 3);
    }
    a0 += b0;
    a1 += b1;
    if (n2 > n4) {
      a0 += c(n4);
      a1 += c(n4 + 1);
    }
  }
  double r = a0 + a1;
  for (int i = n2; i < n; i++) r += c(i);
  return r;
}

double dot(const Vec& a, const Vec& b) {
  return redux((int)a.size(), [&](int i) { return a[i] * b[i]; });
}

double norm(const Vec& a) { return std::sqrt(dot(a, a)); }

// middle of three values (the reference sorts the three)
double mid3(double a, double b, double c) {
  return std::max(std::min(a, b), std::min(std::max(a, b), c));
}

// gp = g with the components that push x out through an active bound zeroed
// (VecBoundGradientProjection, BLMVM.cpp:958-983)
void project(const Vec& g, const Vec& x, const Vec& lo, const Vec& hi, Vec& gp) {
  for (size_t i = 0; i < x.size(); i++) {
    double v = g[i];
    if (v > 0 && x[i] <= lo[i])
      v = 0;
    else if (v < 0 && x[i] >= hi[i])
      v = 0;
    gp[i] = v;
  }
}

// ---- the LMVM matrix (BLMVM.cpp) --------------------------------------
class Lmvm {
 public:
  static constexpr int LM = 5;
  static constexpr double DELTA_MIN = 1e-7, DELTA_MAX = 100.0, PHI = 0.125;
  static constexpr double ZERO_SAFEGUARD = 1e-8;

  explicit Lmvm(int n) : n_(n), S_(LM + 1, Vec(n)), Y_(LM + 1, Vec(n)), D_(n), xprev_(n), gprev_(n) {
    rho_.assign(LM + 1, 0.0);
    beta_.assign(LM + 1, 0.0);
  }

  // SetDelta (BLMVM.cpp:1014-1019)
  void set_delta(double d) {
    delta_ = std::fabs(d);
    delta_ = delta_ > DELTA_MIN ? delta_ : DELTA_MIN;
    delta_ = delta_ < DELTA_MAX ? delta_ : DELTA_MAX;
  }

  // MatReset (BLMVM.cpp:105-144): forget the pairs, D = delta
  void reset() {
    for (int i = 0; i < LM; i++) rho_[i] = 0.0;
    rho_[0] = 1.0;
    std::fill(D_.begin(), D_.end(), delta_);
    iter_ = 0;
    lmnow_ = 0;
  }

  // Update (BLMVM.cpp:176-826) with the reference's scaling choices
  void update(const Vec& x, const Vec& g) {
    if (iter_ == 0) {
      reset();
    } else {
      Vec y(n_), s(n_);
      for (int i = 0; i < n_; i++) {
        y[i] = g[i] - gprev_[i];
        s[i] = x[i] - xprev_[i];
      }
      const double ys = dot(y, s);
      if (ys > 0.0) {  // the curvature test y's > eps y'y, eps = 0
        lmnow_ = std::min(lmnow_ + 1, LM);
        for (int i = LM - 1; i >= 0; --i) {
          S_[i + 1] = S_[i];
          Y_[i + 1] = Y_[i];
          rho_[i + 1] = rho_[i];
        }
        S_[0] = s;
        Y_[0] = y;
        rho_[0] = 1.0 / ys;
        broyden_scale(s, y, ys);
      }
    }
    iter_++;
    xprev_ = x;
    gprev_ = g;
  }

  // MatSolve (BLMVM.cpp:832-952): two-loop recursion around H0 = diag(D)
  void solve(const Vec& b, Vec& x) {
    if (lmnow_ < 1) rho_[0] = 1.0;
    x = b;
    for (int l = 0; l < lmnow_; ++l) {
      beta_[l] = dot(x, S_[l]) * rho_[l];
      const double c = -beta_[l];
      for (int i = 0; i < n_; i++) x[i] += c * Y_[l][i];
    }
    for (int i = 0; i < n_; i++) x[i] = x[i] * D_[i];
    for (int l = lmnow_ - 1; l >= 0; --l) {
      const double yq = dot(x, Y_[l]);
      const double c = beta_[l] - yq * rho_[l];
      for (int i = 0; i < n_; i++) x[i] += c * S_[l][i];
    }
  }

 private:
  // Broyden-class diagonal update of D from the newest pair, blended with
  // phi, then rescaled by ys / y'Dy (BLMVM.cpp:349-700, MatLMVM_Scale_Broyden
  // with MatLMVM_Rescale_Scalar, r_alpha = 1, r_beta = 0.5, history 1)
  void broyden_scale(const Vec& s, const Vec& y, double ys) {
    // (ys > 0 here, so its zero safeguard never applies)
    Vec P(n_), Q(n_), V(n_), W(n_), U(n_);
    for (int i = 0; i < n_; i++) {
      P[i] = 1.0 / D_[i];
      Q[i] = P[i];
      V[i] = y[i] * y[i];
      W[i] = s[i] * P[i];
    }
    double sDs = dot(W, s);
    if (sDs == 0.0) sDs = ZERO_SAFEGUARD;
    const double c1 = 1.0 / ys, c2 = -1.0 / sDs;
    const double c3 = 1.0 / ys + sDs / (ys * ys), c4 = -2.0 / ys;
    for (int i = 0; i < n_; i++) {
      const double ww = W[i] * W[i];
      P[i] += c1 * V[i];
      P[i] += c2 * ww;
      const double wy = W[i] * y[i];
      Q[i] += c3 * V[i];
      Q[i] += c4 * wy;
      U[i] = (1.0 - PHI) * P[i] + PHI * Q[i];
      U[i] = std::fabs(1.0 / U[i]);
    }
    // rescale: sigma = ys / (y' U y) with the newest pair
    for (int i = 0; i < n_; i++) V[i] = Y_[0][i] * U[i];
    const double yy_sum = dot(V, Y_[0]);
    const double sigma = ys / yy_sum;
    if (std::isfinite(sigma) && sigma != 0.0)
      for (int i = 0; i < n_; i++) U[i] *= sigma;
    D_ = U;
  }

  int n_;
  std::vector<Vec> S_, Y_;
  Vec rho_, beta_, D_, xprev_, gprev_;
  double delta_ = 1.0;
  int iter_ = 0, lmnow_ = 0;
};

// ---- the Moré-Thuente line search (MORE_THUENTE.cpp) ------------------
enum LsReason {
  LS_CONTINUE = 0,
  LS_SUCCESS = 1,
  LS_FAILED_INFORNAN = -1,
  LS_FAILED_ASCENT = -3,
  LS_HALTED_OTHER = 3,
  LS_HALTED_UPPERBOUND = 5,
  LS_HALTED_LOWERBOUND = 6,
  LS_HALTED_RTOL = 7,
};

class MoreThuente {
 public:
  static constexpr double FTOL = 1e-4, GTOL = 0.9, RTOL = 1e-10, XTRAPF = 4.0;

  MoreThuente(const Vec& lo, const Vec& hi, int max_funcs, const blmvm::Objective& fg)
      : lo_(lo), hi_(hi), max_funcs_(max_funcs), fg_(fg) {}

  // One search from x along s (projected onto the bounds first); on return
  // x, f, g hold the last trial point.  Returns the callback's status.
  int apply(Vec& x, double& f, Vec& g, Vec& s, double initstep, int& evals) {
    reason_ = LS_CONTINUE;
    const int n = (int)x.size();
    // bounded: drop the direction's components that leave through an active
    // bound, then bound the step (VecStepBoundInfo, LINE_SEARCH.cpp:54-96)
    for (int i = 0; i < n; i++) s[i] *= -1.0;
    project(s, x, lo_, hi_, s);
    for (int i = 0; i < n; i++) s[i] *= -1.0;
    double bmin = 1.0e300, bwolfe = 1.0e300, bmax = 0.0;
    for (int i = 0; i < n; i++) {
      double t;
      if (s[i] > 0)
        t = (hi_[i] - x[i]) / s[i];
      else if (s[i] < 0)
        t = (lo_[i] - x[i]) / s[i];
      else
        continue;
      bmin = std::min(t, bmin);
      if (bmin > 0) bwolfe = std::min(t, bwolfe);
      bmax = std::max(t, bmax);
    }
    stepmax_ = std::min(bmax, 1.0e15);

    const double dginit = dot(g, s);
    if (std::isnan(dginit) || std::isinf(dginit)) {
      reason_ = LS_FAILED_INFORNAN;
      return 0;
    }
    if (dginit >= 0.0) {
      reason_ = LS_FAILED_ASCENT;
      return 0;
    }
    bracket_ = false;
    bool stage1 = true;
    const double finit = f;
    const double dgtest = FTOL * dginit;
    double width = stepmax_ - stepmin_;  // stepmin_ as the previous search left it
    double width1 = width * 2.0;
    double stx = 0.0, fx = finit, dgx = dginit;
    double sty = 0.0, fy = finit, dgy = dginit;
    double step = initstep;
    Vec work(x);
    for (int it = 0; it < max_funcs_; it++) {
      if (bracket_) {
        stepmin_ = std::min(stx, sty);
        stepmax_ = std::max(stx, sty);
      } else {
        stepmin_ = stx;
        stepmax_ = step + XTRAPF * (step - stx);
      }
      step = std::max(step, stepmin_);
      step = std::min(step, stepmax_);
      if (stx != 0 && ((bracket_ && (step <= stepmin_ || step >= stepmax_)) ||
                       (bracket_ && (stepmax_ - stepmin_ <= RTOL * stepmax_)) || infoc_ == 0))
        step = stx;
      for (int i = 0; i < n; i++) work[i] = mid3(lo_[i], x[i] + step * s[i], hi_[i]);
      evals++;
      if (int rc = fg_(work.data(), &f, g.data())) return rc;
      double dg = (dot(g, work) - dot(g, x)) / step;
      if (std::isinf(f) || std::isnan(f) || std::isinf(dg) || std::isnan(dg)) {
        f = 1.0e100;
        dg = 1.0e100;
      }
      const double ftest1 = finit + step * dgtest;
      const double ftest2 = finit + step * dgtest * FTOL;
      if (f - ftest1 <= 1.0e-10 * std::fabs(finit) && std::fabs(dg) + GTOL * dginit <= 0.0) {
        reason_ = LS_SUCCESS;
        break;
      }
      if (f <= ftest2 && step >= bwolfe) break;  // accepted, but not reported as success
      if ((bracket_ && (step <= stepmin_ || step >= stepmax_)) || !infoc_) {
        reason_ = LS_HALTED_OTHER;
        break;
      }
      if (step == stepmax_ && f <= ftest1 && dg <= dgtest) {
        reason_ = LS_HALTED_UPPERBOUND;
        break;
      }
      if (step == stepmin_ && f >= ftest1 && dg >= dgtest) {
        reason_ = LS_HALTED_LOWERBOUND;
        break;
      }
      if (bracket_ && stepmax_ - stepmin_ <= RTOL * stepmax_) {
        reason_ = LS_HALTED_RTOL;
        break;
      }
      if (stage1 && f <= ftest1 && dg >= dginit * std::min(FTOL, GTOL)) stage1 = false;
      if (stage1 && f <= fx && f > ftest1) {
        // the modified function psi(t) = f(t) - f(0) - t ftol f'(0)
        double fm = f - step * dgtest;
        double fxm = fx - stx * dgtest;
        double fym = fy - sty * dgtest;
        double dgm = dg - dgtest;
        double dgxm = dgx - dgtest;
        double dgym = dgy - dgtest;
        mcstep(stx, fxm, dgxm, sty, fym, dgym, step, fm, dgm);
        fx = fxm + stx * dgtest;
        fy = fym + sty * dgtest;
        dgx = dgxm + dgtest;
        dgy = dgym + dgtest;
      } else {
        mcstep(stx, fx, dgx, sty, fy, dgy, step, f, dg);
      }
      if (bracket_) {
        if (std::fabs(sty - stx) >= 0.66 * width1) step = stx + 0.5 * (sty - stx);
        width1 = width;
        width = std::fabs(sty - stx);
      }
    }
    x = work;
    return 0;
  }

  int reason() const { return reason_; }

 private:
  // Safeguarded cubic/quadratic step and interval update of Moré and Thuente
  // (MINPACK-2 dcstep as in Nocedal's mcstep; MORE_THUENTE.cpp:91-318)
  void mcstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp,
              double fp, double dp) {
    infoc_ = 0;
    if (bracket_ && (stp <= std::min(stx, sty) || stp >= std::max(stx, sty))) return;
    if (dx * (stp - stx) >= 0.0) return;
    if (stepmax_ < stepmin_) return;
    const double sgnd = dp * (dx / std::fabs(dx));
    double stpf, stpc, stpq, theta, s, gamma, p, q, r;
    bool bound;
    if (fp > fx) {
      // case 1: higher function value; the minimum is bracketed
      infoc_ = 1;
      bound = true;
      theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
      s = std::max(std::max(std::fabs(theta), std::fabs(dx)), std::fabs(dp));
      const double ts = theta / s;
      gamma = s * std::sqrt(ts * ts - (dx / s) * (dp / s));
      if (stp < stx) gamma = -gamma;
      p = (gamma - dx) + theta;
      q = ((gamma - dx) + gamma) + dp;
      r = p / q;
      stpc = stx + r * (stp - stx);
      stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) * 0.5) * (stp - stx);
      stpf = std::fabs(stpc - stx) < std::fabs(stpq - stx) ? stpc : stpc + 0.5 * (stpq - stpc);
      bracket_ = true;
    } else if (sgnd < 0.0) {
      // case 2: lower value, derivatives of opposite sign; bracketed
      infoc_ = 2;
      bound = false;
      theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
      s = std::max(std::max(std::fabs(theta), std::fabs(dx)), std::fabs(dp));
      const double ts = theta / s;
      gamma = s * std::sqrt(ts * ts - (dx / s) * (dp / s));
      if (stp > stx) gamma = -gamma;
      p = (gamma - dp) + theta;
      q = ((gamma - dp) + gamma) + dx;
      r = p / q;
      stpc = stp + r * (stx - stp);
      stpq = stp + (dp / (dp - dx)) * (stx - stp);
      stpf = std::fabs(stpc - stp) > std::fabs(stpq - stp) ? stpc : stpq;
      bracket_ = true;
    } else if (std::fabs(dp) < std::fabs(dx)) {
      // case 3: lower value, same sign, derivative magnitude decreases
      infoc_ = 3;
      bound = true;
      theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
      s = std::max(std::max(std::fabs(theta), std::fabs(dx)), std::fabs(dp));
      const double ts = theta / s;
      gamma = s * std::sqrt(std::max(0.0, ts * ts - (dx / s) * (dp / s)));
      if (stp > stx) gamma = -gamma;
      p = (gamma - dp) + theta;
      q = (gamma + (dx - dp)) + gamma;
      r = p / q;
      if (r < 0.0 && gamma != 0.0)
        stpc = stp + r * (stx - stp);
      else if (stp > stx)
        stpc = stepmax_;
      else
        stpc = stepmin_;
      stpq = stp + (dp / (dp - dx)) * (stx - stp);
      if (bracket_)
        stpf = std::fabs(stp - stpc) < std::fabs(stp - stpq) ? stpc : stpq;
      else
        stpf = std::fabs(stp - stpc) > std::fabs(stp - stpq) ? stpc : stpq;
    } else {
      // case 4: lower value, same sign, derivative magnitude does not decrease
      infoc_ = 4;
      bound = false;
      if (bracket_) {
        theta = 3 * (fp - fy) / (sty - stp) + dy + dp;
        s = std::max(std::max(std::fabs(theta), std::fabs(dy)), std::fabs(dp));
        const double ts = theta / s;
        gamma = s * std::sqrt(ts * ts - (dy / s) * (dp / s));
        if (stp > sty) gamma = -gamma;
        p = (gamma - dp) + theta;
        q = ((gamma - dp) + gamma) + dy;
        r = p / q;
        stpf = stp + r * (sty - stp);
      } else {
        stpf = stp > stx ? stepmax_ : stepmin_;
      }
    }
    // the interval of uncertainty
    if (fp > fx) {
      sty = stp;
      fy = fp;
      dy = dp;
    } else {
      if (sgnd < 0.0) {
        sty = stx;
        fy = fx;
        dy = dx;
      }
      stx = stp;
      fx = fp;
      dx = dp;
    }
    stpf = std::min(stepmax_, stpf);
    stpf = std::max(stepmin_, stpf);
    stp = stpf;
    if (bracket_ && bound) {
      if (sty > stx)
        stp = std::min(stx + 0.66 * (sty - stx), stp);
      else
        stp = std::max(stx + 0.66 * (sty - stx), stp);
    }
  }

  const Vec& lo_;
  const Vec& hi_;
  int max_funcs_;
  const blmvm::Objective& fg_;
  int reason_ = LS_CONTINUE;
  bool bracket_ = false;
  int infoc_ = 1;
  double stepmin_ = 1.0e-20, stepmax_ = 1.0e20;
};

double initial_delta(double f, double gnorm) {
  return f != 0.0 ? 2.0 * std::fabs(f) / (gnorm * gnorm) : 2.0 / (gnorm * gnorm);
}

}  // namespace

namespace blmvm {

int minimize(int n, double* x_io, const double* lower, const double* upper, const Objective& fg,
             const Monitor& monitor, const Settings& st, Stats& stats) {
  stats = Stats{};
  Vec lo(lower, lower + n), hi(upper, upper + n), x(n);
  // project the start onto the bounds (TAO_SOLVER.cpp:105)
  for (int i = 0; i < n; i++) x[i] = mid3(lo[i], hi[i], x_io[i]);
  MoreThuente ls(lo, hi, st.ls_max_funcs, fg);
  Lmvm lmvm(n);
  Vec ug(n), g(n), d(n), xold, gold;
  double f = 0.0;
  int rc = fg(x.data(), &f, ug.data());
  stats.evaluations = 1;
  auto finish = [&](int code) {
    std::copy(x.begin(), x.end(), x_io);
    stats.f = f;
    return code;
  };
  if (rc) return finish(rc);
  project(ug, x, lo, hi, g);
  double gnorm = norm(g);
  stats.gnorm = gnorm;
  const double gnorm0 = gnorm;
  lmvm.set_delta(initial_delta(f, gnorm));

  int reason = CONTINUE_ITERATING;
  int iter = 0;
  while (reason == CONTINUE_ITERATING) {
    lmvm.update(x, g);
    lmvm.solve(ug, d);
    project(d, x, lo, hi, g);
    if (dot(ug, g) <= 0) {
      // not a descent direction: scaled gradient step from a fresh matrix
      stats.grad_steps++;
      lmvm.set_delta(initial_delta(f, gnorm));
      lmvm.reset();
      lmvm.update(x, ug);
      lmvm.solve(ug, d);
    }
    for (int i = 0; i < n; i++) d[i] *= -1.0;
    const double fold = f;
    xold = x;
    gold = ug;
    if ((rc = ls.apply(x, f, ug, d, 1.0, stats.evaluations))) return finish(rc);
    if (ls.reason() != 1) {
      // failed search: back to the old point, fresh matrix, gradient step
      stats.resets++;
      f = fold;
      x = xold;
      ug = gold;
      lmvm.set_delta(initial_delta(f, gnorm));
      lmvm.reset();
      lmvm.update(x, ug);
      lmvm.solve(ug, d);
      for (int i = 0; i < n; i++) d[i] *= -1.0;
      if ((rc = ls.apply(x, f, ug, d, 1.0, stats.evaluations))) return finish(rc);
      if (ls.reason() != 1) {
        reason = DIVERGED_LS_FAILURE;
        break;
      }
    }
    project(ug, x, lo, hi, g);
    gnorm = norm(g);
    stats.gnorm = gnorm;
    iter++;
    stats.iterations = iter;
    // DefaultConvergenceTest (TAO_SOLVER.cpp:695-790) with no constraints
    // and the step-tolerance test never true (step 1 against steptol 0)
    const double g2 = gnorm * gnorm;
    if (std::isinf(f) || std::isnan(f))
      reason = DIVERGED_NAN;
    else if (f <= -1e100)
      reason = CONVERGED_MINF;
    else if (g2 <= st.fatol)
      reason = CONVERGED_FATOL;
    else if (f != 0 && g2 / std::fabs(f) <= st.frtol)
      reason = CONVERGED_FRTOL;
    else if (gnorm <= st.gatol)
      reason = CONVERGED_GATOL;
    else if (f != 0 && std::fabs(gnorm / f) <= st.grtol)
      reason = CONVERGED_GRTOL;
    else if (gnorm0 != 0 && gnorm / gnorm0 <= st.gttol)
      reason = CONVERGED_GTTOL;
    else if (iter > st.max_it)
      reason = DIVERGED_MAXITS;
    if (monitor && monitor(iter, f, gnorm, x.data()) && reason == CONTINUE_ITERATING)
      reason = CONVERGED_USER;
  }
  stats.reason = reason;
  return finish(0);
}

}  // namespace blmvm
}  // namespace qj

extern "C" {

int qjg_blmvm(int32_t n, double* x, const double* lower, const double* upper, qjg_objective_fn fg,
              void* fg_user, qjg_monitor_fn monitor, void* monitor_user,
              const qjg_blmvm_settings* settings, qjg_blmvm_stats* stats) {
  if (n < 1 || !x || !lower || !upper || !fg) return QJG_ERR_ARG;
  for (int i = 0; i < n; i++)
    if (!(lower[i] <= upper[i])) return QJG_ERR_ARG;
  qj::blmvm::Settings st;
  if (settings) st = qj::blmvm::settings_from(*settings);
  if (st.max_it < 0 || st.ls_max_funcs < 1) return QJG_ERR_ARG;
  qj::blmvm::Objective obj = [&](const double* xx, double* f, double* g) {
    return fg(fg_user, n, xx, f, g);
  };
  qj::blmvm::Monitor mon;
  if (monitor)
    mon = [&](int it, double f, double gn, const double* xx) {
      return monitor(monitor_user, it, f, gn, xx);
    };
  qj::blmvm::Stats s;
  const int rc = qj::blmvm::minimize(n, x, lower, upper, obj, mon, st, s);
  if (stats) qj::blmvm::stats_to(s, stats);
  return rc;
}

void qjg_blmvm_defaults(qjg_blmvm_settings* out) {
  if (out) qj::blmvm::settings_to(qj::blmvm::Settings{}, out);
}

}  // extern "C"
