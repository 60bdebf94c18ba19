// The BLMVM minimiser (blmvm.cpp) for in-library callers.
#pragma once
#include <functional>

#include "../../include/quijibo_gpu.h"

namespace qj {
namespace blmvm {

// f(x) and its gradient into *f, g; non-zero stops the solver with that code
using Objective = std::function<int(const double* x, double* f, double* g)>;
// after each iteration; non-zero ends the run (CONVERGED_USER)
using Monitor = std::function<int(int iter, double f, double gnorm, const double* x)>;

// TAO_SOLVER's SOLVER_STATE codes (src/TOUPEE/TAO_SOLVER.h:62-81)
enum Reason {
  CONTINUE_ITERATING = 0,
  CONVERGED_FATOL = 1,
  CONVERGED_FRTOL = 2,
  CONVERGED_GATOL = 3,
  CONVERGED_GRTOL = 4,
  CONVERGED_GTTOL = 5,
  CONVERGED_MINF = 7,
  CONVERGED_USER = 8,
  DIVERGED_MAXITS = -2,
  DIVERGED_NAN = -4,
  DIVERGED_LS_FAILURE = -6,
};

// defaults: TAO_SOLVER's constructor (TAO_SOLVER.cpp:40-63) with the
// tolerances toothOptimizer sets (toothOptimizer.cpp:150-160)
struct Settings {
  int max_it = 2000;
  int ls_max_funcs = 30;
  double fatol = 1e-8, frtol = 1e-8, gatol = 1e-8, grtol = 1e-8, gttol = 0.0;
};

struct Stats {
  int reason = CONTINUE_ITERATING;
  int iterations = 0;
  int evaluations = 0;
  int grad_steps = 0;
  int resets = 0;
  double f = 0.0;
  double gnorm = 0.0;
};

inline Settings settings_from(const qjg_blmvm_settings& s) {
  Settings o;
  o.max_it = s.max_it;
  o.ls_max_funcs = s.ls_max_funcs;
  o.fatol = s.fatol;
  o.frtol = s.frtol;
  o.gatol = s.gatol;
  o.grtol = s.grtol;
  o.gttol = s.gttol;
  return o;
}

inline void settings_to(const Settings& s, qjg_blmvm_settings* o) {
  o->max_it = s.max_it;
  o->ls_max_funcs = s.ls_max_funcs;
  o->fatol = s.fatol;
  o->frtol = s.frtol;
  o->gatol = s.gatol;
  o->grtol = s.grtol;
  o->gttol = s.gttol;
}

inline void stats_to(const Stats& s, qjg_blmvm_stats* o) {
  o->reason = s.reason;
  o->iterations = s.iterations;
  o->evaluations = s.evaluations;
  o->grad_steps = s.grad_steps;
  o->resets = s.resets;
  o->pad_ = 0;
  o->f = s.f;
  o->gnorm = s.gnorm;
}

// Minimise over lower <= x <= upper from x_io (the solution is written
// back).  Returns 0 or the first non-zero objective status.
int minimize(int n, double* x_io, const double* lower, const double* upper, const Objective& fg,
             const Monitor& monitor, const Settings& st, Stats& stats);

}  // namespace blmvm
}  // namespace qj
