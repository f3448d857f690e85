// newton_control.h -- the per-instance Newton / line-search state machine.
//
// One device thread owns one instance's NState and advances it between the
// node- and element-parallel kernels.  The transitions restate, step for step:
//   OptimSolver::SolveFull          source/PhySim/Solvers/OptimSolver.cpp:163-311
//   OptimSolver_USQP_LS::SolveStepInternal  source/PhySim/Solvers/OptimSolver_USQP_LS.cpp:18-68
//   OptimSolver::ComputeStep        OptimSolver.cpp:313-352 (step clamp to maxStepSize)
//   OptimSolver::LineSearch_Simple  OptimSolver.cpp:688-736
//   OptimSolver::UpdateStepResult   OptimSolver.cpp:402-466
//   regularisation retry loop       source/PhySim/Solvers/LinearSolver_EigenCG.cpp:67-122,
//                                   (a truncated FP32 solve, LIN_TRUNCATED, is kept as is)
//                                   LinearSolver.cpp:57-66 (regT = 1e-6 ||A||_F, cumulative
//                                   shift regT * 10^(i-1) at trial i)
// The header is plain C++ so the same code is exercised on the host by the tests.
#pragma once

#include <math.h>

#include "phx_types.h"

namespace phx {

constexpr double kBackFactor = 1e2;  // restart points of the FP64 finish: ||g|| above this x tolerance

enum OSResult : int32_t { OS_ONGOING = 0, OS_SUCCESS = 1, OS_MINSTEP = 2, OS_MINIMPR = 3,
                          OS_FAILURE = 4, OS_MAXITER = 5, OS_NONDESC = 6 };

// OptimProblem_BasicStatic::IsFullyConstrained (OptimProblem_BasicStatic.cpp:119-121): every
// boundary condition at its last stage (Simulable::BoundaryConditionsLoaded); always true for
// the dynamic problem (OptimProblem_BasicDynamic.cpp:117-119).
PHX_HD inline bool ctl_fully_constrained(const NState& s, const DevOpts& o) {
  return o.dynamic || o.num_stages <= 1 || s.stage >= o.num_stages;
}

// SolveFull's decisions after one SolveStep; returns the next phase.  Its stop rules apply
// only while the problem is fully constrained (OptimSolver.cpp:213); before that, only the
// iteration limit ends a solve.
PHX_HD inline int32_t ctl_post_step(NState& s, const DevOpts& o) {
  bool brk = false;
  if (!ctl_fully_constrained(s, o)) {
    if (s.it + 1 > o.num_max_iters) {
      s.result = OS_MAXITER;
      return PH_DONE;
    }
    return PH_ITER;
  }
  if (s.result == OS_NONDESC) {
    if (!o.try_steepest) brk = true;
    else if (s.steepest) brk = true;
    else s.steepest = 1;
  }
  if (!brk && s.result == OS_MINIMPR) {
    if (s.min_impr_count == o.min_impr_max_count) brk = true;
    else if (o.try_steepest) s.steepest = !s.steepest;
  }
  if (!brk && s.result == OS_MINSTEP) {
    if (s.min_step_count == o.min_step_max_count) brk = true;
    else if (o.try_steepest) s.steepest = !s.steepest;
  }
  if (!brk && s.result == OS_SUCCESS) {
    if (s.opt <= s.tol_eff) brk = true;
    else s.result = OS_ONGOING;
  }
  if (!brk && s.result == OS_ONGOING) s.steepest = 0;
  if (!brk && s.it + 1 > o.num_max_iters) {
    s.result = OS_MAXITER;
    brk = true;
  }
  if (brk) {
    if (o.dynamic) s.vecop |= VO_VEL;
    return PH_DONE;
  }
  return PH_ITER;
}

// Moves to the next device phase, through a vector op when one is pending.
PHX_HD inline void ctl_goto(NState& s, int32_t next) {
  if (s.vecop) {
    s.next_phase = next;
    s.phase = PH_VEC;
  } else {
    s.phase = next;
  }
}

// Relative tolerance of this Newton step's linear solve.  The plain FP64 path keeps the
// reference's fixed ls_tol_max_error (LinearSolver_EigenCG with lsTolMaxError).  The FP32
// path solves inexactly with Eisenstat-Walker forcing terms (choice 2: gamma = 0.9,
// alpha = 2, safeguarded, eta_max = 0.1), never tighter than needed to reach the
// nonlinear tolerance and never tighter than ls_tol_max_error; the FP64 gradient and
// the nonlinear test decide convergence.
PHX_HD inline double ctl_forcing(NState& s, const DevOpts& o) {
  if (o.precision == 0) return o.ls_tol_max_error;
  const double eta_max = 0.1, gamma = 0.9;
  double eta;
  if (s.opt_prev <= 0.0 || s.eta <= 0.0) {
    eta = eta_max;
  } else {
    double r = s.opt / s.opt_prev;
    eta = gamma * r * r;
    double safe = gamma * s.eta * s.eta;
    if (safe > 0.1 && safe > eta) eta = safe;
  }
  if (eta > eta_max) eta = eta_max;
  double need = (s.opt > 0.0) ? 0.5 * s.tol_eff / s.opt : eta_max;
  if (eta < need) eta = need;
  if (eta > eta_max) eta = eta_max;
  if (eta < o.ls_tol_max_error) eta = o.ls_tol_max_error;
  s.eta = eta;
  return eta;
}

// Start of SolveStepInternal (energy, gradient and ||g|| at x are known).
PHX_HD inline void ctl_iter_begin(NState& s, const DevOpts& o) {
  s.it++;
  if (s.opt0 < 0) {
    s.opt0 = s.opt;
    s.tol_eff = (o.tol_rel > 0.0 && o.tol_rel * s.opt0 > o.tol_max_error) ? o.tol_rel * s.opt0 : o.tol_max_error;
  }
  s.num_bis = 0;
  if (s.opt < s.tol_eff) {
    s.result = OS_SUCCESS;
    s.step_result = OS_SUCCESS;
    s.log_step = 0.0;
    s.log_pending = 1;
    ctl_goto(s, ctl_post_step(s, o));
    return;
  }
  int qp = s.steepest ? 0 : o.qp_solver;
  if (qp == 0) {
    // Steepest: dx = -g, so ||dx|| = ||g|| and dx . g = -||g||^2
    s.dx_norm = s.opt;
    s.dg = -s.opt * s.opt;
    s.scale = (s.dx_norm > o.max_step_size) ? o.max_step_size / s.dx_norm : 1.0;
    s.factor = 1.0;
    s.alpha_trial = s.scale * s.factor;
    s.purpose = 1;
    s.vecop = VO_STEEP | VO_TRIAL;
    ctl_goto(s, PH_EVAL);
  } else {
    s.reg_trial = 0;
    s.shift = 0.0;
    s.hess_count++;
    s.lin_tol = ctl_forcing(s, o);
    s.opt_prev = s.opt;
    s.phase = PH_HESS;
  }
}

// Solves a linear solver makes, the first unregularised: LinearSolverOptions::regIters
// (include/PhySim/Solvers/LinearSolver.h:32).  OptimSolver::Init never sets it from
// lsNumRegTrials (OptimSolver.cpp:59-62), whose loop in SolveStepInternal computes one step
// because ComputeStep always succeeds (OptimSolver_USQP_LS.cpp:53-55, OptimSolver.cpp:312-352).
constexpr int kLinRegIters = 10;

// After a linear solve: regularise and retry, or clamp the step and start the line search.
PHX_HD inline void ctl_lin_done(NState& s, const DevOpts& o) {
  bool bad = (s.lin_status == LIN_BREAKDOWN) || !(s.b_dot_dx >= 0.0) || !isfinite(s.dx_norm);
  if (bad && s.reg_trial + 1 < kLinRegIters) {
    s.reg_trial++;
    s.total_reg++;
    s.shift += s.regT * pow(10.0, (double)(s.reg_trial - 1));
    s.phase = PH_JACOBI;
    return;
  }
  s.scale = (s.dx_norm > o.max_step_size) ? o.max_step_size / s.dx_norm : 1.0;
  s.factor = 1.0;
  s.num_bis = 0;
  s.alpha_trial = s.scale * s.factor;
  s.dg = -s.b_dot_dx;  // b = -g
  s.purpose = 1;
  s.vecop = VO_TRIAL;
  ctl_goto(s, PH_EVAL);
}

// Acceptance test of a line-search trial with energy objNew at bisection factor f, the
// `if` inside each LineSearch_* loop (OptimSolver.cpp:688-884).  With dxIn = scale * dx the
// clamped step and g the gradient at the search's start:
//   None (0): always; Simple (1): objNew < obj;
//   Armijo (2): objNew <= obj + f * c1 * (dxIn / |dxIn|) . g;
//   WolfeWeak (3): objNew <= obj + f * c1 * m and -dxIn . gNew <= -c2 * m, m = dxIn . g;
//   WolfeStrong (4): both, and |dxIn . gNew| <= c2 * |m|.
// The Wolfe tests read dx . gNew of the trial (dg_eval), so those searches evaluate their
// trials one at a time, with gradients.
PHX_HD inline bool ctl_ls_accepts(const NState& s, const DevOpts& o, double objNew, double f) {
  switch (o.lsearch_type) {
    case 0:
      return true;
    case 2: {
      const double t = s.dx_norm > 0.0 ? o.lsearch_wolfe1 * (s.dg / s.dx_norm) : 0.0;
      return objNew <= s.obj + f * t;
    }
    case 3:
    case 4: {
      const double m = s.scale * s.dg, dgn = s.scale * s.dg_eval;
      bool ok = objNew <= s.obj + f * (o.lsearch_wolfe1 * m) && -dgn <= -o.lsearch_wolfe2 * m;
      if (o.lsearch_type == 4) ok = ok && fabs(dgn) <= o.lsearch_wolfe2 * fabs(m);
      return ok;
    }
    default:
      return objNew < s.obj;
  }
}

// A rejected line-search trial of energy objNew (the LineSearch_* loops, OptimSolver.cpp:
// 688-884): sets up the next, shorter trial and returns true, or applies the failure and
// returns false.  On failure the state is restored, and UpdateStepResult (OptimSolver.cpp:
// 404-430) judges the last trial: no improvement is NONDESC; an improvement that the
// Armijo / Wolfe tests still refused counts as a step of its size (MINIMPR, MINSTEP or
// ONGOING) although the restored state stays, so that the next step starts from it again.
PHX_HD inline bool ctl_ls_reject(NState& s, const DevOpts& o, double objNew) {
  const double stepCur = s.alpha_trial * s.dx_norm;
  s.factor *= o.lsearch_alpha;
  if (stepCur > o.tol_min_step && s.num_bis <= o.lsearch_num_try) {
    s.num_bis++;
    s.alpha_trial = s.scale * s.factor;
    return true;
  }
  const double impr = s.obj - objNew;
  if (impr > 0) {
    if (impr < o.tol_min_impr) {
      s.min_impr_count++;
      s.result = OS_MINIMPR;
    } else if (stepCur < o.tol_min_step) {
      s.min_step_count++;
      s.result = OS_MINSTEP;
    } else {  // SUCCESS or ONGOING there; the restored gradient is above the tolerance, so ONGOING
      s.result = OS_ONGOING;
      s.min_impr_count = 0;
      s.min_step_count = 0;
    }
  } else {
    s.result = OS_NONDESC;
  }
  s.step_result = s.result;
  s.total_bis += s.num_bis;
  s.log_step = stepCur;
  s.log_pending = 1;
  s.vecop = VO_RESTORE;
  ctl_goto(s, ctl_post_step(s, o));
  return false;
}

// Evaluates the current trial step.  Once two trials of a search were rejected (long
// searches are the rule there), the next ls_parallel trials (the same step lengths the
// one-at-a-time search would try) are evaluated together, energies only.
PHX_HD inline void ctl_ls_next(NState& s, const DevOpts& o) {
  const int K = o.ls_parallel > kLsK ? kLsK : o.ls_parallel;
  // only the Simple and Armijo tests read energies alone.  Screening Wolfe trials in batches
  // by the energy part of their test, then checking curvature one by one, was slower on the
  // 512-instance batch (318 against 410 solves/s one at a time): most trials that pass the
  // energy part fail the curvature part there
  const bool energy_only = o.lsearch_type == 1 || o.lsearch_type == 2;
  if (K > 1 && s.num_bis >= 2 && energy_only) {
    double f = s.factor;
    s.ls_a[0] = s.alpha_trial;
    for (int k = 1; k < K; ++k) {
      f *= o.lsearch_alpha;
      s.ls_a[k] = s.scale * f;
    }
    s.lsk = K;
    s.purpose = 2;
    s.phase = PH_EVALK;
    return;
  }
  s.vecop = VO_TRIAL;
  ctl_goto(s, PH_EVAL);
}

PHX_HD inline void ctl_lsk_check(NState& s, const DevOpts& o);

// Line-search trial evaluated: accept, bisect, or give up (LineSearch_Simple + UpdateStepResult).
PHX_HD inline void ctl_ls_check(NState& s, const DevOpts& o) {
  double objNew = s.E_eval;
  if (!ctl_ls_accepts(s, o, objNew, s.factor)) {
    if (ctl_ls_reject(s, o, objNew)) ctl_ls_next(s, o);
    return;
  }
  double impr = s.obj - objNew;
  double step = s.alpha_trial * s.dx_norm;
  double optNew = sqrt(s.gg_eval);
  if (!(impr > 0)) {
    // accepted without improvement (None, or Armijo / Wolfe along a non-descent direction):
    // NONDESC, and the trial stays applied; the next step starts from it
    s.result = OS_NONDESC;
    s.step_result = OS_NONDESC;
    s.obj = objNew;
    s.opt = optNew;
    s.total_bis += s.num_bis;
    s.log_step = step;
    s.log_pending = 1;
    s.vecop = VO_GCOPY | VO_SAVE;
    ctl_goto(s, ctl_post_step(s, o));
    return;
  }
  if (impr < o.tol_min_impr) {
    s.min_impr_count++;
    s.result = OS_MINIMPR;
  } else if (step < o.tol_min_step) {
    s.min_step_count++;
    s.result = OS_MINSTEP;
  } else if (optNew <= s.tol_eff) {
    s.result = OS_SUCCESS;
    s.min_impr_count = 0;
    s.min_step_count = 0;
  } else {
    s.result = OS_ONGOING;
    s.min_impr_count = 0;
    s.min_step_count = 0;
  }
  s.step_result = s.result;
  // the iterate being left becomes the FP64 finish's restart point while its gradient is
  // still well above the tolerance (an FP32 solve can stall inside the band where the
  // energy comparison no longer resolves a step)
  const int back = (s.opt > kBackFactor * s.tol_eff) ? VO_BACK : 0;
  s.obj = objNew;
  s.opt = optNew;
  s.total_bis += s.num_bis;
  s.log_step = step;
  s.log_pending = 1;
  s.vecop = VO_ACCEPT | VO_SAVE | back;
  ctl_goto(s, ctl_post_step(s, o));
}

// Line-search trials evaluated together (PH_EVALK, Simple and Armijo searches, whose tests
// read energies only): scans them in order with the rules of the one-at-a-time search, so
// it takes the same decisions: the first trial the test accepts is evaluated again with its
// gradient (PH_EVAL) and checked as usual; a rejected trial goes through ctl_ls_reject like
// a sequential one.
PHX_HD inline void ctl_lsk_check(NState& s, const DevOpts& o) {
  for (int k = 0; k < s.lsk; ++k) {
    // s.alpha_trial and s.factor are trial k's here (the same recurrence)
    if (ctl_ls_accepts(s, o, s.ls_e[k], s.factor)) {
      s.purpose = 1;
      s.vecop = VO_TRIAL;
      ctl_goto(s, PH_EVAL);
      return;
    }
    if (!ctl_ls_reject(s, o, s.ls_e[k])) return;  // the search failed at trial k
  }
  ctl_ls_next(s, o);
}

// Advances one instance until it needs device work or is done.
PHX_HD inline void ctl_advance(NState& s, const DevOpts& o) {
  for (int guard = 0; guard < 8; ++guard) {
    switch (s.phase) {
      case PH_START:
        s.it = 0;
        s.result = OS_SUCCESS;
        s.step_result = OS_ONGOING;
        s.steepest = 0;
        s.min_impr_count = 0;
        s.min_step_count = 0;
        s.total_bis = 0;
        s.total_reg = 0;
        s.total_sweeps = 0;
        s.pcg_total = 0;
        s.pcg_slices = 0;
        s.hess_count = 0;
        s.opt0 = -1.0;
        s.eta = 0.0;
        s.opt_prev = 0.0;
        s.log_count = 0;
        s.log_pending = 0;
        s.tol_eff = o.tol_max_error;
        s.purpose = 0;
        s.iter_staged = 0;
        s.vecop = o.dynamic ? VO_PRED : 0;
        if (o.dynamic && o.num_stages > 0 && s.stage < o.num_stages) {
          // OnSolveStart of the dynamic problem (OptimProblem_BasicDynamic.cpp:121-135): the
          // conditions' next stage, before the predictor overwrites every position (so only
          // the soft targets and stiffness of the stage take effect)
          s.stage++;
          if (o.stage_values) s.vecop |= VO_STAGE;
        }
        ctl_goto(s, PH_EVAL);
        return;
      case PH_EVAL_DONE:
        if (s.purpose == 3) {  // re-evaluated at the iteration start after a stage moved its targets
          s.obj = s.E_eval;
          s.opt = sqrt(s.gg_eval);
          s.vecop = VO_GNEW | VO_SAVE;
          s.next_phase = PH_ITER;
          s.phase = PH_VEC;
          return;
        }
        if (s.purpose == 0) {
          s.obj = s.E_eval;
          s.opt = sqrt(s.gg_eval);
          s.vecop = VO_GCOPY | VO_SAVE;
          s.next_phase = PH_ITER;
          s.phase = PH_VEC;
          return;
        }
        if (s.purpose == 2) ctl_lsk_check(s, o);
        else ctl_ls_check(s, o);
        if (s.phase == PH_ITER) continue;
        return;
      case PH_ITER:
        if (!o.dynamic && !s.iter_staged && o.num_stages > 0 && s.stage < o.num_stages) {
          // OnIterStart of the static problem: StepBoundaryConditions (Simulable.cpp:1496-1500)
          s.stage++;
          s.iter_staged = 1;
          if (o.stage_values) {  // new targets or stiffness: energy and gradient again
            s.purpose = 3;
            s.vecop = VO_STAGE;
            ctl_goto(s, PH_EVAL);
            return;
          }
        }
        s.iter_staged = 0;
        ctl_iter_begin(s, o);
        if (s.phase == PH_ITER) continue;
        return;
      case PH_LIN_DONE:
        ctl_lin_done(s, o);
        return;
      default:
        return;  // a device phase, a pending vector op, or done
    }
  }
}

}  // namespace phx
