/*
 * phx_oracle.h -- CPU restatement of PhySim's tet-FEM Newton path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU path is
 * compared against (tests, the smoke check and the CPU-baseline leg of the
 * benchmark).  Nothing in the product links or calls it.
 *
 * Parity of the material laws is pinned against the reference's own generated
 * code (inc/Utils/Auto/FEMVol_{CoNH,StVK}_{Energy,Gradient,Hessian}.mcg)
 * through golden vectors committed under tests/golden/.  The Newton, line
 * search, assembly and linear-solver semantics are restated from the reference
 * sources cited beside each function in phx_oracle.cpp.
 */
#ifndef PHX_ORACLE_H
#define PHX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mesh {
  int32_t n;                 /* nodes */
  int32_t m;                 /* tets */
  const double* X0;          /* [3n] rest positions */
  const int32_t* T;          /* [4m] tets */
  const double* lame;        /* [2m] (lambda, mu) per tet */
  const double* rho;         /* [m] density per tet */
  const uint8_t* model;      /* [m] 0 = CoNH, 1 = StVK */
  const uint8_t* fixed;      /* [3n] hard-fixed DoFs, may be NULL */
  const double* force;       /* [3n] EnergyElement_Force f, may be NULL */
  double gravity[3];
  const double* soft_k;      /* [n] BC_FixDoF soft mode stiffness per node (0: none), may be NULL */
  const double* soft_target; /* [3n] its targets, NULL: X0 */
} orc_mesh;

/* Mirrors OptimSolverOptions (inc/Solvers/OptimSolver.h:47-70). */
typedef struct orc_options {
  int32_t qp_solver;         /* 0 = Steepest, 1 = Newton (QPSolverType) */
  double tol_max_error;      /* absolute ||g|| */
  double tol_min_step;
  int32_t min_step_max_count;
  double tol_min_impr;
  int32_t min_impr_max_count;
  int32_t num_max_iters;
  int32_t try_steepest;
  double max_step_size;
  int32_t ls_solver;         /* 1 = EigenCG, 2 = EigenLDLT (LSSolverType order) */
  int32_t ls_num_max_iters;
  double ls_tol_max_error;
  int32_t ls_num_reg_trials;
  int32_t lsearch_type;      /* LSearchType: 0 None, 1 Simple, 2 Armijo, 3 WolfeWeak, 4 WolfeStrong */
  double lsearch_alpha;
  int32_t lsearch_num_try;
  double lsearch_wolfe1;     /* Armijo / Wolfe c1 */
  double lsearch_wolfe2;     /* Wolfe c2 */
  int32_t cg_block_jacobi;   /* CG preconditioner: 0 = diagonal (Eigen), 1 = 3x3 block Jacobi */
  int32_t threads;           /* OpenMP threads for element loops; <= 0 keeps the default */
  int32_t cg_parallel;       /* 1: row-parallel CG products and blocked inner products (large systems) */
} orc_options;

typedef struct orc_report {
  int32_t result;            /* OSResult: 0 ONGOING 1 SUCCESS 2 MINSTEP 3 MINIMPR 4 FAILURE 5 MAXITER 6 NONDESC */
  int32_t iterations;
  int32_t bisections;        /* summed over iterations */
  int32_t reg_trials;        /* regularised linear solves */
  int64_t lin_iterations;    /* CG iterations summed */
  double obj;
  double opt;                /* final ||g|| */
  double opt0;               /* ||g|| at the first SolveStep (after BCs are loaded) */
  double seconds;
  /* per-phase seconds, named like the reference's CustomTimer ids */
  double t_cal_ene, t_cal_gra, t_cal_hes, t_ass_gra, t_ass_hes, t_opt_sol, t_opt_lis;
} orc_report;

/* One staged boundary condition (BCondition, inc/Physics/Boundary/BCondition.h:85-155):
 * BC_FixDoF on a node set, hard or soft, loaded over num_stages stages with its targets
 * animated by VectorAnimator_LerpT3D (inc/Utils/VectorAnimators.h:103-145):
 *   target(a) = a * shift + (I + a * move) * x_ini,   a = stage / num_stages,
 * and, when soft, the stiffness k_start + a (k_end - k_start) (BC_FixDoF.cpp:85-110). */
typedef struct orc_stage_group {
  int32_t num_stages;        /* m_numStage (>= 1) */
  int32_t soft;              /* 0: hard (the DoFs take the targets), 1: soft (targets and stiffness) */
  double k_start, k_end;     /* m_kAini, m_kAend */
  double move[9];            /* row-major 3x3 */
  double shift[3];
  int32_t num_nodes;
  const int32_t* nodes;
} orc_stage_group;

typedef struct orc_handle_s* orc_handle;

void orc_default_options(orc_options* o);

/* Builds rest-state data, the Hessian pattern and (lazily) the LDLT symbolic analysis. */
int orc_create(const orc_mesh* mesh, orc_handle* out);
void orc_destroy(orc_handle h);

/* Per-element values at positions x[3n]: E[m], g[12m], H[144m] (row-major 12x12). Any may be NULL. */
int orc_element_local(orc_handle h, const double* x, double* E, double* g, double* H);

/* Material laws at one deformation gradient (column-major Fv[9]). */
int orc_material(int model, double lame1, double lame2, const double* Fv,
                 double* psi, double* P, double* dPdF /* row-major 9x9, dP_i/dF_j */);

/* Global energy, gradient (fix != 0 applies FixVectorDoFs), Hessian values on the pattern. */
int orc_energy(orc_handle h, const double* x, double* E);
int orc_gradient(orc_handle h, const double* x, double* g, int fix);
int64_t orc_hessian_nnz(orc_handle h);
int orc_hessian_pattern(orc_handle h, int32_t* colptr /* 3n+1 */, int32_t* rowidx /* nnz */);
int orc_hessian(orc_handle h, const double* x, double* vals, int fix);
/* Lower-block slot of the 10 local node pairs (0,0),(1,0),(1,1),(2,0),...,(3,3) of each tet,
 * counting blocks in the column-major order of the pattern (one block per 3x3 tile). */
int orc_scatter_map(orc_handle h, int32_t* map /* 10m */);

/* OptimSolver::SolveFull on OptimProblem_BasicStatic, x in/out [3n]. */
int orc_solve_static(orc_handle h, const orc_options* opt, double* x, orc_report* rep);
/* One implicit-Euler step (OptimProblem_BasicDynamic + SolveFull); x, v in/out [3n]. */
int orc_solve_dynamic(orc_handle h, const orc_options* opt, double dt, double* x, double* v,
                      orc_report* rep);
/* One linear solve H dx = b with the configured linear solver (regularisation loop included). */
int orc_linear_solve(orc_handle h, const orc_options* opt, const double* x, const double* b,
                     double* dx, int32_t* lsresult, int64_t* iters);

/* Staged loading: the groups (their targets start from x_ini [3n]) and num_stages, the largest
 * m_numStage of all the model's boundary conditions (0 or 1: loaded from the first step).  The
 * stage counter goes back to 0; each static Newton iteration start (OnIterStart) and each
 * dynamic solve start (OnSolveStart) advances it, as StepBoundaryConditions does.  Soft groups
 * need soft records on their nodes (orc_mesh.soft_k > 0). */
int orc_set_staging(orc_handle h, int32_t count, const orc_stage_group* groups, int32_t num_stages,
                    const double* x_ini);
int orc_stage(orc_handle h);
/* Replaces the soft records (stiffness k[n], targets t[3n]) of nodes that have one. */
int orc_set_soft(orc_handle h, const double* k, const double* t);

/* Per-iteration log of the last solve: obj, opt, bisections, step norm per iteration. */
int orc_last_log(orc_handle h, double* obj, double* opt, int32_t* bis, double* step, int32_t cap);

#ifdef __cplusplus
}
#endif
#endif
