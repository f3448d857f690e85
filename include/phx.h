/*
 * phx.h -- C ABI of the GB300-native tet-FEM Newton path.
 *
 * The library replaces PhySim's CPU hot path for nonlinear tetrahedral FEM:
 * per-tet energy / gradient / Hessian, global assembly, and the Newton solver
 * with its linear solve and backtracking line search.  Everything runs on one
 * GPU (sm_103a); these entry points take plain host pointers and sizes.
 *
 * Conventions
 *  - Every call returns an int status: PHX_OK (0) or a negative PHX_E* code.
 *    No C++ exception crosses this boundary.  phx_last_error() gives a message.
 *  - Host buffers are caller owned; device state is library owned.
 *  - All calls are synchronous and thread-compatible: one context per host
 *    thread; a context and its instances must not be used from two threads at once.
 *  - DoF layout: DoF d of node v is 3*v + d (KinematicsTree offsets,
 *    source/PhySim/Kinematics/KinematicsTree.cpp:25-40).
 */
#ifndef PHX_H
#define PHX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PHX_OK 0
#define PHX_EINVAL (-1)   /* invalid argument or malformed mesh */
#define PHX_ENOMEM (-2)   /* device arena or host memory exhausted / admission refused */
#define PHX_ETIMEOUT (-3) /* a bounded device wait gave up */
#define PHX_ECUDA (-4)    /* CUDA runtime error */
#define PHX_EBUSY (-5)    /* object in use (e.g. instance already admitted) */
#define PHX_ENOTFOUND (-6)

/* OSResult (include/PhySim/BasicTypes.h:69-77), same numbering */
#define PHX_OS_ONGOING 0
#define PHX_OS_SUCCESS 1
#define PHX_OS_MINSTEP 2
#define PHX_OS_MINIMPR 3
#define PHX_OS_FAILURE 4
#define PHX_OS_MAXITER 5
#define PHX_OS_NONDESC 6

/* LSResult (include/PhySim/BasicTypes.h:61-67) */
#define PHX_LS_SUCCESS 0
#define PHX_LS_FAILURE 1

/* material models (MaterialModel_3Din3D_CoNH / _StVK, MaterialModels.h:166-299) */
#define PHX_MODEL_CONH 0
#define PHX_MODEL_STVK 1

/* arithmetic of the Hessian, element-Hessian kernel and PCG */
#define PHX_PREC_FP64 0         /* plain path: FP64 everywhere */
#define PHX_PREC_FP32_REFINE 1  /* served path: FP32 Hessian + PCG, FP64 residual refinement */

typedef struct phx_context_s* phx_context;
typedef struct phx_instance_s* phx_instance;

/* One FEM volume (Simulable_FEM + its boundary conditions).  Replaces the
 * model set-up path Simulable::Setup (source/PhySim/Physics/Simulables/Simulable.cpp:73-106)
 * with Tet4 shape functions and the Tet1 quadrature. */
typedef struct phx_mesh {
  int32_t num_nodes;
  int32_t num_tets;
  const double* X0;       /* [3*num_nodes] rest positions (Tag::Position_0) */
  const int32_t* tets;    /* [4*num_tets] node ids, positive rest volume required */
  const double* lame;     /* [2*num_tets] (LAME1 = lambda, LAME2 = mu) per tet */
  const double* rho;      /* [num_tets] density per tet (lumped mass) */
  const uint8_t* model;   /* [num_tets] PHX_MODEL_*; NULL = all CoNH */
  const uint8_t* fixed;   /* [3*num_nodes] hard-fixed DoFs (BC_FixDoF hard mode); NULL = none */
  const double* force;    /* [3*num_nodes] EnergyElement_Force f (energy x.f); NULL = none */
  double gravity[3];      /* BC_Gravity value */
  const double* soft_k;   /* [num_nodes] BC_FixDoF soft mode: stiffness k of each node's
                             EnergyElement_SoftConstraint, E = k/2 |x - t|^2 (0 = none); NULL = none */
  const double* soft_target; /* [3*num_nodes] their targets t; NULL = X0 */
} phx_mesh;

/* Mirrors OptimSolverOptions (include/PhySim/Solvers/OptimSolver.h:23-70): every field
 * with the same meaning and default, listed in the order of its constructor's
 * assignments (:47-70) rather than its declaration order, plus the GPU-path settings
 * at the end. */
typedef struct phx_options {
  int32_t qp_solver;          /* 0 Steepest, 1 Newton (QPSolverType) */
  double tol_max_error;       /* absolute ||g|| */
  double tol_min_step;
  int32_t min_step_max_count;
  double tol_min_impr;
  int32_t min_impr_max_count;
  int32_t num_max_iters;
  int32_t try_steepest;
  double max_step_size;
  int32_t ls_solver;          /* 1 EigenCG semantics (the only linear solver on the device) */
  int32_t ls_num_max_iters;   /* PCG iterations per linear solve */
  double ls_tol_max_error;    /* PCG relative residual ||r|| < tol ||b|| */
  int32_t ls_num_reg_trials;  /* >= 1; as in the reference, the linear solve's own 10 regularisation
                                 attempts (LinearSolverOptions::regIters) do not depend on it */
  int32_t lsearch_type;      /* LSearchType: 0 None, 1 Simple, 2 Armijo, 3 WolfeWeak, 4 WolfeStrong */
  double lsearch_alpha;
  int32_t lsearch_num_try;
  double lsearch_wolfe1;      /* Armijo / Wolfe sufficient-decrease constant c1 (1e-4) */
  double lsearch_wolfe2;      /* Wolfe curvature constant c2 (0.9) */
  /* GPU path */
  int32_t precision;          /* PHX_PREC_* */
  int32_t precond;            /* 0 diagonal (Eigen DiagonalPreconditioner), 1 3x3 block Jacobi */
  double inner_tol;           /* FP32 inner PCG relative tolerance per refinement sweep */
  int32_t max_refine_sweeps;  /* FP64 refinement sweeps per linear solve (FP32 path) */
  int32_t warm_guess;         /* 1: PCG starts from the previous accepted step (EigenCG solveWithGuess) */
  int32_t pcg_chunk;          /* PCG iterations per device round (launch granularity) */
  double tol_rel;             /* if > 0: stop at ||g|| <= max(tol_max_error, tol_rel * ||g0||), g0 after loading */
  int32_t pcg_cluster;        /* FP32 instances up to 13000 nodes run each PCG solve inside one 8-CTA cluster:
                                 1 rows in shared memory, z exchanged through distributed shared
                                 memory (default); 2 rows in L2, two-reduction CG.  Larger FP32
                                 instances then iterate in the whole-GPU PCG kernels (k_gpcg_a/b,
                                 the engine's PCG stages at the occupancy of a small kernel, the
                                 same bits).  0: every PCG iteration runs inside the engine */
  int32_t fp64_finish;        /* 1 (default): an FP32 solve that stalls (line search, progress or iteration
                                 limit) within 1000x of its tolerance, or after reducing ||g|| a
                                 hundredfold, is finished in FP64 from its last accepted iterate with
                                 ||g|| above 100x the tolerance, to the same tolerance; static solves
                                 only */
  int32_t lsearch_parallel;   /* once two trials of a line search were rejected, this many further trials
                                 (the step lengths the one-at-a-time search would try) are evaluated
                                 together and scanned in order with its rules: the same decisions in
                                 fewer rounds; 0 or 1: one at a time; at most 8 (default 8) */
  int32_t negative_curvature; /* FP32 path when the PCG meets p.Ap < 0 (an indefinite Hessian): 0 (default)
                                 truncates the solve there (Steihaug); 1 goes on with a negative step
                                 as Eigen's ConjugateGradient does, which the FP64 path always does,
                                 and regularises when the step is not a descent direction */
} phx_options;

typedef struct phx_report {
  int32_t result;           /* PHX_OS_* */
  int32_t iterations;       /* Newton iterations (SolveFull itCount) */
  int32_t bisections;       /* line-search bisections summed */
  int32_t reg_trials;       /* regularised linear solves */
  int64_t pcg_iterations;   /* PCG iterations summed */
  int32_t refine_sweeps;    /* FP64 residual refinement sweeps summed */
  int32_t status;           /* PHX_OK or a device-side error code */
  double obj;               /* final energy */
  double opt;               /* final ||g|| */
  double opt0;              /* ||g|| at the first step (after the loads are applied) */
  double seconds;           /* wall time of the call */
  int32_t hessian_evals;    /* element Hessian + assembly passes */
  int32_t fp64_iterations;  /* Newton iterations of the FP64 finish (0: none); included in iterations */
  int32_t pcg_slices;       /* cluster-PCG solves that left their cluster at a time slice's end and resumed
                               in a later launch (scheduling only: the results are the same) */
} phx_report;

/* ---- library ----------------------------------------------------------- */
int phx_version(void);
const char* phx_last_error(void);
void phx_default_options(phx_options* opts);

/* ---- context: one device, one stream, one device-memory arena ----------
 * arena_bytes = 0 picks a default (a quarter of free device memory). */
int phx_context_create(int32_t device, int64_t arena_bytes, phx_context* out);
int phx_context_destroy(phx_context ctx);
int phx_context_memory(phx_context ctx, int64_t* used_bytes, int64_t* capacity_bytes);
/* Test hook of the bounded device waits; no counterpart in the reference.  Every wait of
 * the engine (a grid barrier between two stages) gives up after a cycle limit, flags the
 * launch and the call returns PHX_ETIMEOUT with the context still usable.  With
 * barrier_tag in 1..22, the engine's grid barrier of that number waits, in every launch
 * that follows, for one arrival more than the CTAs taking part, so it runs out after
 * limit_cycles SM cycles (1000 .. 4e9).  Tag 1 is the barrier after each round's
 * bookkeeping, reached by every solve.  barrier_tag 0 switches the hook off and restores
 * the default limit (4e9 cycles, about 2 s). */
int phx_debug_unmet_barrier(phx_context ctx, int32_t barrier_tag, int64_t limit_cycles);

/* ---- launch settings and the batch tuner (no counterpart in the reference) -----------
 * How a context schedules its batch solves.  None of them changes a result: every instance
 * runs the same state machine whatever the schedule (a batch solve gives the bits of solving
 * each instance alone).
 *   graph        1: the solve loop runs as CUDA-graph launches (a device while-loop of
 *                k_prep, the engine, the cluster PCG kernels and the loop test; the host
 *                looks in every 256 passes); 0: one host step per engine launch.
 *                Profiling (phx_context_profile) always takes the host loop.
 *   wait_rounds  engine rounds an instance may wait for the cluster PCG kernel ...
 *   wait_share   ... or until 1/wait_share of the active instances wait for it
 *   rounds       engine rounds per engine launch
 *   pcg_grid     1: FP32 instances above the cluster size (13,000 nodes) iterate their PCG in the
 *                whole-GPU kernels k_gpcg_a/b, which run until each such instance has finished
 *                its linear solve; 0 (default): inside the engine's PCG stages, interleaved with
 *                the other instances' work (lower latency for small requests beside large ones) */
typedef struct phx_launch_settings {
  int32_t graph;
  int32_t wait_rounds;
  int32_t wait_share;
  int32_t rounds;
  int32_t pcg_grid;
  int32_t slice_share;  /* a cluster-PCG solve ends its time slice (and resumes in the next cluster
                           launch) once clusters/slice_share of the launch's clusters found no solve
                           left and another solve of the launch ended; 0: no time slices */
  int32_t slice_min;    /* PCG iterations a solve runs in a launch before its slice may end */
} phx_launch_settings;
/* Reads the context's default settings into *get (if not NULL), then sets them from *set (if
 * not NULL; values checked: graph 0/1, wait_rounds 1..64, wait_share 1..64, rounds 1..1024,
 * pcg_grid 0/1, slice_share 0..64, slice_min 1..1000000).  The serving calls use the context's defaults. */
int phx_context_launch_settings(phx_context ctx, phx_launch_settings* get, const phx_launch_settings* set);
/* Tunes the settings for a batch: times phx_batch_solve-style solves of the instances from
 * their current positions under the default settings and candidates around them (one
 * setting changed at a time, kept when at least 1 % faster), then puts the instances back as
 * they were (positions and warm-start steps).  The best settings are cached under the
 * batch's mix key (precision and the count of instances per power-of-two node-count bucket):
 * later batch solves of the context with that key use them.  Instances with staged boundary
 * conditions are refused (a trial would advance their stages).  chosen, default_seconds,
 * best_seconds and trials may be NULL. */
int phx_tune_batch(phx_context ctx, int32_t count, phx_instance* insts, const phx_options* opts,
                   phx_launch_settings* chosen, double* default_seconds, double* best_seconds, int32_t* trials);

/* ---- instances: Simulable_FEM set-up (replaces Simulable::Setup + the first
 * triplet assembly that fixes the Hessian pattern, source/PhySim/BasicTypes.cpp:118-145).
 * Validates the mesh (PHX_EINVAL on bad ids or non-positive rest volume),
 * builds the 3x3 block pattern and the scatter map, uploads everything. */
int phx_instance_create(phx_context ctx, const phx_mesh* mesh, phx_instance* out);
/* count instances at once (serving admission, batch set-up): the host parts (validation,
 * pattern, scatter map) are built on several host threads, then each is set up on the
 * device; out[i] for meshes[i].  On an error none is created. */
int phx_instances_create(phx_context ctx, int32_t count, const phx_mesh* meshes, phx_instance* out);
int phx_instance_destroy(phx_instance inst);
int phx_instance_sizes(phx_instance inst, int64_t* num_dofs, int64_t* hessian_nnz,
                       int64_t* lower_blocks, int64_t* full_blocks);
/* Positions back to rest (Tag::Position_0), velocities and the warm-start step to zero, on the device. */
int phx_instance_reset(phx_instance inst);
/* Model state (ISimulable::Get/SetDOFVector, Tag::Position_X / Tag::Velocity, Simulable.h:55-94) */
int phx_instance_set_positions(phx_instance inst, const double* x);
int phx_instance_get_positions(phx_instance inst, double* x);
int phx_instance_set_velocities(phx_instance inst, const double* v);
int phx_instance_get_velocities(phx_instance inst, double* v);
/* Replace the nodal loads (EnergyElement_Force f, BC_Gravity g) of a live instance; warm re-solves. */
int phx_instance_update_load(phx_instance inst, const double* force, const double* gravity);

/* ---- staged boundary conditions ----------------------------------------
 * BCondition stages (include/PhySim/Physics/Boundary/BCondition.h:85-155, BCondition.cpp:42-67):
 * every condition advances one stage at each Newton iteration start of a static solve
 * (OptimProblem_BasicStatic::OnIterStart) and at each dynamic step's start
 * (OptimProblem_BasicDynamic::OnSolveStart), up to its own num_stages; SolveFull applies its
 * stop rules only once every condition is at its last stage (IsFullyConstrained,
 * OptimSolver.cpp:213).  A group is one BC_FixDoF on a node set (BC_FixDoF.cpp:51-121):
 * hard (its nodes must be fixed in all three DoFs; the static problem moves them to the
 * targets) or soft (its nodes need a soft record; targets and stiffness change).  Its
 * targets follow VectorAnimator_LerpT3D (include/PhySim/Utils/VectorAnimators.h:103-145):
 *   target(a) = a * shift + (I + a * move) * v,   a = min(stage, num_stages) / num_stages,
 * v the node's position when phx_instance_set_staging is called; a soft stiffness is
 * k_start + a (k_end - k_start).  (The reference's scene loader builds `move` as R*S from
 * the animation's rotation and scale, so a full stage applies I + R*S, not R*S.) */
typedef struct phx_stage_group {
  int32_t num_stages;  /* BCondition::m_numStage (>= 1) */
  int32_t soft;        /* 0 hard, 1 soft */
  double k_start, k_end;
  double move[9];      /* row-major 3x3 */
  double shift[3];
  int32_t num_nodes;
  const int32_t* nodes;
} phx_stage_group;
/* Sets the groups (a node in one group at most) and num_stages, the largest m_numStage over
 * all the model's conditions (a condition without targets, e.g. BC_Gravity with numStep, only
 * delays full constraint); the stage goes back to 0.  count 0 and num_stages 0: no staging.
 * phx_instance_reset also takes the stage back to 0 (Simulable::ResetBoundaryConditions). */
int phx_instance_set_staging(phx_instance inst, int32_t count, const phx_stage_group* groups, int32_t num_stages);
int phx_instance_stage(phx_instance inst, int32_t* stage, int32_t* num_stages);

/* ---- scene files -----------------------------------------------------------
 * The reference's XML vocabulary (source/PhySim/Utils/Serializer_XML.cpp): the element read by
 * LoadSimulable_VolumeFEM (:1199-1325) as <simulable type="VolumeFEM">, LoadOptimProblem's
 * (:1327-1354) as <problem>, LoadOptimSolver's (:1356-1505) as <solver> and LoadBoundary's
 * <bc> list (:1507-1647) inside <boundary>, all under one root element (the reference has
 * no top-level reader; this is the layout that holds its loaders' elements).  meshInit /
 * meshRest are FILEVOLUME TetGen meshes (<base>.node + <base>.ele; the reference declares
 * Serializer_Mesh::ReadVolume_TET without a body), relative to the scene file; TET4 with
 * TET_LIN / TET_1, CONH / STVK, CONSTANT or VARIABLE distributions; Gravity and FixPosition
 * (hard or soft, numStep, Transform3D animation, AllNodes / BoundaryNodes / IndexNodes /
 * BoxNodes selections).  Anything else is refused with PHX_EINVAL and a message. */
typedef struct phx_scene_s* phx_scene;
int phx_scene_load(const char* path, phx_scene* out);
int phx_scene_destroy(phx_scene sc);
/* counts; reoriented: tetrahedra of negative volume in the file whose corners 1, 2 were swapped */
int phx_scene_info(phx_scene sc, int32_t* num_nodes, int32_t* num_tets, int32_t* dynamic, double* dt,
                   int32_t* num_groups, int32_t* num_stages, int32_t* reoriented);
/* The model as a phx_mesh (pointers into the scene, valid while it lives) and, if x_init is
 * not NULL, its start positions [3n] (meshInit; the rest shape is meshRest, else meshInit). */
int phx_scene_mesh(phx_scene sc, phx_mesh* mesh, double* x_init);
/* phx_default_options with the scene's <solver> attributes applied */
int phx_scene_options(phx_scene sc, phx_options* opts);
/* Up to cap staged groups (animated FixPosition conditions); returns their count. */
int phx_scene_staging(phx_scene sc, phx_stage_group* groups, int32_t cap);
/* Creates the scene's instance: the mesh, its start positions and its staging. */
int phx_scene_instance(phx_context ctx, phx_scene sc, phx_instance* out);

/* ---- field output: SVL scalar grids ---------------------------------------
 * Serializer_Field::ReadGrid_SVL / WriteGrid_SVL (source/PhySim/Utils/Serializer_Field.cpp:
 * 50-112, 114-140) on ScalarField_Grid (include/PhySim/Geometry/Volumes/ScalarField_Grid.h):
 * a header of shape (3 int32), origin (3 double), delta (3 double) and the value type (int32,
 * PHX_SVL_*), then shape[0]*shape[1]*shape[2] values in native byte order, x fastest (the
 * column-major order of the grid's Eigen tensor: value (i, j, k) at i + s0*(j + s1*k)).
 * Value (i, j, k) belongs to the cell centre origin + (i + 1/2, j + 1/2, k + 1/2) * delta
 * (ScalarField_Grid::Sample's coordinates). */
#define PHX_SVL_INT8 0    /* "char": read and written as signed 8-bit */
#define PHX_SVL_INT16 1
#define PHX_SVL_INT32 2
#define PHX_SVL_FLOAT 3
#define PHX_SVL_DOUBLE 4
typedef struct phx_grid {
  int32_t shape[3];  /* >= 1 each (ScalarField_Grid::Setup) */
  double origin[3];
  double delta[3];
} phx_grid;
/* Writes a grid file; values holds prod(shape) values of the given format. */
int phx_svl_write(const char* path, const phx_grid* grid, int32_t format, const void* values);
/* Reads a grid file's header (grid may be NULL) and value type (format may be NULL). */
int phx_svl_read_header(const char* path, phx_grid* grid, int32_t* format);
/* Reads a grid file's values as `as_format` into values (room for `capacity` values).  A file
 * of another value type is converted value by value, as the reference's
 * readBinaryArrayWithCast does; a value the target type cannot hold (out of range, or NaN to
 * an integer type) is refused with PHX_EINVAL instead of converted.  A short file, a shape
 * below 1 or an unknown value type is PHX_EINVAL. */
int phx_svl_read(const char* path, int32_t as_format, void* values, int64_t capacity);

/* Fields of a solve sampled on a grid (phx_instance_sample_grid). */
#define PHX_FIELD_DISPLACEMENT_X 0     /* u = x - X0, interpolated linearly in the owning tet */
#define PHX_FIELD_DISPLACEMENT_Y 1
#define PHX_FIELD_DISPLACEMENT_Z 2
#define PHX_FIELD_DISPLACEMENT_NORM 3  /* |u| of the interpolated u */
#define PHX_FIELD_VOLUME_RATIO 4       /* J = det F of the owning tet */
#define PHX_FIELD_ENERGY_DENSITY 5     /* the owning tet's elastic energy / rest volume */
/* Samples a field of the instance on the cell centres of a grid laid over the REST shape,
 * on the device.  A centre belongs to the tet of lowest index that contains it: the four
 * sub-volumes it cuts the tet into are each >= -1e-12 of the tet's (six times) volume; a
 * centre that no tet contains gets `fill` and owner -1 (ScalarField_Grid::Sample returns -1
 * outside its box).  x[3n] are the positions to sample (NULL: the instance's current ones;
 * like phx_energy_gradient, a given x becomes the instance's positions).  values
 * [prod(shape)] as in an SVL file; owner (may be NULL) the owning tet of each value.  At
 * most 2^31 - 1 values. */
int phx_instance_sample_grid(phx_instance inst, const double* x, int32_t field, const phx_grid* grid,
                             double fill, double* values, int32_t* owner);

/* ---- model evaluation (ISimulable::GetEnergy / GetGradient / GetHessian) --- */
/* Energy and gradient at x[3n] (x == NULL: current positions).  fix != 0 applies
 * FixVectorDoFs (Simulable.cpp:735-744). */
int phx_energy_gradient(phx_instance inst, const double* x, double* energy, double* gradient, int32_t fix);
/* Hessian values on the Eigen lower pattern (diagonal 3x3 node blocks in full),
 * column-major like MatrixSd; fix != 0 applies FixMatrixDoFs (Simulable.cpp:746-760). */
int phx_hessian(phx_instance inst, const double* x, int32_t precision, double* values, int32_t fix);
int phx_hessian_pattern(phx_instance inst, int32_t* colptr /* 3n+1 */, int32_t* rowidx /* nnz */);
/* Lower-block slot of the 10 local node pairs (0,0),(1,0),(1,1),(2,0),(2,1),(2,2),(3,0),...,(3,3)
 * of every tet, blocks counted column-major over the pattern (DerivativeAssembler.cpp:205-300). */
int phx_scatter_map(phx_instance inst, int32_t* map /* 10*num_tets */);
/* Per-element values (IEnergyElement::GetLocal*, EnergyElement_FEM.cpp:125-222):
 * E[m], g[12m], H[144m] row-major 12x12; any output may be NULL.  Energy and gradient are
 * FP64 on both paths; precision selects the Hessian kernel (PHX_PREC_FP32_REFINE: FP32). */
int phx_element_local(phx_instance inst, const double* x, int32_t precision, double* E, double* g, double* H);

/* ---- solver (IOptimSolver::SolveFull / SolveStep, OptimSolver.cpp:148-311,
 * on OptimProblem_BasicStatic / OptimProblem_BasicDynamic) -------------- */
/* Static equilibrium from x_inout (NULL: from the instance's current positions). */
int phx_solve_static(phx_instance inst, const phx_options* opts, double* x_inout, phx_report* rep);
/* One SolveStep (a single Newton iteration with its line search). */
int phx_solve_step(phx_instance inst, const phx_options* opts, double* x_inout, phx_report* rep);
/* One implicit-Euler step: minimises the incremental potential (OptimProblem_BasicDynamic). */
int phx_dynamic_step(phx_instance inst, const phx_options* opts, double dt, double* x_inout,
                     double* v_inout, phx_report* rep);
/* Per-iteration trace of the instance's last solve (OptimSolver::LineSearch logging,
 * OptimSolver.cpp:385-395): objective, ||g||, bisections and step length per Newton
 * iteration, up to cap entries (at most 256 are kept).  Returns the iteration count (>= 0). */
int phx_solve_log(phx_instance inst, double* obj, double* opt, int32_t* bisections, double* step, int32_t cap);
/* Many independent static solves in one device batch (persistent kernels over a
 * packed instance index).  x_inout[i] may be NULL; reps has count entries. */
int phx_batch_solve(phx_context ctx, int32_t count, phx_instance* insts, const phx_options* opts,
                    double* const* x_inout, phx_report* reps);
/* Batched implicit-Euler steps (one per instance). */
int phx_batch_dynamic_step(phx_context ctx, int32_t count, phx_instance* insts, const phx_options* opts,
                           double dt, phx_report* reps);

/* ---- serving: continuous batching over the same device engine ----------
 * No counterpart in the reference (its solver runs one object per call).  Requests are
 * admitted at Newton-round boundaries while the device is busy with others, bounded by
 * free slots and a device-memory budget; admitted requests are solved together in the
 * engine's rounds, each instance with its own reduction order, so a result is the same
 * alone and in the mix.  Instances the server creates for cold requests stay on the
 * device while idle (mesh, pattern and last solution kept for warm re-solves) and count
 * against the budget; when a request does not fit, idle ones are evicted, least recently
 * used first (positions and velocities kept on the host; the instance is rebuilt on its
 * next request).  A request larger than the whole budget is refused with PHX_ENOMEM: at
 * submission for a caller's instance, through its report (status PHX_ENOMEM, result
 * FAILURE) for a cold request, whose size is known once its pattern is built. */
typedef struct phx_server_s* phx_server;
int phx_server_create(phx_context ctx, int32_t max_slots, int64_t budget_bytes, const phx_options* opts,
                      phx_server* out);
/* Instances created by phx_server_submit_mesh stay valid (the caller destroys them); one
 * that is off the device then keeps only its host state. */
int phx_server_destroy(phx_server srv);
/* Queue a static solve of inst from its current positions (a warm re-solve when it holds a
 * previous solution, e.g. after phx_instance_update_load); tag is returned by poll. */
int phx_server_submit(phx_server srv, phx_instance inst, int64_t tag);
/* Queue one implicit-Euler step of inst (OptimProblem_BasicDynamic), time step dt. */
int phx_server_submit_step(phx_server srv, phx_instance inst, double dt, int64_t tag);
/* A cold request: the server copies the mesh, builds its pattern and scatter map on host
 * worker threads, and creates the instance on the device when the request is admitted;
 * then a static solve from rest.  *out is the new instance (for warm re-solves and for
 * reading the result; the caller destroys it).  Until admitted, and after an eviction, calls
 * that need its device part return PHX_EBUSY; its positions and velocities stay readable. */
int phx_server_submit_mesh(phx_server srv, const phx_mesh* mesh, int64_t tag, phx_instance* out);
/* Device bytes the server holds now and at most so far, instances it created that are on
 * the device, and evictions so far; any pointer may be NULL. */
int phx_server_stats(phx_server srv, int64_t* in_use, int64_t* peak, int64_t* resident, int64_t* evictions);
/* Advance the device by one round; admits queued requests first. */
int phx_server_progress(phx_server srv, int32_t* active, int32_t* queued);
/* Pop up to cap finished requests: tags, reports. Returns the number popped (>= 0) or an error. */
int phx_server_poll(phx_server srv, int64_t* tags, phx_report* reps, int32_t cap);

/* ---- measurement hooks ------------------------------------------------- */
/* Kernel timing with CUDA events on the library's stream; kind names:
 * "elem_eg", "gather", "elem_hess", "assemble", "jacobi", "spmv", "pcg_update", ... */
int phx_profile_enable(phx_context ctx, int32_t on);
int phx_profile_read(phx_context ctx, const char* kind, int64_t* launches, double* total_ms);
int phx_profile_reset(phx_context ctx);
/* Algorithmic bytes the launches of one kernel kind moved since the last reset (profiling on):
 * matrix blocks, indices and vectors each launch must read or write once, per active instance. */
int phx_profile_bytes(phx_context ctx, const char* kind, double* bytes);
/* CUDA events on the library's stream: record slot (0..15); elapsed ms between two recorded slots. */
int phx_timer_mark(phx_context ctx, int32_t slot);
int phx_timer_elapsed(phx_context ctx, int32_t slot_a, int32_t slot_b, double* ms);
/* Launch count of the library's own kernels since creation (or the last reset). */
int64_t phx_kernel_launches(phx_context ctx);

/* ---- element Hessian + assembly without allocation -----------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory
 * (an engine that owns all GPU memory in its own pool, a runtime that forbids
 * cudaMalloc while frames run): every argument is a caller-owned device pointer and the
 * only scratch is a fixed static device array of PHX_NOALLOC_MAX_TETS * 90 doubles
 * (about 23.6 MB, held by every GPU that loads the library until exit).  Computes the
 * model Hessian (no fixed DoFs applied) as the lower 3x3 node blocks of the Eigen
 * pattern, in the same element order as phx_hessian:
 *   tets [4m] int32, rest [12m] (column-major Dm^-1, rest volume, lambda, mu per tet),
 *   model [m] (NULL = CoNH), x, X0 [3n] positions and rest positions,
 *   seg_ptr [nlo+1], seg_c [10m]: for each lower block, its (tet*10 + local pair)
 *   contributions in element order (the inverted scatter map of phx_scatter_map),
 *   blocks [9*nlo] out, row-major per block: entry (a, b) = H(3R + a, 3C + b).
 * Kernels are queued on `stream` (a cudaStream_t; NULL = legacy default stream) and the
 * call returns without waiting.  The scratch's device address is looked up on the first
 * call on each device (with that device current), so that call must precede any stream
 * capture; the address is then kept for the life of the process, so the entry point
 * assumes the device's primary context throughout (no use after cudaDeviceReset).
 * Calls that overlap on the GPU race on the shared scratch.  More than
 * PHX_NOALLOC_MAX_TETS tets: PHX_EINVAL.  The indices are trusted, not checked on the
 * device: every tets entry lies in [0, num_nodes), seg_ptr rises from 0 to 10*num_tets
 * and every seg_c entry lies in [0, 10*num_tets). */
#define PHX_NOALLOC_MAX_TETS 32768
int phx_hessian_blocks_noalloc(int32_t num_nodes, int32_t num_tets, int32_t num_lower_blocks, const int32_t* tets,
                               const double* rest, const uint8_t* model, const double* x, const double* X0,
                               const int32_t* seg_ptr, const int32_t* seg_c, double* blocks, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PHX_H */
