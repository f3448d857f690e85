"""Device-resident Newton solves against the oracle.

Parity bar: converged displacements within 1e-6 relative of the oracle's
LDLT Newton solve, FP64 energies at the same positions within 1e-9 relative.
Iterate-level parity is checked against the oracle's CG mode, whose linear
solver has the same semantics as the device PCG.
"""
import numpy as np
import pytest

import oracle
import physim_gb300 as px
from physim_gb300 import mesh as M
from conftest import rel

pytestmark = pytest.mark.gpu


def oracle_solution(m, rel_tol):
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    x, rep = orc.solve_static(x0, tol_max_error=rel_tol * g0, tol_min_impr=0.0, tol_min_step=0.0)
    return orc, x0, g0, x, rep


def disp_err(x, xr, x0):
    return rel(x - x0, xr - x0)


@pytest.fixture(scope="module")
def c1_oracle():
    return oracle_solution(M.cantilever(), 1e-10)


def test_cantilever_fp64_plain(gpu_ctx, c1_oracle):
    orc, x0, g0, xr, rep = c1_oracle
    inst = px.Instance(gpu_ctx, orc.mesh)
    o = px.options(tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    x, r = inst.solve_static(o, x0)
    assert r["result_name"] == "SUCCESS", r
    assert r["opt"] <= 1e-8 * g0 and abs(r["opt0"] - g0) <= 1e-12 * g0
    assert disp_err(x, xr, x0) < 1e-6
    # energy at the same positions
    Eg, _ = inst.energy_gradient(x)
    assert abs(Eg - orc.energy(x)) <= 1e-9 * abs(orc.energy(x))
    assert abs(r["obj"] - orc.energy(x)) <= 1e-9 * abs(orc.energy(x))


def test_cantilever_fp32_refine(gpu_ctx, c1_oracle):
    """The served FP32+refinement path at its specified tolerance (1e-6 of the starting
    gradient): the energy comparison of the line search stops resolving steps near 7e-8 of
    g0 on this mesh, which the path's linear final convergence can land in, so tighter
    tolerances are not a property of the path."""
    orc, x0, g0, xr, rep = c1_oracle
    inst = px.Instance(gpu_ctx, orc.mesh)
    o = px.options(precision=px.PREC_FP32_REFINE, tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    x, r = inst.solve_static(o, x0)
    assert r["result_name"] == "SUCCESS", r
    assert r["refine_sweeps"] > 0 and r["fp64_iterations"] == 0
    assert r["opt"] <= 1e-6 * g0
    assert disp_err(x, xr, x0) < 1e-6


def test_iterates_match_oracle_cg_mode(gpu_ctx):
    m = M.cantilever(3, 3, 10)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-9 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    log = orc.last_log()
    inst = px.Instance(gpu_ctx, m)
    x, r = inst.solve_static(px.options(**kw), x0)
    assert r["iterations"] == ro["iterations"] and r["bisections"] == ro["bisections"]
    assert abs(r["pcg_iterations"] - ro["lin_iterations"]) <= 2 * ro["iterations"]
    assert disp_err(x, xo, x0) < 1e-9
    # one SolveStep from rest lands on the oracle's first iterate
    inst2 = px.Instance(gpu_ctx, m)
    x1, r1 = inst2.solve_step(px.options(**kw), x0)
    assert abs(r1["obj"] - log["obj"][0]) <= 1e-10 * abs(log["obj"][0])


def test_stvk_traction_box(gpu_ctx):
    m = M.make_box(3, 3, 6, (0.03, 0.03, 0.06), 2e5, 0.35, 1000.0, M.MODEL_STVK, (0.0, 0.0, 0.0),
                   clamp_face=4, load_face=5, traction=(400.0, -300.0, 800.0))
    orc, x0, g0, xr, rep = oracle_solution(m, 1e-9)
    inst = px.Instance(gpu_ctx, m)
    for prec in (px.PREC_FP64, px.PREC_FP32_REFINE):
        x, r = inst.solve_static(px.options(precision=prec, tol_max_error=1e-7 * g0, tol_min_impr=0.0,
                                            tol_min_step=0.0), x0)
        assert r["result_name"] == "SUCCESS"
        assert disp_err(x, xr, x0) < 1e-6


def test_reference_default_options(gpu_ctx):
    # reference defaults end in SUCCESS / MINIMPR like the oracle does
    m = M.cantilever(2, 2, 6)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1)
    inst = px.Instance(gpu_ctx, m)
    x, r = inst.solve_static(px.options(), x0)
    assert r["result"] == ro["result"] and r["iterations"] == ro["iterations"]
    assert disp_err(x, xo, x0) < 1e-6


def test_implicit_euler_steps(gpu_ctx):
    m = M.make_box(3, 3, 3, (0.03, 0.03, 0.03), 1e5, 0.45, 1000.0, 0, (0.0, -9.81, 0.0), clamp_face=2)
    orc = oracle.Oracle(m)
    x = orc.rest()
    v = np.zeros(orc.N)
    v[1::3] = 0.5 * np.sin(np.pi * m.X0[:, 0] / 0.03)
    v[m.fixed.astype(bool)] = 0
    inst = px.Instance(gpu_ctx, m)
    xg, vg = x.copy(), v.copy()
    # the strict energy decrease of the line search resolves ||g|| down to about
    # sqrt(eps |E| m/dt^2) ~ 3e-8 here; tighter absolute tolerances are noise for any solver
    kw = dict(tol_max_error=2e-7, tol_min_impr=0.0, tol_min_step=0.0)
    for step in range(5):
        x, v, ro = orc.solve_dynamic(x, v, 1e-3, **kw)
        for prec in (px.PREC_FP64,):
            xg, vg, r = inst.dynamic_step(px.options(precision=prec, **kw), 1e-3, xg, vg)
        assert r["result_name"] == "SUCCESS"
        assert rel(xg - orc.rest(), x - orc.rest()) < 1e-6
        assert rel(vg, v) < 1e-5


def test_batch_equals_alone_bitwise(gpu_ctx):
    meshes = [M.batch_instance(3, i) for i in range(6)]
    o = px.options(precision=px.PREC_FP32_REFINE, tol_max_error=1e-7, tol_min_impr=0.0, tol_min_step=0.0)
    alone = []
    for m in meshes:
        inst = px.Instance(gpu_ctx, m)
        x, r = inst.solve_static(o, m.X0.ravel())
        alone.append((x, r))
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    reps, xs = gpu_ctx.batch_solve(insts, o, [m.X0.ravel().copy() for m in meshes])
    for (xa, ra), xb, rb in zip(alone, xs, reps):
        assert np.array_equal(xa, xb)
        assert ra["iterations"] == rb["iterations"] and ra["pcg_iterations"] == rb["pcg_iterations"]
        assert ra["obj"] == rb["obj"]


def test_engine_pcg_batch_equals_alone_bitwise(gpu_ctx):
    """Instances whose PCG runs in the engine (the FP64 path) get the same bits alone and in a
    batch of 40: their PCG tile width, and with it the order of the per-tile partial sums, is
    the instance's own, whatever the number of active instances."""
    meshes = [M.batch_instance(3, i) for i in range(200, 240)]
    o = px.options(precision=px.PREC_FP64, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    reps, xs = gpu_ctx.batch_solve(insts, o, [m.X0.ravel().copy() for m in meshes])
    for k in (0, 17, 39):
        inst = px.Instance(gpu_ctx, meshes[k])
        xa, ra = inst.solve_static(o, meshes[k].X0.ravel())
        assert np.array_equal(xa, xs[k])
        assert ra["iterations"] == reps[k]["iterations"] and ra["pcg_iterations"] == reps[k]["pcg_iterations"]
        assert ra["obj"] == reps[k]["obj"]


def test_cluster_time_slices_keep_the_bits(gpu_ctx):
    """Long cluster-PCG solves that leave their cluster at the end of a time slice (another
    solve of the launch has ended and half the clusters found nothing left) and resume in a
    later launch give the bits of the same instances solved alone, where no slice ends."""
    # six with PCG solves of 300-400 iterations, five small ones, nine others: 20 solves wait
    # for the 15 clusters of the first launch
    idx = [52, 399, 96, 217, 276, 86, 16, 38, 63, 71, 83] + list(range(100, 109))
    meshes = [M.batch_instance(3, i) for i in idx]
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    saved = gpu_ctx.launch_settings()
    try:
        gpu_ctx.launch_settings(wait_share=1)  # every waiting solve in one cluster launch
        alone = []
        for m in meshes:
            inst = px.Instance(gpu_ctx, m)
            alone.append(inst.solve_static(o, m.X0.ravel()))
        insts = [px.Instance(gpu_ctx, m) for m in meshes]
        reps, xs = gpu_ctx.batch_solve(insts, o, [m.X0.ravel().copy() for m in meshes])
    finally:
        gpu_ctx.launch_settings(**saved)
    assert all(ra["pcg_slices"] == 0 for _, ra in alone)
    assert sum(r["pcg_slices"] for r in reps) > 0
    for (xa, ra), xb, rb in zip(alone, xs, reps):
        assert np.array_equal(xa, xb)
        assert ra["iterations"] == rb["iterations"] and ra["pcg_iterations"] == rb["pcg_iterations"]
        assert ra["obj"] == rb["obj"] and ra["result_name"] == rb["result_name"]


def test_batch_against_oracle(gpu_ctx):
    meshes = [M.batch_instance(3, i) for i in range(10, 14)]
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    tols = []
    for m in meshes:
        orc = oracle.Oracle(m)
        tols.append(np.linalg.norm(orc.gradient(orc.rest())))
    o = px.options(precision=px.PREC_FP32_REFINE, tol_max_error=1e-6 * min(tols), tol_min_impr=0.0,
                   tol_min_step=0.0)
    reps, xs = gpu_ctx.batch_solve(insts, o, [m.X0.ravel().copy() for m in meshes])
    for m, x, r in zip(meshes, xs, reps):
        orc, x0, g0, xr, _ = oracle_solution(m, 1e-10)
        assert r["result_name"] == "SUCCESS"
        assert disp_err(x, xr, x0) < 1e-6


def test_server_results_same_alone_and_in_the_mix(gpu_ctx):
    meshes = [M.serving_request(11, i) for i in range(8)]
    meshes = [m for m in meshes if m.m < 40000][:5]
    o = px.options(precision=px.PREC_FP32_REFINE, tol_max_error=1e-7, tol_min_impr=0.0, tol_min_step=0.0)
    alone = {}
    for i, m in enumerate(meshes):
        inst = px.Instance(gpu_ctx, m)
        x, r = inst.solve_static(o, m.X0.ravel())
        alone[i] = x
    srv = px.Server(gpu_ctx, max_slots=3, budget_bytes=8 << 30, opts=o)
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    done = {}
    submitted = 0
    rounds = 0
    while len(done) < len(insts):
        if submitted < len(insts) and rounds % 3 == 0:  # staggered arrivals while others run
            srv.submit(insts[submitted], submitted)
            submitted += 1
        srv.progress()
        for tag, rep in srv.poll():
            assert rep["result_name"] == "SUCCESS"
            done[tag] = insts[tag].positions()
        rounds += 1
        assert rounds < 100000
    for i in alone:
        assert np.array_equal(alone[i], done[i])
    srv.close()


def test_warm_resolve_after_load_update(gpu_ctx):
    m = M.serving_request(11, 2)
    inst = px.Instance(gpu_ctx, m)
    # the served FP32 path is specified at 1e-6 relative residual: its Newton steps use the
    # FP32-stored Hessian, so convergence turns linear near kappa * 1e-7 on slender bars
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    x1, r1 = inst.solve_static(o, m.X0.ravel())
    m2 = M.perturb_load(m, 11, 2)
    inst.update_load(m2.force, m2.gravity)
    x2, r2 = inst.solve_static(o)  # from the previous equilibrium
    orc, x0, g0, xr, _ = oracle_solution(m2, 1e-10)
    assert r2["result_name"] == "SUCCESS"
    assert r2["iterations"] <= r1["iterations"]
    assert disp_err(x2, xr, x0) < 1e-6


def test_fp32_stall_finishes_in_fp64(gpu_ctx, c1_oracle):
    """An FP32 solve that stops short (here: an iteration cap) after reducing the gradient a
    hundredfold is finished in FP64 from its last iterate with ||g|| above 100x the tolerance,
    to the same tolerance; without the finish it reports where FP32 stopped.  The tolerance
    (1e-6 of the starting gradient) sits well above the band where the FP64 energy
    comparison of the line search stops resolving a step on this mesh (about 1e-7)."""
    orc, x0, g0, xr, rep = c1_oracle
    inst = px.Instance(gpu_ctx, orc.mesh)
    base = dict(precision=px.PREC_FP32_REFINE, tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0,
                num_max_iters=9)
    x, r = inst.solve_static(px.options(fp64_finish=0, **base), x0)
    assert r["result_name"] == "MAXITER" and r["fp64_iterations"] == 0
    assert r["opt"] <= 1e-2 * r["opt0"]
    x, r = inst.solve_static(px.options(fp64_finish=1, **base), x0)
    assert r["result_name"] == "SUCCESS", r
    assert r["fp64_iterations"] > 0 and r["iterations"] > r["fp64_iterations"]
    assert r["opt"] <= 1e-6 * g0
    assert disp_err(x, xr, x0) < 1e-5


@pytest.mark.parametrize("lst", [1, 2])
def test_parallel_line_search_same_result_on_gpu(gpu_ctx, lst):
    """A StVK batch instance whose solve takes hundreds of line-search bisections: trials
    evaluated together (Simple and Armijo searches) give the same iterations, bisections,
    result and positions."""
    m = M.batch_instance(3, 0)
    inst = px.Instance(gpu_ctx, m)
    out = []
    for k in (0, 8):
        o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                       tol_min_step=0.0, lsearch_parallel=k, fp64_finish=0, lsearch_type=lst)
        inst.reset()
        x, r = inst.solve_static(o)
        out.append((x, r))
    (xa, ra), (xb, rb) = out
    assert ra["bisections"] > 50
    for key in ("result", "iterations", "bisections", "pcg_iterations"):
        assert ra[key] == rb[key], key
    assert np.array_equal(xa, xb)


def _load_free(m):
    out = m.copy()
    out.force = np.zeros_like(m.force)
    out.gravity = np.zeros(3)
    return out


@pytest.mark.parametrize("prec", [px.PREC_FP64, px.PREC_FP32_REFINE])
def test_no_load_stays_at_rest(gpu_ctx, prec):
    """Zero right-hand side: the solve returns the rest shape at once (SolveFull's first
    check), for a free-standing loaded mesh with its loads removed."""
    m = _load_free(M.cantilever(2, 2, 6))
    inst = px.Instance(gpu_ctx, m)
    x, r = inst.solve_static(px.options(precision=prec, tol_max_error=1e-12, tol_min_impr=0.0, tol_min_step=0.0),
                             m.X0.ravel())
    assert r["result_name"] == "SUCCESS" and r["iterations"] == 1
    assert r["opt"] == 0.0 and np.array_equal(x, m.X0.ravel())


def test_fully_clamped_instance(gpu_ctx):
    """Every DoF fixed: the gradient is zero after fixing, the solve succeeds at once and
    nothing moves, in a batch with a loaded instance.  (The stopping test is the reference's
    strict ||g|| < tol, so a zero gradient needs a positive absolute floor: tol_rel times a
    zero starting gradient is zero.)"""
    m = M.cantilever(2, 2, 6)
    clamped = m.copy()
    clamped.fixed = np.ones_like(m.fixed)
    a, b = px.Instance(gpu_ctx, clamped), px.Instance(gpu_ctx, m)
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=1e-14, tol_min_impr=0.0,
                   tol_min_step=0.0)
    reps, xs = gpu_ctx.batch_solve([a, b], o, [clamped.X0.ravel(), m.X0.ravel()])
    assert reps[0]["result_name"] == "SUCCESS" and np.array_equal(xs[0], clamped.X0.ravel())
    assert reps[1]["result_name"] == "SUCCESS" and reps[1]["iterations"] > 1


def test_empty_batch(gpu_ctx):
    reps, _ = gpu_ctx.batch_solve([], px.options())
    assert reps == []
    assert gpu_ctx.batch_dynamic_step([], px.options(), 1e-3) == []


def test_dynamic_step_at_rest_without_load(gpu_ctx):
    """Implicit Euler from rest with no load and no velocity: the step keeps rest."""
    m = _load_free(M.cantilever(2, 2, 6))
    inst = px.Instance(gpu_ctx, m)
    inst.reset()
    x, v, r = inst.dynamic_step(px.options(tol_max_error=1e-12, tol_min_impr=0.0, tol_min_step=0.0), 1e-3)
    assert r["result_name"] == "SUCCESS"
    assert np.array_equal(x, m.X0.ravel()) and not np.any(v)


def _ls_case(model):
    if model == 0:
        return M.cantilever(2, 2, 4)
    return M.make_box(2, 2, 4, (0.04, 0.04, 0.08), 2e5, 0.35, 1000.0, 1, (0.0, -9.81, 0.0), clamp_face=4,
                      load_face=5, traction=(300.0, -500.0, 200.0))


@pytest.mark.parametrize("lst", [0, 2, 3, 4])
@pytest.mark.parametrize("model", [0, 1])
def test_line_search_types_on_gpu(gpu_ctx, model, lst):
    """LineSearch_None / Armijo / WolfeWeak / WolfeStrong on the device (plain FP64 path):
    the oracle's result, iteration and bisection counts and iterate.  Armijo's stall
    (its normalised-direction test refuses every trial once the step is shorter than about
    c1) ends at MAXITER in both; there only the result, the count and the iterate to 1e-4."""
    m = _ls_case(model)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, num_max_iters=40, lsearch_type=lst)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    inst = px.Instance(gpu_ctx, m)
    x, r = inst.solve_static(px.options(**kw), x0)
    assert (r["result"], r["iterations"]) == (ro["result"], ro["iterations"])
    if lst == 2 and ro["result_name"] == "MAXITER":
        assert disp_err(x, xo, x0) < 1e-4
    else:
        assert r["bisections"] == ro["bisections"]
        assert disp_err(x, xo, x0) < 1e-8


def test_wolfe_line_search_served_path(gpu_ctx):
    """The served FP32 path with a strong-Wolfe search reaches the oracle's equilibrium."""
    m = M.batch_instance(3, 11)
    orc, x0, g0, xr, _ = oracle_solution(m, 1e-10)
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0, lsearch_type=4)
    inst = px.Instance(gpu_ctx, m)
    x, r = inst.solve_static(o, x0)
    assert r["result_name"] == "SUCCESS"
    assert disp_err(x, xr, x0) < 1e-6


def test_soft_fixed_position_on_gpu(gpu_ctx):
    """Soft fixed-position conditions (EnergyElement_SoftConstraint, k/2 |x - t|^2 per
    node) on the device: energy, gradient and the assembled Hessian through the C ABI, the
    FP64 solve at the oracle's iterates, and the served FP32 solve at its equilibrium."""
    m = M.soft_clamped(M.cantilever(2, 2, 6), 1e5, target_shift=(1e-3, 2e-3, 0.0))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    rng = np.random.default_rng(4)
    x = x0 + 1e-3 * rng.standard_normal(orc.N)
    inst = px.Instance(gpu_ctx, m)
    E, g = inst.energy_gradient(x)
    assert abs(E - orc.energy(x)) <= 1e-10 * max(1.0, abs(orc.energy(x)))
    assert rel(g, orc.gradient(x)) < 1e-10
    vals = inst.hessian(x)
    assert rel(vals, orc.hessian(x)) < 1e-10
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-9 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    xg, r = px.Instance(gpu_ctx, m).solve_static(px.options(**kw), x0)
    assert r["result_name"] == "SUCCESS" and ro["result_name"] == "SUCCESS"
    assert (r["iterations"], r["bisections"]) == (ro["iterations"], ro["bisections"])
    assert disp_err(xg, xo, x0) < 1e-9
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    xs, rs = px.Instance(gpu_ctx, m).solve_static(o, x0)
    assert rs["result_name"] == "SUCCESS"
    assert disp_err(xs, xo, x0) < 1e-5


def test_batch_creation_equals_one_at_a_time(gpu_ctx):
    """phx_instances_create builds the host parts on several threads: the instances solve to
    the same bits as ones created one at a time; a bad mesh fails the whole call."""
    meshes = [M.batch_instance(3, i) for i in range(20, 26)]
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    a = gpu_ctx.create_instances(meshes)
    b = [px.Instance(gpu_ctx, m) for m in meshes]
    ra, xa = gpu_ctx.batch_solve(a, o, [m.X0.ravel().copy() for m in meshes])
    rb, xb = gpu_ctx.batch_solve(b, o, [m.X0.ravel().copy() for m in meshes])
    for u, v, p, q in zip(xa, xb, ra, rb):
        assert np.array_equal(u, v) and p["iterations"] == q["iterations"]
    bad = meshes[0].copy()
    bad.T = bad.T.copy()
    bad.T[0, 0] = bad.n + 5
    with pytest.raises(px.PhxError):
        gpu_ctx.create_instances([meshes[1], bad])


def test_negative_curvature_follows_eigen_cg(gpu_ctx):
    """A Newton step whose Hessian is indefinite: the FP64 PCG goes on through negative
    curvature as Eigen's ConjugateGradient does, and regularises only if the result fails
    b.x >= 0 (LinearSolver_EigenCG.cpp:95-107).  On this box the third step's PCG meets
    p.q < 0 twice and still converges with b.x > 0, so neither side regularises and the
    iterates stay the oracle's."""
    m = M.make_box(2, 1, 5, (0.02, 0.01, 0.05), 1.7e4, 0.28, 1000.0, M.MODEL_CONH, (0.0, 0.0, 0.0),
                   clamp_face=4, load_face=5, traction=(-2855.0, 2021.0, 2534.0))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0, try_steepest=1)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    assert ro["result_name"] == "SUCCESS" and ro["reg_trials"] == 0
    inst = px.Instance(gpu_ctx, m)
    x, r = inst.solve_static(px.options(**kw), x0)
    assert r["result_name"] == "SUCCESS" and r["reg_trials"] == 0, r
    assert r["iterations"] == ro["iterations"] and r["bisections"] == ro["bisections"]
    # CG through negative curvature is sensitive to the order of its sums: counts within 10 %
    assert abs(r["pcg_iterations"] - ro["lin_iterations"]) <= 0.1 * ro["lin_iterations"]
    assert disp_err(x, xo, x0) < 1e-9


def test_regularised_retries_match_oracle(gpu_ctx):
    """An FP64 solve whose linear solves need five regularised retries in all: the device
    takes them as LinearSolver_EigenCG does (up to 10 per solve, whatever ls_num_reg_trials)
    and keeps the oracle's iterates."""
    m = M.make_box(2, 1, 3, (0.02, 0.01, 0.03), 23300.0, 0.43, 1000.0, M.MODEL_CONH, (0.0, 0.0, 0.0),
                   clamp_face=4, load_face=5, traction=(2566.0, -1657.0, -2403.0))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, ls_num_reg_trials=1)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    assert ro["result_name"] == "SUCCESS" and ro["reg_trials"] == 5
    inst = px.Instance(gpu_ctx, m)
    x, r = inst.solve_static(px.options(**kw), x0)
    assert r["result_name"] == "SUCCESS" and r["reg_trials"] == 5, r
    assert r["iterations"] == ro["iterations"] and r["bisections"] == ro["bisections"]
    assert disp_err(x, xo, x0) < 1e-9


def test_renumbered_mesh_matches_oracle(gpu_ctx):
    """Unstructured numbering (random node ids, tet order and corner order): the FP64 solve
    keeps the oracle's iterates and the served solve reaches its equilibrium."""
    m = M.renumbered(M.batch_instance(3, 42), 2)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    inst = px.Instance(gpu_ctx, m)
    E, g = inst.energy_gradient(x0)
    assert abs(E - orc.energy(x0)) <= 1e-12 * max(1.0, abs(orc.energy(x0)))
    # At rest the elastic gradient cancels to zero: the device's displacement form returns the
    # load exactly, while the oracle's F = Ds Dm^-1 carries about 2.5e-11 of roundoff there.
    # The 1e-12 element bound is therefore checked away from rest, where the elastic part is
    # the gradient's own scale; at rest the bound is that roundoff's size.
    assert rel(g, orc.gradient(x0)) < 1e-9
    rng = np.random.default_rng(5)
    h = np.min(np.linalg.norm(m.X0[m.T[:, 1]] - m.X0[m.T[:, 0]], axis=1))
    xp = x0 + 0.03 * h * rng.standard_normal(x0.shape)
    Ep, gp = inst.energy_gradient(xp)
    gpo = orc.gradient(xp)
    assert abs(Ep - orc.energy(xp)) <= 1e-11 * max(abs(Ep), 1e-300) + 1e-15 * np.abs(orc.element_local(xp)[0]).sum()
    assert np.abs(gp - gpo).max() <= 1e-12 * np.abs(gpo).max()
    kw = dict(tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    x, r = inst.solve_static(px.options(**kw), x0)
    assert (r["result"], r["iterations"], r["bisections"]) == (ro["result"], ro["iterations"], ro["bisections"])
    assert disp_err(x, xo, x0) < 1e-9
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)
    inst.reset()
    x, r = inst.solve_static(o)
    if ro["result_name"] == "SUCCESS":
        # at a 1e-6 relative residual (the batch's served errors reach 3.8e-7)
        assert r["result_name"] == "SUCCESS" and disp_err(x, xo, x0) < 5e-6


def test_element_local_at_extreme_deformations(gpu_ctx):
    """The FP64 element kernels under a uniform deformation far from rest (every tet with
    the same F): strong compression, strong stretch and a shear, CoNH and StVK, against the
    oracle, whose material laws are pinned to the reference's code at such F."""
    rng = np.random.default_rng(11)
    U, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    V, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    if np.linalg.det(U) < 0:
        U[:, 0] *= -1
    if np.linalg.det(V) < 0:
        V[:, 0] *= -1
    maps = [U @ np.diag([0.05, 0.3, 0.8]) @ V.T, U @ np.diag([20.0, 3.0, 1.5]) @ V.T,
            np.array([[1.0, 0.9, 0.0], [0.0, 1.0, 0.4], [0.0, 0.0, 1.0]])]
    for model in (M.MODEL_CONH, M.MODEL_STVK):
        m = M.make_box(2, 2, 3, (0.02, 0.02, 0.03), 2e5, 0.4, 1000.0, model, (0.0, 0.0, 0.0), clamp_face=None)
        inst = px.Instance(gpu_ctx, m)
        orc = oracle.Oracle(m)
        for A in maps:
            x = (m.X0 @ A.T).ravel()
            E, g, H = inst.element_local(x, px.PREC_FP64)
            Eo, go, Ho = orc.element_local(x)
            assert np.max(np.abs(E - Eo) / np.maximum(np.abs(Eo), 1e-300)) < 1e-10
            assert np.max(np.abs(g - go)) <= 1e-10 * np.abs(go).max()
            assert np.max(np.abs(H - Ho)) <= 1e-10 * np.abs(Ho).max()
