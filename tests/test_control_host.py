"""The product's Newton / line-search state machine, driven on the host, against the oracle's SolveFull."""
import numpy as np
import pytest

import oracle
from physim_gb300 import mesh as M
import ctl_harness as H
from conftest import rel


def _case(model=0, dims=(2, 2, 6)):
    if model == 0:
        return M.cantilever(*dims)
    return M.make_box(*dims, (0.02 * dims[0], 0.02 * dims[1], 0.02 * dims[2]), 2e5, 0.35, 1000.0, 1,
                      (0.0, -9.81, 0.0), clamp_face=4, load_face=5, traction=(300.0, -500.0, 200.0))


@pytest.mark.parametrize("model", [0, 1])
def test_static_newton_matches_oracle(ctl_shim, model):
    m = _case(model)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    # below ~1e-9 the strict E_new < E_old test sits in double-precision noise for the StVK case
    tol = (1e-9 if model == 0 else 1e-6) * g0
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, tol_max_error=tol, tol_min_impr=0.0,
                              tol_min_step=0.0)
    opts = H.make_opts(tol_max_error=tol, tol_min_impr=0.0, tol_min_step=0.0)
    x, _, s = H.run(ctl_shim, orc, x0, opts)
    assert ro["result_name"] == "SUCCESS" and s.result == 1
    assert s.it == ro["iterations"]
    assert s.total_bis == ro["bisections"]
    assert rel(x - x0, xo - x0) < 1e-9
    assert abs(s.obj - ro["obj"]) <= 1e-10 * abs(ro["obj"])
    log = orc.last_log()
    assert s.opt0 == pytest.approx(g0, rel=1e-12)


def test_default_tolerances_stop_like_the_reference(ctl_shim):
    # reference defaults (absolute tolMaxError 1e-6, tolMinImpr 1e-9, tolMinStep 1e-5): MINIMPR/MINSTEP paths
    m = _case(0, (2, 2, 4))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts())
    assert s.result == ro["result"] and s.it == ro["iterations"]
    assert rel(x - x0, xo - x0) < 1e-7


def test_steepest_only(ctl_shim):
    m = _case(0, (1, 1, 3))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    xo, ro = orc.solve_static(x0, qp_solver=0, num_max_iters=15)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(qp_solver=0, num_max_iters=15))
    assert s.result == ro["result"] and s.it == ro["iterations"] and s.total_bis == ro["bisections"]
    assert rel(x - x0, xo - x0) < 1e-10


def test_implicit_euler_step_matches_oracle(ctl_shim):
    m = M.make_box(2, 2, 3, (0.02, 0.02, 0.03), 1e5, 0.3, 1000.0, 0, (0.0, -9.81, 0.0), clamp_face=2)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    v0 = np.zeros(orc.N)
    v0[1::3] = 0.2
    v0[m.fixed.astype(bool)] = 0
    dt = 1e-3
    kw = dict(tol_max_error=1e-11, tol_min_impr=0.0, tol_min_step=0.0)
    xo, vo, ro = orc.solve_dynamic(x0, v0, dt, ls_solver=1, cg_block_jacobi=1, **kw)
    x, v, s = H.run(ctl_shim, orc, x0, H.make_opts(dynamic=1, dt=dt, **kw), dynamic=True, v0=v0)
    assert s.result == ro["result"] == 1 and s.it == ro["iterations"]
    assert rel(x - x0, xo - x0) < 1e-9
    assert rel(v, vo) < 1e-9


def test_max_iterations_cap(ctl_shim):
    m = _case(0, (2, 2, 6))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(num_max_iters=2, tol_max_error=1e-14))
    assert s.result == 5 and s.it == 2  # MAXITER after two SolveSteps


def test_inexact_newton_forcing_converges_to_the_same_point(ctl_shim):
    """The FP32 path's Eisenstat-Walker forcing terms change the linear tolerances, not the answer."""
    m = _case(0, (2, 2, 6))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-9 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    xo, ro = orc.solve_static(x0, **kw)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(precision=1, **kw))
    assert s.result == 1 and s.opt <= 1e-9 * g0
    assert rel(x - x0, xo - x0) < 1e-8
    _, _, s64 = H.run(ctl_shim, orc, x0, H.make_opts(**kw))
    assert s.pcg_total < s64.pcg_total  # looser linear solves on the way


def test_parallel_line_search_takes_the_same_decisions(ctl_shim):
    """Trials evaluated eight at a time (after two rejections) and scanned in order give the
    same iterates, bisection count and result as the one-at-a-time line search, on a StVK
    box that needs hundreds of bisections."""
    m = M.make_box(2, 2, 6, (0.04, 0.04, 0.12), 2e5, 0.35, 1000.0, 1, (0.0, -9.81, 0.0), clamp_face=4,
                   load_face=5, traction=(20000.0, -30000.0, 10000.0))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    runs = []
    for k in (0, 8):
        opts = H.make_opts(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, ls_parallel=k)
        x, _, s = H.run(ctl_shim, orc, x0, opts)
        runs.append((x, s.result, s.it, s.total_bis, H.stats["evalk"]))
    (xa, ra, ia, ba, ka), (xb, rb, ib, bb, kb) = runs
    assert ba > 100 and ka == 0 and kb > 0 and kb < ba / 4
    assert (ra, ia, ba) == (rb, ib, bb)
    assert np.array_equal(xa, xb)


@pytest.mark.parametrize("lst", [0, 2, 3, 4])
@pytest.mark.parametrize("model", [0, 1])
def test_line_search_types_match_oracle(ctl_shim, model, lst):
    """LineSearch_None / Armijo / WolfeWeak / WolfeStrong (OptimSolver.cpp:738-900): the
    state machine takes the oracle's decisions (result, iterations, bisections, iterate).
    The reference's Armijo test uses the normalised direction, c1 (d/|d|).g, so once the
    Newton step is shorter than about c1 no trial passes: both stall to MAXITER, failing
    searches whose last trial lowered the energy counting as steps; their bisection counts
    there are decided in rounding noise and are not compared."""
    m = _case(model, (2, 2, 4))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, num_max_iters=40)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, lsearch_type=lst, **kw)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(lsearch_type=lst, **kw))
    assert (s.result, s.it) == (ro["result"], ro["iterations"])
    if lst == 2 and ro["result_name"] == "MAXITER":  # stalled short of the tolerance
        assert rel(x - x0, xo - x0) < 1e-4
    else:
        assert s.total_bis == ro["bisections"]
        assert rel(x - x0, xo - x0) < 1e-8


def test_armijo_parallel_trials_take_the_same_decisions(ctl_shim):
    """The Armijo test reads energies only, so its trials may be evaluated eight at a time:
    the same iterates, bisections and result as one at a time."""
    m = M.make_box(2, 2, 6, (0.04, 0.04, 0.12), 2e5, 0.35, 1000.0, 1, (0.0, -9.81, 0.0), clamp_face=4,
                   load_face=5, traction=(20000.0, -30000.0, 10000.0))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    runs = []
    for k in (0, 8):
        opts = H.make_opts(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, ls_parallel=k,
                           lsearch_type=2)
        x, _, s = H.run(ctl_shim, orc, x0, opts)
        runs.append((x, s.result, s.it, s.total_bis, H.stats["evalk"]))
    (xa, ra, ia, ba, ka), (xb, rb, ib, bb, kb) = runs
    assert ba > 20 and ka == 0 and kb > 0
    assert (ra, ia, ba) == (rb, ib, bb)
    assert np.array_equal(xa, xb)


def test_wolfe_searches_evaluate_one_trial_at_a_time(ctl_shim):
    m = _case(1, (2, 2, 4))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    H.run(ctl_shim, orc, x0, H.make_opts(lsearch_type=3, ls_parallel=8, num_max_iters=10))
    assert H.stats["evalk"] == 0


def test_soft_fixed_position_matches_oracle(ctl_shim):
    """A cantilever held by soft fixed-position conditions (BC_FixDoF soft mode) instead of
    hard-fixed DoFs, with shifted targets: the oracle's decisions and iterate."""
    m = M.soft_clamped(M.cantilever(2, 2, 4), 1e5, target_shift=(0.0, 2e-3, 0.0))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(**kw))
    assert ro["result_name"] == "SUCCESS"
    assert (s.result, s.it, s.total_bis) == (ro["result"], ro["iterations"], ro["bisections"])
    assert rel(x - x0, xo - x0) < 1e-9


@pytest.mark.parametrize("lst", [1, 3, 4])
@pytest.mark.parametrize("idx", [16, 38, 46, 48, 57])
def test_line_searches_on_batch_instances(ctl_shim, idx, lst):
    """Small batch instances (CoNH and StVK, 196-455 nodes): Simple and the Wolfe searches
    take the oracle's decisions exactly (result, iterations, bisections) and reach its
    iterate.  (Armijo's decisions there are decided in rounding noise once its normalised
    test stalls, see test_line_search_types_match_oracle.)"""
    m = M.batch_instance(3, idx)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, num_max_iters=60, lsearch_type=lst)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(**kw))
    assert ro["result_name"] == "SUCCESS"
    assert (s.result, s.it, s.total_bis) == (ro["result"], ro["iterations"], ro["bisections"])
    assert rel(x - x0, xo - x0) < 1e-10


@pytest.mark.parametrize("k", [1e4, 1e6])
@pytest.mark.parametrize("idx", [16, 48])
def test_soft_clamped_batch_instances(ctl_shim, idx, k):
    """Batch instances with their clamped face held by soft fixed-position conditions of two
    stiffnesses: the oracle's decisions and iterate."""
    m = M.soft_clamped(M.batch_instance(3, idx), k)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    # (below about 3e-7 g0 the energy comparison of the line search is in rounding noise)
    kw = dict(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, num_max_iters=60)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(**kw))
    assert ro["result_name"] == "SUCCESS"
    assert (s.result, s.it, s.total_bis) == (ro["result"], ro["iterations"], ro["bisections"])
    assert rel(x - x0, xo - x0) < 1e-9


@pytest.mark.parametrize("lst", [1, 4])
def test_soft_clamped_implicit_euler_step(ctl_shim, lst):
    """An implicit-Euler step of a box held by soft fixed-position conditions (inertia and
    soft terms in one gradient), with the Simple and the strong-Wolfe search: the oracle's
    result, iterations and state."""
    base = M.make_box(2, 2, 3, (0.02, 0.02, 0.03), 1e5, 0.3, 1000.0, 0, (0.0, -9.81, 0.0), clamp_face=2)
    m = M.soft_clamped(base, 1e5)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    v0 = np.zeros(orc.N)
    v0[1::3] = 0.2
    dt = 1e-3
    # ||g|| starts at about 69 here (the soft-held nodes move with v0); 1e-7 is above the
    # band where the line search's energy comparison is in rounding noise
    kw = dict(tol_max_error=1e-7, tol_min_impr=0.0, tol_min_step=0.0, lsearch_type=lst)
    xo, vo, ro = orc.solve_dynamic(x0, v0, dt, ls_solver=1, cg_block_jacobi=1, **kw)
    x, v, s = H.run(ctl_shim, orc, x0, H.make_opts(dynamic=1, dt=dt, **kw), dynamic=True, v0=v0)
    assert ro["result_name"] == "SUCCESS"
    assert (s.result, s.it, s.total_bis) == (ro["result"], ro["iterations"], ro["bisections"])
    assert rel(x - x0, xo - x0) < 1e-9
    assert rel(v, vo) < 1e-9


def test_random_options_match_oracle(ctl_shim):
    """Seeded option combinations on small boxes: step type, steepest fallback, line search
    (None, Simple, WolfeWeak, WolfeStrong), its factor and try limit, trials one at a time or
    eight per round, step clamp, iteration cap and the minimum-step / minimum-improvement
    tests.  Tolerances stop well above the
    band where energy comparisons are decided by rounding; the decisions, counts and iterate
    must then be the oracle's.  (Armijo compares against a normalised direction and stalls
    into that band whenever the step is shorter than c1; it has its own tests above.)"""
    rng = np.random.default_rng(7)
    checked = 0
    for case in range(120):
        model = int(rng.integers(0, 2))
        dims = (int(rng.integers(1, 3)), int(rng.integers(1, 3)), int(rng.integers(2, 6)))
        E = 10 ** rng.uniform(4, 6)
        nu = rng.uniform(0.2, 0.45)
        trac = tuple(rng.uniform(-1, 1, 3) * 10 ** rng.uniform(2, 3.5))
        grav = (0.0, -9.81, 0.0) if rng.random() < 0.5 else (0.0, 0.0, 0.0)
        m = M.make_box(*dims, (0.01 * dims[0], 0.01 * dims[1], 0.01 * dims[2]), E, nu, 1000.0, model, grav,
                       clamp_face=4, load_face=5, traction=trac)
        orc = oracle.Oracle(m)
        x0 = orc.rest()
        g0 = float(np.linalg.norm(orc.gradient(x0)))
        o = dict(qp_solver=int(rng.random() < 0.85), try_steepest=int(rng.integers(0, 2)),
                 lsearch_type=int(rng.choice([0, 1, 3, 4])), lsearch_alpha=float(rng.choice([0.5, 0.3])),
                 lsearch_num_try=int(rng.choice([3, 8, 32])),
                 max_step_size=float(rng.choice([1000.0, 1e-3, 3e-4])), num_max_iters=int(rng.choice([6, 25, 60])),
                 tol_max_error=float(rng.choice([1e-3, 1e-4])) * g0,
                 tol_min_step=float(rng.choice([1e-5, 0.0])), tol_min_impr=float(rng.choice([1e-9, 0.0])))
        xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **o)
        par = int(rng.choice([0, 8]))  # line-search trials one at a time or eight per round
        x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(ls_parallel=par, **o))
        key = (case, par, o)
        assert (s.result, s.it, s.total_bis) == (ro["result"], ro["iterations"], ro["bisections"]), key
        assert rel(x - x0, xo - x0) < 1e-8, key
        checked += 1
    assert checked == 120


def test_random_dynamic_and_soft_cases_match_oracle(ctl_shim):
    """Seeded implicit-Euler steps and static solves, half of them with soft fixed-position
    clamps, under random options (as above): the same decisions, counts and iterate."""
    rng = np.random.default_rng(5)
    for case in range(80):
        model = int(rng.integers(0, 2))
        dims = (int(rng.integers(1, 3)), int(rng.integers(1, 3)), int(rng.integers(2, 5)))
        E = 10 ** rng.uniform(4, 6)
        nu = rng.uniform(0.2, 0.45)
        trac = tuple(rng.uniform(-1, 1, 3) * 10 ** rng.uniform(2, 3.5))
        m = M.make_box(*dims, (0.01 * dims[0], 0.01 * dims[1], 0.01 * dims[2]), E, nu, 1000.0, model,
                       (0.0, -9.81, 0.0), clamp_face=4, load_face=5, traction=trac)
        if rng.random() < 0.5:
            m = M.soft_clamped(m, float(10 ** rng.uniform(1, 4)), tuple(rng.uniform(-1, 1, 3) * 1e-3))
        orc = oracle.Oracle(m)
        x0 = orc.rest()
        dyn = rng.random() < 0.5
        o = dict(qp_solver=int(rng.random() < 0.9), try_steepest=int(rng.integers(0, 2)),
                 lsearch_type=int(rng.choice([0, 1, 3, 4])), lsearch_alpha=float(rng.choice([0.5, 0.3])),
                 lsearch_num_try=int(rng.choice([3, 8, 32])), max_step_size=float(rng.choice([1000.0, 1e-3])),
                 num_max_iters=int(rng.choice([6, 25])), tol_min_step=float(rng.choice([1e-5, 0.0])),
                 tol_min_impr=float(rng.choice([1e-9, 0.0])))
        if dyn:
            dt = float(rng.choice([1e-3, 1e-2]))
            v0 = np.zeros(orc.N)
            v0[1::3] = rng.uniform(-0.5, 0.5)
            v0[m.fixed.astype(bool)] = 0
            o["tol_max_error"] = 1e-6
            xo, vo, ro = orc.solve_dynamic(x0, v0, dt, ls_solver=1, cg_block_jacobi=1, **o)
            x, v, s = H.run(ctl_shim, orc, x0, H.make_opts(dynamic=1, dt=dt, **o), dynamic=True, v0=v0)
            assert rel(v, vo) < 1e-8, (case, o)
        else:
            g0 = float(np.linalg.norm(orc.gradient(x0)))
            o["tol_max_error"] = float(rng.choice([1e-3, 1e-4])) * g0
            xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **o)
            x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(**o))
        assert (s.result, s.it, s.total_bis) == (ro["result"], ro["iterations"], ro["bisections"]), (case, dyn, o)
        assert rel(x - x0, xo - x0) < 1e-8, (case, dyn, o)


@pytest.mark.parametrize("trials", [1, 3, 10])
def test_linear_solve_regularises_ten_times_whatever_ls_num_reg_trials(ctl_shim, trials):
    """LinearSolver_EigenCG regularises up to LinearSolverOptions::regIters = 10 times, a
    value OptimSolver never sets from lsNumRegTrials (its own loop computes one step): a
    solve that needs five regularised retries takes them with any ls_num_reg_trials."""
    m = M.make_box(2, 1, 3, (0.02, 0.01, 0.03), 23300.0, 0.43, 1000.0, M.MODEL_CONH, (0.0, 0.0, 0.0),
                   clamp_face=4, load_face=5, traction=(2566.0, -1657.0, -2403.0))
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = np.linalg.norm(orc.gradient(x0))
    kw = dict(tol_max_error=1e-6 * g0, tol_min_impr=0.0, tol_min_step=0.0, ls_num_reg_trials=trials)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    x, _, s = H.run(ctl_shim, orc, x0, H.make_opts(**kw))
    assert ro["result_name"] == "SUCCESS" and ro["reg_trials"] == 5
    assert (s.result, s.it, s.total_bis, s.total_reg) == (ro["result"], ro["iterations"], ro["bisections"], 5)
    assert rel(x - x0, xo - x0) < 1e-12
