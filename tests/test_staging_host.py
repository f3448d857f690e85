"""Staged boundary-condition loading, driven on the host: the product's state machine
(newton_control.h through tests/ctl_harness.py) against the oracle's SolveFull.

The reference advances every boundary condition one stage per Newton iteration start
(BCondition::StepLoading, BCondition.cpp:42-67, via OptimProblem_BasicStatic::OnIterStart),
moves the targets of BC_FixDoF by its animator (VectorAnimator_LerpT3D) and ramps a soft
stiffness from kAini to kAend (BC_FixDoF.cpp:80-121); SolveFull applies its stop rules only
once every condition is at its last stage (OptimSolver.cpp:213).  The oracle restates that
(test_oracle covers it against known answers); here the device's state machine must take
the same decisions, iteration for iteration.
"""
import numpy as np
import pytest

import oracle
from physim_gb300 import mesh as M
import ctl_harness as H
from conftest import rel

KW = dict(tol_min_impr=0.0, tol_min_step=0.0)


def rot_z(deg):
    t = np.deg2rad(deg)
    return np.array([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0.0, 0.0, 1.0]])


def clamped_nodes(m):
    return np.where(m.fixed.reshape(-1, 3).all(axis=1))[0]


def opts_for(groups, num_stages, **kw):
    most = max([num_stages] + [g.get("num_stages", 1) for g in groups])
    moves = any(g.get("soft", 0) or np.any(np.asarray(g.get("move", 0)) != 0) or np.any(np.asarray(g.get("shift", 0)) != 0)
                for g in groups)
    return H.make_opts(num_stages=most, stage_values=int(moves), **kw)


def compare(ctl_shim, m, groups, num_stages, tol, dynamic=False, dt=0.0, v0=None):
    ref = oracle.Oracle(m)
    ev = oracle.Oracle(m)  # the harness's evaluator, its soft records driven by the state machine
    x0 = ref.rest()
    ref.set_staging(groups, num_stages, x0)
    if dynamic:
        xo, vo, ro = ref.solve_dynamic(x0, v0, dt, ls_solver=1, cg_block_jacobi=1, tol_max_error=tol, **KW)
    else:
        xo, ro = ref.solve_static(x0, ls_solver=1, cg_block_jacobi=1, tol_max_error=tol, **KW)
    o = opts_for(groups, num_stages, tol_max_error=tol, dynamic=int(dynamic), dt=dt, **KW)
    x, v, s = H.run(ctl_shim, ev, x0, o, dynamic=dynamic, v0=v0, staging=(groups, x0))
    assert (s.result, s.it, s.total_bis) == (ro["result"], ro["iterations"], ro["bisections"]), (s.result, s.it, ro)
    assert s.stage == ref.stage()
    assert rel(x - x0, xo - x0) < 1e-9
    return x, s, ro, ref


def test_hard_clamp_rotated_over_stages(ctl_shim):
    """The clamped end turned 12 degrees about the bar's axis over 4 stages: the reference's
    animator applies I + a (R - I) here (move = R - I), the clamp ends on R X0."""
    m = M.cantilever(2, 2, 6)
    nodes = clamped_nodes(m)
    R = rot_z(12.0)
    g = dict(num_stages=4, soft=0, move=R - np.eye(3), nodes=nodes)
    g0 = np.linalg.norm(oracle.Oracle(m).gradient(m.X0.ravel()))
    x, s, ro, _ = compare(ctl_shim, m, [g], 4, 1e-6 * g0)
    assert s.stage == 4 and ro["result_name"] == "SUCCESS"
    # the clamp ends on R X0 (to the CG tolerance: the start guess of each step carries the
    # clamp's move, which the inexact linear solve takes back to ~1e-9 of it)
    assert np.abs(x.reshape(-1, 3)[nodes] - m.X0[nodes] @ R.T).max() < 1e-10


def test_loaded_only_after_the_last_stage(ctl_shim):
    """Gravity loaded over 6 stages (numStep) changes no value: only SolveFull's stop rules wait,
    so a problem that converges in fewer iterations keeps iterating until the last stage."""
    m = M.cantilever(1, 1, 3)
    g0 = np.linalg.norm(oracle.Oracle(m).gradient(m.X0.ravel()))
    x, s, ro, _ = compare(ctl_shim, m, [], 6, 1e-6 * g0)
    assert s.stage == 6 and s.it >= 6


def test_soft_targets_and_stiffness_ramp(ctl_shim):
    """A soft clamp (BC_FixDoF soft mode) whose stiffness ramps 1e2 -> 1e6 and whose targets
    shift 1 mm along x over 3 stages."""
    base = M.cantilever(2, 2, 5)
    m = M.soft_clamped(base, 1e4)
    nodes = np.where(np.asarray(m.soft_k) > 0)[0]
    g = dict(num_stages=3, soft=1, k_start=1e2, k_end=1e6, shift=[1e-3, 0.0, 0.0], nodes=nodes)
    g0 = np.linalg.norm(oracle.Oracle(m).gradient(m.X0.ravel()))
    compare(ctl_shim, m, [g], 3, 1e-6 * g0)


def test_two_groups_with_their_own_stage_counts(ctl_shim):
    """Two hard groups, one loaded in 2 stages and one in 5 (each at min(stage, N) / N)."""
    m = M.make_box(2, 2, 4, (0.02, 0.02, 0.04), 2e5, 0.3, 1000.0, 0, (0.0, -9.81, 0.0), clamp_face=None)
    fx = np.zeros(m.n, dtype=bool)
    bot = np.where(m.X0[:, 2] < 1e-12)[0]
    top = np.where(m.X0[:, 2] > 0.04 - 1e-12)[0]
    fx[bot] = True
    fx[top] = True
    m.fixed = np.repeat(fx, 3).astype(np.uint8)
    groups = [dict(num_stages=2, soft=0, move=rot_z(5.0) - np.eye(3), nodes=bot),
              dict(num_stages=5, soft=0, shift=[0.0, 0.0, 2e-3], nodes=top)]
    g0 = np.linalg.norm(oracle.Oracle(m).gradient(m.X0.ravel()))
    x, s, ro, _ = compare(ctl_shim, m, groups, 0, 1e-6 * max(g0, 1e-12) + 1e-12)
    assert s.stage == 5


def test_dynamic_step_stages_soft_targets_only(ctl_shim):
    """Implicit Euler: one stage per step at its start; the predictor overwrites every position
    afterwards, so only soft targets and stiffness take effect (OptimProblem_BasicDynamic.cpp:121-135)."""
    base = M.make_box(2, 2, 3, (0.02, 0.02, 0.03), 1e5, 0.3, 1000.0, 0, (0.0, -9.81, 0.0), clamp_face=None)
    m = M.soft_clamped(base, 1e3) if np.any(base.fixed) else base
    if getattr(m, "soft_k", None) is None:
        k = np.zeros(m.n)
        k[m.X0[:, 2] < 1e-12] = 1e3
        m.soft_k = k
    nodes = np.where(np.asarray(m.soft_k) > 0)[0]
    g = dict(num_stages=4, soft=1, k_start=1e2, k_end=1e4, shift=[0.0, 1e-3, 0.0], nodes=nodes)
    v0 = np.zeros(3 * m.n)
    compare(ctl_shim, m, [g], 4, 1e-11, dynamic=True, dt=1e-3, v0=v0)


def test_stage_persists_across_solves(ctl_shim):
    """A solve cut off by its iteration cap leaves the conditions at their stage; the next
    solve goes on from there (the reference's BCs keep m_curStage between SolveFull calls)."""
    m = M.cantilever(2, 2, 5)
    nodes = clamped_nodes(m)
    g = dict(num_stages=6, soft=0, move=rot_z(10.0) - np.eye(3), nodes=nodes)
    ref = oracle.Oracle(m)
    ev = oracle.Oracle(m)
    x0 = ref.rest()
    ref.set_staging([g], 6, x0)
    o = opts_for([g], 6, tol_max_error=1e-9, num_max_iters=3, **KW)
    x1o, r1 = ref.solve_static(x0, ls_solver=1, cg_block_jacobi=1, tol_max_error=1e-9, num_max_iters=3, **KW)
    x1, _, s1 = H.run(ctl_shim, ev, x0, o, staging=([g], x0))
    assert r1["result_name"] == "MAXITER" and s1.result == 5 and s1.stage == ref.stage() == 3
    assert rel(x1 - x0, x1o - x0) < 1e-9
    o2 = opts_for([g], 6, tol_max_error=1e-9, **KW)
    x2o, r2 = ref.solve_static(x1o, ls_solver=1, cg_block_jacobi=1, tol_max_error=1e-9, **KW)
    x2, _, s2 = H.run(ctl_shim, ev, x1, o2, staging=([g], x0), stage=s1.stage)
    assert (s2.result, s2.it) == (r2["result"], r2["iterations"]) and s2.stage == ref.stage() == 6
    assert rel(x2 - x0, x2o - x0) < 1e-9
