"""Staged boundary-condition loading on the GPU, through the C ABI, against the oracle.

A BCondition advances one stage per Newton iteration start of a static solve (BCondition.cpp:
42-67); BC_FixDoF targets follow their animator and a soft stiffness ramps (BC_FixDoF.cpp:
80-121); SolveFull applies its stop rules only once every condition is loaded
(OptimSolver.cpp:213).  The FP64 device solve must take the oracle's decisions (result,
iterations, bisections) in its CG mode; the served FP32 solve must reach the same equilibrium.
"""
import numpy as np
import pytest

import oracle
import physim_gb300 as px
from physim_gb300 import mesh as M

pytestmark = pytest.mark.gpu

KW = dict(tol_min_impr=0.0, tol_min_step=0.0)


def rot_z(deg):
    t = np.deg2rad(deg)
    return np.array([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0.0, 0.0, 1.0]])


def disp_err(x, xr, x0):
    return float(np.linalg.norm(x - xr) / np.linalg.norm(xr - x0))


def oracle_solve(m, groups, num_stages, tol):
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    orc.set_staging(groups, num_stages, x0)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, tol_max_error=tol, **KW)
    return x0, xo, ro, orc.stage()


def test_staged_clamp_rotation_matches_oracle(gpu_ctx):
    m = M.cantilever(2, 2, 6)
    nodes = np.where(m.fixed.reshape(-1, 3).all(axis=1))[0]
    g = dict(num_stages=4, soft=0, move=rot_z(12.0) - np.eye(3), nodes=nodes)
    g0 = np.linalg.norm(oracle.Oracle(m).gradient(m.X0.ravel()))
    tol = 1e-6 * g0
    x0, xo, ro, stage = oracle_solve(m, [g], 4, tol)
    inst = px.Instance(gpu_ctx, m)
    inst.set_staging([g], 4)
    assert inst.stage() == (0, 4)
    x, r = inst.solve_static(px.options(tol_max_error=tol, **KW), x0)
    assert (r["result"], r["iterations"], r["bisections"]) == (ro["result"], ro["iterations"], ro["bisections"])
    assert inst.stage() == (stage, 4) == (4, 4)
    assert disp_err(x, xo, x0) < 1e-9
    # the served path from stage 0 again (phx_instance_reset takes the stage back), to the
    # oracle's absolute tolerance: a relative one would be taken after the first stage, whose
    # moved clamp makes ||g0|| far larger than the loads alone
    inst.reset()
    assert inst.stage()[0] == 0
    o = px.options(precision=px.PREC_FP32_REFINE, tol_max_error=tol, **KW)
    x32, r32 = inst.solve_static(o)
    assert r32["result_name"] == "SUCCESS" and inst.stage()[0] == 4
    assert disp_err(x32, xo, x0) < 5e-6


def test_staged_soft_ramp_and_gravity_stages(gpu_ctx):
    """A soft clamp whose stiffness ramps and whose targets shift over 3 stages, with six stages
    in all (a gravity condition with numStep 6 keeps the problem not fully constrained)."""
    m = M.soft_clamped(M.cantilever(2, 2, 5), 1e4)
    nodes = np.where(np.asarray(m.soft_k) > 0)[0]
    g = dict(num_stages=3, soft=1, k_start=1e2, k_end=1e6, shift=[1e-3, 0.0, 0.0], nodes=nodes)
    g0 = np.linalg.norm(oracle.Oracle(m).gradient(m.X0.ravel()))
    tol = 1e-6 * g0
    x0, xo, ro, stage = oracle_solve(m, [g], 6, tol)
    inst = px.Instance(gpu_ctx, m)
    inst.set_staging([g], 6)
    x, r = inst.solve_static(px.options(tol_max_error=tol, **KW), x0)
    assert (r["result"], r["iterations"], r["bisections"]) == (ro["result"], ro["iterations"], ro["bisections"])
    assert r["iterations"] >= 6 and inst.stage() == (stage, 6)
    assert disp_err(x, xo, x0) < 1e-9


def test_staged_instances_batch_equals_alone(gpu_ctx):
    """Instances with different staging solved together give the bits they give alone."""
    meshes = [M.cantilever(2, 2, 6), M.cantilever(2, 3, 5)]
    stagings = [[dict(num_stages=3, soft=0, move=rot_z(8.0) - np.eye(3),
                      nodes=np.where(meshes[0].fixed.reshape(-1, 3).all(axis=1))[0])],
                [dict(num_stages=5, soft=0, shift=[0.0, 1e-3, 0.0],
                      nodes=np.where(meshes[1].fixed.reshape(-1, 3).all(axis=1))[0])]]
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, **KW)
    alone = []
    for m, st in zip(meshes, stagings):
        inst = px.Instance(gpu_ctx, m)
        inst.set_staging(st, 0)
        alone.append(inst.solve_static(o, m.X0.ravel())[0])
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    for inst, st in zip(insts, stagings):
        inst.set_staging(st, 0)
    reps, xs = gpu_ctx.batch_solve(insts, o, [m.X0.ravel() for m in meshes])
    for x, a, r in zip(xs, alone, reps):
        assert r["result_name"] == "SUCCESS" and np.array_equal(x, a)


def test_staging_rejects_inconsistent_groups(gpu_ctx):
    m = M.cantilever(2, 2, 4)
    inst = px.Instance(gpu_ctx, m)
    free = np.where(~m.fixed.reshape(-1, 3).any(axis=1))[0][:3]
    with pytest.raises(px.PhxError) as ei:  # a hard group must hold fixed nodes
        inst.set_staging([dict(num_stages=2, soft=0, nodes=free)], 2)
    assert ei.value.code == px.PHX_EINVAL
    with pytest.raises(px.PhxError):  # a soft group needs soft records
        inst.set_staging([dict(num_stages=2, soft=1, nodes=free)], 2)
    with pytest.raises(px.PhxError):  # num_stages >= 1
        inst.set_staging([dict(num_stages=0, soft=0, nodes=free)], 2)


def test_scene_file_solves_like_the_oracle(gpu_ctx, tmp_path):
    """A scene file (TetGen mesh, FixPosition clamp moved by a Transform3D animation over 3
    stages, gravity) through phx_scene_instance, against the oracle given the scene's mesh and
    staging.  Scale 0 in the animation makes the reference's I + a R S a pure translation."""
    import os
    from test_scene import scene_xml, write_tetgen
    ref = M.cantilever(2, 2, 6)
    write_tetgen(os.path.join(tmp_path, "bar"), ref.X0, ref.T)
    bc = ('<bc type="FixPosition" soft="false" numStep="3"><selection type="BoxNodes" field="Pos0">'
          '<minCorner>-1e-9, -1e-9, -1e-9</minCorner><maxCorner>1, 1, 1e-9</maxCorner></selection>'
          '<animation type="Transform3D"><position>0, 0.004, 0</position><scale>0, 0, 0</scale></animation></bc>'
          '<bc type="Gravity"><gravity>0, -9.81, 0</gravity></bc>')
    p = os.path.join(tmp_path, "scene.xml")
    with open(p, "w") as f:
        f.write(scene_xml(boundary=bc))
    sc = px.Scene(p)
    m, x0 = sc.mesh()
    groups = sc.staging()
    info = sc.info()
    orc = oracle.Oracle(m)
    g0 = np.linalg.norm(orc.gradient(x0))
    tol = 1e-6 * g0
    orc.set_staging(groups, info["num_stages"], x0)
    xo, ro = orc.solve_static(x0, ls_solver=1, cg_block_jacobi=1, tol_max_error=tol, **KW)
    inst = sc.instance(gpu_ctx)
    o = sc.options()
    o.tol_max_error, o.tol_min_impr, o.tol_min_step = tol, 0.0, 0.0
    x, r = inst.solve_static(o)
    assert (r["result"], r["iterations"], r["bisections"]) == (ro["result"], ro["iterations"], ro["bisections"])
    assert inst.stage() == (orc.stage(), 3)
    assert disp_err(x, xo, x0) < 1e-9
    clamp = groups[0]["nodes"]
    assert np.abs(x.reshape(-1, 3)[clamp] - (m.X0[clamp] + [0.0, 0.004, 0.0])).max() < 1e-10
