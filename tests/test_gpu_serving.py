"""Serving on the GPU: cold requests built at admission, the memory budget with eviction of
idle instances, implicit-step requests, and refusals reported per request.

Each served result is compared bit for bit with the same solve made through the plain
entry points on an instance created the usual way: the server runs the same device code
with per-instance reductions, so batching must not change a single bit.
"""
import time

import numpy as np
import pytest

import physim_gb300 as px
from physim_gb300 import mesh as M

pytestmark = pytest.mark.gpu

SERVED = dict(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)


def drain(srv, want, limit=100000):
    done = {}
    for _ in range(limit):
        active, queued = srv.progress()
        done.update(dict(srv.poll()))
        if want <= set(done):
            return done
        if active == 0 and queued > 0:
            time.sleep(5e-4)  # cold requests whose patterns are still being built on the host
    raise AssertionError(f"requests {sorted(want - set(done))} did not finish")


def alone(ctx, m, o, x=None):
    inst = px.Instance(ctx, m)
    xs, r = inst.solve_static(o, m.X0.ravel() if x is None else x)
    return inst, xs, r


def test_cold_requests_equal_create_then_solve(gpu_ctx):
    meshes = [M.serving_request(11, i) for i in range(6)]
    meshes = [m for m in meshes if m.m < 30000][:4]
    o = px.options(**SERVED)
    ref = [alone(gpu_ctx, m, o)[1] for m in meshes]
    srv = px.Server(gpu_ctx, max_slots=8, budget_bytes=8 << 30, opts=o)
    try:
        insts = [srv.submit_mesh(m, k) for k, m in enumerate(meshes)]
        done = drain(srv, set(range(len(meshes))))
        for k, inst in enumerate(insts):
            assert done[k]["result_name"] == "SUCCESS" and done[k]["status"] == px.PHX_OK
            assert np.array_equal(inst.positions(), ref[k])
        st = srv.stats()
        assert st["resident"] == len(meshes) and st["evictions"] == 0
        assert st["in_use"] == st["peak"] > 0
    finally:
        srv.close()
    for inst in insts:
        inst.close()


def test_budget_evicts_idle_instances_and_warm_resolve_rebuilds(gpu_ctx):
    a, b = M.serving_request(11, 0), M.serving_request(11, 1)
    o = px.options(**SERVED)
    # device bytes of each, measured by a server that holds both
    srv = px.Server(gpu_ctx, max_slots=4, budget_bytes=8 << 30, opts=o)
    ia = srv.submit_mesh(a, 0)
    drain(srv, {0})
    bytes_a = srv.stats()["in_use"]
    ib = srv.submit_mesh(b, 1)
    drain(srv, {1})
    bytes_b = srv.stats()["in_use"] - bytes_a
    srv.close()
    ia.close()
    ib.close()
    # a budget that holds either instance but not both
    budget = max(bytes_a, bytes_b) + min(bytes_a, bytes_b) // 2
    srv = px.Server(gpu_ctx, max_slots=4, budget_bytes=budget, opts=o)
    try:
        ia = srv.submit_mesh(a, 0)
        drain(srv, {0})
        xa = ia.positions()
        ib = srv.submit_mesh(b, 1)
        drain(srv, {1})
        st = srv.stats()
        assert st["evictions"] == 1 and st["resident"] == 1 and st["peak"] <= budget
        # the evicted instance keeps its solution on the host
        assert np.array_equal(ia.positions(), xa)
        with pytest.raises(px.PhxError) as ei:
            ia.energy_gradient()
        assert ei.value.code == px.PHX_EBUSY
        # warm re-solve of the evicted instance under a perturbed load: rebuilt from its kept
        # mesh and positions, it evicts b in turn
        a2 = M.perturb_load(a, 11, 0)
        ia.update_load(a2.force, a2.gravity)
        srv.submit(ia, 2)
        done = drain(srv, {2})
        assert done[2]["result_name"] == "SUCCESS"
        st = srv.stats()
        assert st["evictions"] == 2 and st["peak"] <= budget
        # the same warm re-solve through the plain entry points: a fresh instance of the
        # perturbed mesh started from the first solution
        _, xw, rw = alone(gpu_ctx, a2, o, xa)
        assert np.array_equal(ia.positions(), xw)
        assert done[2]["iterations"] == rw["iterations"]
    finally:
        srv.close()
    ia.close()
    ib.close()


def test_implicit_step_requests_equal_dynamic_step(gpu_ctx):
    meshes = [M.make_box(3, 3, 4, (0.03, 0.03, 0.04), 2e5, 0.45, 1000.0, M.MODEL_CONH, (0.0, -9.81, 0.0),
                         clamp_face=4) for _ in range(2)]
    o = px.options(**SERVED)
    dt = 1e-3
    ref = []
    for m in meshes:
        inst = px.Instance(gpu_ctx, m)
        x, v = m.X0.ravel().copy(), np.zeros(3 * m.n)
        for _ in range(3):
            x, v, r = inst.dynamic_step(o, dt, x, v)
        ref.append((x, v))
    srv = px.Server(gpu_ctx, max_slots=4, budget_bytes=4 << 30, opts=o)
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    try:
        tag = 0
        for step in range(3):
            tags = set()
            for inst in insts:
                srv.submit_step(inst, dt, tag)
                tags.add(tag)
                tag += 1
            done = drain(srv, tags)
            assert all(done[t]["result_name"] == "SUCCESS" for t in tags)
        for inst, (x, v) in zip(insts, ref):
            assert np.array_equal(inst.positions(), x) and np.array_equal(inst.velocities(), v)
    finally:
        srv.close()


def test_refusals_come_back_in_the_report(gpu_ctx):
    o = px.options(**SERVED)
    good = M.cantilever(2, 2, 4)
    bad = good.copy()
    bad.T[3, [1, 2]] = bad.T[3, [2, 1]]  # negative rest volume: rejected when its pattern is built
    big = M.cantilever(8, 8, 32)
    srv = px.Server(gpu_ctx, max_slots=4, budget_bytes=1 << 20, opts=o)
    try:
        i_bad = srv.submit_mesh(bad, 0)
        i_big = srv.submit_mesh(big, 1)
        i_good = srv.submit_mesh(good, 2)
        done = drain(srv, {0, 1, 2})
        assert done[0]["status"] == px.PHX_EINVAL and done[0]["result_name"] == "FAILURE"
        assert done[1]["status"] == px.PHX_ENOMEM and done[1]["result_name"] == "FAILURE"
        assert done[2]["status"] == px.PHX_OK and done[2]["result_name"] == "SUCCESS"
        _, x, _ = alone(gpu_ctx, good, o)
        assert np.array_equal(i_good.positions(), x)
    finally:
        srv.close()
    for i in (i_bad, i_big, i_good):
        i.close()
