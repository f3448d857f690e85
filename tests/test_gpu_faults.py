"""Failure paths on the GPU that fault, trap or hang nothing.

* A bounded device wait that runs out: the engine's grid barrier is made to wait for an
  arrival that never comes (phx_debug_unmet_barrier, a short cycle limit).  The solve must
  return PHX_ETIMEOUT naming the barrier, and the same context must then solve the same
  problem to the same bits as before.  The barrier touches global memory only.
* Admission refusal: a request larger than the server's memory budget is refused with
  PHX_ENOMEM at submission, and the server keeps serving the others.
"""
import numpy as np
import pytest

import physim_gb300 as px
from physim_gb300 import mesh as M

pytestmark = pytest.mark.gpu

LIMIT = 20_000_000  # SM cycles, about 10 ms


def _same(r1, r2):
    keys = ("result", "iterations", "bisections", "pcg_iterations", "obj", "opt")
    return all(r1[k] == r2[k] for k in keys)


@pytest.mark.parametrize("tag,prec", [(1, px.PREC_FP32_REFINE), (11, px.PREC_FP64)])
def test_engine_barrier_wait_runs_out(gpu_ctx, tag, prec):
    """Tag 1: the barrier after each round's bookkeeping; tag 11: the whole-GPU PCG group's
    barrier, which the FP64 path reaches (its PCG iterates on the whole GPU)."""
    m = M.cantilever(2, 2, 6)
    inst = px.Instance(gpu_ctx, m)
    o = px.options(precision=prec, tol_rel=1e-8, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)
    inst.reset()  # each solve from rest with no warm PCG guess, so the two solves are the same
    x_ref, r_ref = inst.solve_static(o)
    assert r_ref["result_name"] == "SUCCESS"
    inst.reset()
    gpu_ctx.debug_unmet_barrier(tag, LIMIT)
    try:
        with pytest.raises(px.PhxError) as ei:
            inst.solve_static(o)
    finally:
        gpu_ctx.debug_unmet_barrier(0)
    assert ei.value.code == px.PHX_ETIMEOUT
    # tag 11 holds the whole-GPU PCG group; CTAs outside it wait at the round barrier 18,
    # and whichever wait gives up first is named
    names = {f"stage {tag})"} | ({"stage 18)"} if tag == 11 else set())
    assert any(nm in str(ei.value) for nm in names), str(ei.value)
    # the context is still usable: the same solve gives the same bits
    inst.reset()
    x2, r2 = inst.solve_static(o)
    assert np.array_equal(x2, x_ref) and _same(r2, r_ref)


def test_unmet_barrier_hook_rejects_bad_arguments(gpu_ctx):
    for tag, limit in ((23, LIMIT), (-1, LIMIT), (1, 10), (1, 10**10)):
        with pytest.raises(px.PhxError) as ei:
            gpu_ctx.debug_unmet_barrier(tag, limit)
        assert ei.value.code == px.PHX_EINVAL
    gpu_ctx.debug_unmet_barrier(0)


def test_admission_refuses_a_request_above_the_budget(gpu_ctx):
    small = M.cantilever(2, 2, 4)   # 96 tets: well under 1 MB on the device
    big = M.cantilever(8, 8, 32)    # 12,288 tets: its FP64 rest records alone take 1.2 MB
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    i_small, i_big = px.Instance(gpu_ctx, small), px.Instance(gpu_ctx, big)
    x_alone, _ = i_small.solve_static(o, small.X0.ravel())
    i_small.reset()
    # a budget between the two instances' device footprints
    srv = px.Server(gpu_ctx, max_slots=4, budget_bytes=1 << 20, opts=o)
    try:
        with pytest.raises(px.PhxError) as ei:
            srv.submit(i_big, 1)
        assert ei.value.code == px.PHX_ENOMEM
        srv.submit(i_small, 2)
        done = {}
        for _ in range(10000):
            srv.progress()
            done.update(dict(srv.poll()))
            if 2 in done:
                break
        assert done[2]["result_name"] == "SUCCESS"
        assert np.array_equal(i_small.positions(), x_alone)
        # a caller's instance counts against the budget only while it is active
        st = srv.stats()
        assert st["in_use"] == 0 and 0 < st["peak"] <= 1 << 20
    finally:
        srv.close()
