"""The graph-driven solve loop and the batch tuner on the GPU.

* A batch solved through CUDA-graph launches (k_prep, engine, cluster PCG kernels and the
  loop test in a device while-loop) gives the bits of the host-driven loop, on the served
  path (cluster PCG) and on the plain FP64 path (whole-GPU PCG).
* Launch settings change no result: other wait, round and time-slice settings give the same bits.
* The tuner leaves the instances as it found them, caches its choice for the batch's mix, and
  a batch solved after tuning gives the bits of one solved before.
"""
import numpy as np
import pytest

import physim_gb300 as px
from physim_gb300 import mesh as M

pytestmark = pytest.mark.gpu

KEYS = ("result", "iterations", "bisections", "pcg_iterations", "obj", "opt", "refine_sweeps")


def _solve(ctx, meshes, o):
    insts = [px.Instance(ctx, m) for m in meshes]
    reps, xs = ctx.batch_solve(insts, o, [m.X0.ravel().copy() for m in meshes])
    return reps, xs


def _same(a, b):
    (ra, xa), (rb, xb) = a, b
    for r1, r2, x1, x2 in zip(ra, rb, xa, xb):
        assert np.array_equal(x1, x2)
        assert all(r1[k] == r2[k] for k in KEYS), (r1, r2)


@pytest.fixture
def defaults(gpu_ctx):
    d = gpu_ctx.launch_settings()
    yield d
    gpu_ctx.launch_settings(**d)


@pytest.mark.parametrize("prec", [px.PREC_FP32_REFINE, px.PREC_FP64])
def test_graph_loop_equals_host_loop(gpu_ctx, defaults, prec):
    meshes = [M.batch_instance(3, i) for i in range(30, 38)]
    o = px.options(precision=prec, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)
    gpu_ctx.launch_settings(graph=0)
    host = _solve(gpu_ctx, meshes, o)
    gpu_ctx.launch_settings(graph=1)
    n0 = gpu_ctx.kernel_launches()
    graph = _solve(gpu_ctx, meshes, o)
    assert gpu_ctx.kernel_launches() > n0  # the graph's kernels are counted as launches
    _same(host, graph)
    assert all(r["result_name"] == "SUCCESS" for r in graph[0])


def test_launch_settings_change_no_result(gpu_ctx, defaults):
    meshes = [M.batch_instance(3, i) for i in range(40, 60)]  # more solves than clusters: time slices
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    ref = _solve(gpu_ctx, meshes, o)
    for s in ({"wait_rounds": 1, "wait_share": 1, "rounds": 3}, {"wait_rounds": 16, "wait_share": 8, "rounds": 64},
              {"graph": 0, "rounds": 1}, {"slice_share": 0}, {"wait_share": 1, "slice_share": 64, "slice_min": 1},
              {"graph": 0, "wait_share": 1, "slice_share": 16, "slice_min": 8}):
        gpu_ctx.launch_settings(**{**defaults, **s})
        _same(ref, _solve(gpu_ctx, meshes, o))


def test_launch_settings_are_checked(gpu_ctx, defaults):
    for bad in ({"graph": 2}, {"wait_rounds": 0}, {"wait_share": 65}, {"rounds": 0}, {"pcg_grid": 2},
                {"slice_share": -1}, {"slice_share": 65}, {"slice_min": 0}):
        with pytest.raises(px.PhxError) as ei:
            gpu_ctx.launch_settings(**bad)
        assert ei.value.code == px.PHX_EINVAL
    assert gpu_ctx.launch_settings() == defaults


def test_tuner_leaves_instances_and_results_unchanged(gpu_ctx, defaults):
    meshes = [M.batch_instance(3, i) for i in range(50, 58)]
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    ref = _solve(gpu_ctx, meshes, o)
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    start = [m.X0.ravel() + 1e-4 * np.sin(np.arange(3 * m.n)) for m in meshes]
    for i, x in zip(insts, start):
        i.set_positions(x)
    t = gpu_ctx.tune_batch(insts, o)
    assert t["trials"] >= 3 and t["best_seconds"] <= t["default_seconds"]
    assert set(t["chosen"]) == {"graph", "wait_rounds", "wait_share", "rounds", "pcg_grid", "slice_share", "slice_min"}
    for i, x in zip(insts, start):
        assert np.array_equal(i.positions(), x)
    # the tuned settings serve this mix now; results are those of the default settings
    reps, xs = gpu_ctx.batch_solve(insts, o, [m.X0.ravel().copy() for m in meshes])
    _same(ref, (reps, xs))
    assert gpu_ctx.launch_settings() == defaults  # the defaults themselves are not changed


def test_whole_gpu_pcg_kernels_give_the_engine_bits(gpu_ctx, defaults):
    """An FP32 instance above the cluster size (15,379 nodes) iterates its PCG in k_gpcg_a/b
    (launch setting pcg_grid 1) or inside the engine (pcg_grid 0, the default): the same tiles,
    partial sums and decisions, so the same bits; alone and beside cluster instances, on the
    graph and on the host loop."""
    big = M.cantilever(12, 12, 90)
    assert big.n > 13000
    small = [M.batch_instance(3, i) for i in range(60, 63)]
    kw = dict(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)
    gpu_ctx.launch_settings(pcg_grid=0)
    ref = _solve(gpu_ctx, [big], px.options(**kw))
    assert ref[0][0]["result_name"] == "SUCCESS"
    gpu_ctx.launch_settings(pcg_grid=1)
    for graph in (1, 0):
        gpu_ctx.launch_settings(graph=graph)
        _same(ref, _solve(gpu_ctx, [big], px.options(**kw)))
        mixed = _solve(gpu_ctx, small + [big], px.options(**kw))
        _same(ref, ([mixed[0][-1]], [mixed[1][-1]]))
    # profiling (host loop, events around each kernel): the kernels' time and bytes are recorded
    gpu_ctx.profile(True)
    gpu_ctx.profile_reset()
    _same(ref, _solve(gpu_ctx, [big], px.options(**kw)))
    n, ms = gpu_ctx.profile_read("spmv")
    nbytes = gpu_ctx.profile_bytes("spmv")
    gpu_ctx.profile(False)
    assert n > 0 and ms > 0 and nbytes > 0


def test_tuner_puts_instances_back_when_a_trial_fails(gpu_ctx, defaults):
    """A trial that gives up (the engine's round barrier made to wait for an arrival that never
    comes, a short limit) ends the tuning with PHX_ETIMEOUT, the instances back where they
    were, and nothing cached for the mix."""
    meshes = [M.batch_instance(3, i) for i in range(64, 67)]
    o = px.options(precision=px.PREC_FP32_REFINE, tol_rel=1e-6, tol_max_error=0.0, tol_min_impr=0.0,
                   tol_min_step=0.0)
    insts = [px.Instance(gpu_ctx, m) for m in meshes]
    start = [m.X0.ravel() + 1e-4 * np.cos(np.arange(3 * m.n)) for m in meshes]
    for i, x in zip(insts, start):
        i.set_positions(x)
    gpu_ctx.debug_unmet_barrier(1, 20_000_000)
    try:
        with pytest.raises(px.PhxError) as ei:
            gpu_ctx.tune_batch(insts, o)
    finally:
        gpu_ctx.debug_unmet_barrier(0)
    assert ei.value.code == px.PHX_ETIMEOUT
    for i, x in zip(insts, start):
        assert np.array_equal(i.positions(), x)
    # the context still solves the batch (no tuned settings were kept for it)
    reps, _ = gpu_ctx.batch_solve(insts, o, [x.copy() for x in start])
    assert all(r["status"] == px.PHX_OK for r in reps)
