"""The C-ABI library: it loads without a GPU and exports every entry point include/phx.h declares."""
import ctypes as C
import os
import re

import pytest

import physim_gb300 as px
from physim_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "phx.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(phx_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    path = build.build()
    L = C.CDLL(path)
    names = declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(px.EXPORTS) == names


def test_version_and_defaults_without_gpu():
    L = px.lib()
    assert L.phx_version() >= 10000
    o = px.options()
    # OptimSolverOptions defaults (include/PhySim/Solvers/OptimSolver.h:47-70)
    assert (o.qp_solver, o.tol_max_error, o.tol_min_step, o.min_step_max_count) == (1, 1e-6, 1e-5, 3)
    assert (o.tol_min_impr, o.min_impr_max_count, o.num_max_iters, o.try_steepest) == (1e-9, 3, 100, 1)
    assert (o.max_step_size, o.ls_num_max_iters, o.ls_tol_max_error, o.ls_num_reg_trials) == (1000, 1000, 1e-9, 10)
    assert (o.lsearch_type, o.lsearch_alpha, o.lsearch_num_try) == (1, 0.5, 32)
    assert (o.lsearch_wolfe1, o.lsearch_wolfe2) == (1e-4, 0.9)


def test_no_device_is_an_error_not_a_fallback():
    try:
        ctx = px.Context(0, arena_bytes=1 << 20)
    except px.PhxError as e:
        assert e.code == px.PHX_ECUDA or e.code == px.PHX_EINVAL
        return
    ctx.close()
    pytest.skip("a GPU is present")
