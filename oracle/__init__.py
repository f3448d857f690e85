"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates PhySim's CPU tet-FEM Newton path (see phx_oracle.cpp for
the reference file:line each part follows).  Only tests/, the smoke check and
the benchmark's CPU-baseline leg import this package; the product path never
does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None

OS_NAMES = {0: "ONGOING", 1: "SUCCESS", 2: "MINSTEP", 3: "MINIMPR", 4: "FAILURE", 5: "MAXITER", 6: "NONDESC"}


class OrcMesh(C.Structure):
    _fields_ = [("n", C.c_int32), ("m", C.c_int32), ("X0", C.c_void_p), ("T", C.c_void_p),
                ("lame", C.c_void_p), ("rho", C.c_void_p), ("model", C.c_void_p),
                ("fixed", C.c_void_p), ("force", C.c_void_p), ("gravity", C.c_double * 3),
                ("soft_k", C.c_void_p), ("soft_target", C.c_void_p)]


class OrcOptions(C.Structure):
    _fields_ = [("qp_solver", C.c_int32), ("tol_max_error", C.c_double), ("tol_min_step", C.c_double),
                ("min_step_max_count", C.c_int32), ("tol_min_impr", C.c_double),
                ("min_impr_max_count", C.c_int32), ("num_max_iters", C.c_int32),
                ("try_steepest", C.c_int32), ("max_step_size", C.c_double), ("ls_solver", C.c_int32),
                ("ls_num_max_iters", C.c_int32), ("ls_tol_max_error", C.c_double),
                ("ls_num_reg_trials", C.c_int32), ("lsearch_type", C.c_int32),
                ("lsearch_alpha", C.c_double), ("lsearch_num_try", C.c_int32),
                ("lsearch_wolfe1", C.c_double), ("lsearch_wolfe2", C.c_double),
                ("cg_block_jacobi", C.c_int32), ("threads", C.c_int32), ("cg_parallel", C.c_int32)]


class OrcStageGroup(C.Structure):
    _fields_ = [("num_stages", C.c_int32), ("soft", C.c_int32), ("k_start", C.c_double), ("k_end", C.c_double),
                ("move", C.c_double * 9), ("shift", C.c_double * 3), ("num_nodes", C.c_int32),
                ("nodes", C.c_void_p)]


def stage_groups(groups, struct=None):
    """ctypes array of stage groups from dicts (num_stages, soft, k_start, k_end, move, shift,
    nodes); returns the array and the node arrays it points into."""
    struct = struct or OrcStageGroup
    keep = []
    arr = (struct * max(1, len(groups)))()
    for g, d in zip(arr, groups):
        nodes = np.ascontiguousarray(d["nodes"], dtype=np.int32)
        keep.append(nodes)
        g.num_stages = int(d.get("num_stages", 1))
        g.soft = int(d.get("soft", 0))
        g.k_start = float(d.get("k_start", 1e9))
        g.k_end = float(d.get("k_end", 1e9))
        mv = np.asarray(d.get("move", np.zeros((3, 3))), dtype=np.float64).ravel()
        for k in range(9):
            g.move[k] = mv[k]
        sh = np.asarray(d.get("shift", np.zeros(3)), dtype=np.float64)
        for k in range(3):
            g.shift[k] = sh[k]
        g.num_nodes = len(nodes)
        g.nodes = nodes.ctypes.data
    return arr, keep


class OrcReport(C.Structure):
    _fields_ = [("result", C.c_int32), ("iterations", C.c_int32), ("bisections", C.c_int32),
                ("reg_trials", C.c_int32), ("lin_iterations", C.c_int64), ("obj", C.c_double),
                ("opt", C.c_double), ("opt0", C.c_double), ("seconds", C.c_double),
                ("t_cal_ene", C.c_double), ("t_cal_gra", C.c_double), ("t_cal_hes", C.c_double),
                ("t_ass_gra", C.c_double), ("t_ass_hes", C.c_double), ("t_opt_sol", C.c_double),
                ("t_opt_lis", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["result_name"] = OS_NAMES.get(self.result, str(self.result))
        return d


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcMesh), C.POINTER(vp)]
        L.orc_destroy.argtypes = [vp]
        L.orc_default_options.argtypes = [C.POINTER(OrcOptions)]
        L.orc_element_local.argtypes = [vp, vp, vp, vp, vp]
        L.orc_material.argtypes = [C.c_int, C.c_double, C.c_double, vp, vp, vp, vp]
        L.orc_energy.argtypes = [vp, vp, C.POINTER(C.c_double)]
        L.orc_gradient.argtypes = [vp, vp, vp, C.c_int]
        L.orc_hessian_nnz.argtypes = [vp]
        L.orc_hessian_nnz.restype = C.c_int64
        L.orc_hessian_pattern.argtypes = [vp, vp, vp]
        L.orc_hessian.argtypes = [vp, vp, vp, C.c_int]
        L.orc_scatter_map.argtypes = [vp, vp]
        L.orc_solve_static.argtypes = [vp, C.POINTER(OrcOptions), vp, C.POINTER(OrcReport)]
        L.orc_solve_dynamic.argtypes = [vp, C.POINTER(OrcOptions), C.c_double, vp, vp, C.POINTER(OrcReport)]
        L.orc_linear_solve.argtypes = [vp, C.POINTER(OrcOptions), vp, vp, vp, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int64)]
        L.orc_last_log.argtypes = [vp, vp, vp, vp, vp, C.c_int32]
        L.orc_set_staging.argtypes = [vp, C.c_int32, vp, C.c_int32, vp]
        L.orc_stage.argtypes = [vp]
        L.orc_set_soft.argtypes = [vp, vp, vp]
        L.orc_sample_grid.argtypes = [C.c_int32, C.c_int32, vp, vp, vp, vp, C.c_int32, vp, vp, vp,
                                      C.c_double, vp, vp]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own .mcg material code, when it could be built here (else None)."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            return None
        R = C.CDLL(path)
        for f in (R.ref_conh, R.ref_stvk):
            f.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _ref = R
    return _ref


def _p(a):
    return a.ctypes.data if a is not None else None


def default_options(**kw) -> OrcOptions:
    o = OrcOptions()
    lib().orc_default_options(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(k)
        setattr(o, k, v)
    return o


def material(model: int, lam: float, mu: float, Fv: np.ndarray):
    Fv = np.ascontiguousarray(Fv, dtype=np.float64)
    psi = np.zeros(1); P = np.zeros(9); D = np.zeros(81)
    lib().orc_material(int(model), float(lam), float(mu), _p(Fv), _p(psi), _p(P), _p(D))
    return psi[0], P, D.reshape(9, 9)


class Oracle:
    """One mesh instance in the CPU restatement."""

    def __init__(self, mesh):
        self.mesh = mesh
        self._keep = [np.ascontiguousarray(mesh.X0, dtype=np.float64).ravel(),
                      np.ascontiguousarray(mesh.T, dtype=np.int32).ravel(),
                      np.ascontiguousarray(mesh.lame, dtype=np.float64).ravel(),
                      np.ascontiguousarray(mesh.rho, dtype=np.float64).ravel(),
                      np.ascontiguousarray(mesh.model, dtype=np.uint8).ravel(),
                      np.ascontiguousarray(mesh.fixed, dtype=np.uint8).ravel(),
                      np.ascontiguousarray(mesh.force, dtype=np.float64).ravel()]
        d = OrcMesh()
        d.n = mesh.n; d.m = mesh.m
        d.X0, d.T, d.lame, d.rho, d.model, d.fixed, d.force = [a.ctypes.data for a in self._keep]
        for c in range(3):
            d.gravity[c] = float(mesh.gravity[c])
        if getattr(mesh, "soft_k", None) is not None:
            self._keep.append(np.ascontiguousarray(mesh.soft_k, dtype=np.float64).ravel())
            d.soft_k = self._keep[-1].ctypes.data
            if getattr(mesh, "soft_target", None) is not None:
                self._keep.append(np.ascontiguousarray(mesh.soft_target, dtype=np.float64).ravel())
                d.soft_target = self._keep[-1].ctypes.data
        self._desc = d
        h = C.c_void_p()
        if lib().orc_create(C.byref(d), C.byref(h)) != 0:
            raise ValueError("oracle rejected the mesh")
        self.h = h
        self.N = 3 * mesh.n

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_destroy(self.h)
            self.h = None

    def rest(self):
        return np.ascontiguousarray(self.mesh.X0, dtype=np.float64).ravel().copy()

    def element_local(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        m = self.mesh.m
        E = np.zeros(m); g = np.zeros((m, 12)); H = np.zeros((m, 12, 12))
        lib().orc_element_local(self.h, _p(x), _p(E), _p(g), _p(H))
        return E, g, H

    def energy(self, x) -> float:
        x = np.ascontiguousarray(x, dtype=np.float64)
        e = C.c_double()
        lib().orc_energy(self.h, _p(x), C.byref(e))
        return e.value

    def gradient(self, x, fix=True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        g = np.zeros(self.N)
        lib().orc_gradient(self.h, _p(x), _p(g), int(fix))
        return g

    def pattern(self):
        nnz = lib().orc_hessian_nnz(self.h)
        cp = np.zeros(self.N + 1, dtype=np.int32); ri = np.zeros(nnz, dtype=np.int32)
        lib().orc_hessian_pattern(self.h, _p(cp), _p(ri))
        return cp, ri

    def hessian(self, x, fix=True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.zeros(lib().orc_hessian_nnz(self.h))
        lib().orc_hessian(self.h, _p(x), _p(v), int(fix))
        return v

    def scatter_map(self):
        mp = np.zeros((self.mesh.m, 10), dtype=np.int32)
        lib().orc_scatter_map(self.h, _p(mp))
        return mp

    def solve_static(self, x=None, **opts):
        x = self.rest() if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        o = default_options(**opts)
        r = OrcReport()
        lib().orc_solve_static(self.h, C.byref(o), _p(x), C.byref(r))
        return x, r.as_dict()

    def solve_dynamic(self, x, v, dt, **opts):
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        v = np.ascontiguousarray(v, dtype=np.float64).copy()
        o = default_options(**opts)
        r = OrcReport()
        lib().orc_solve_dynamic(self.h, C.byref(o), float(dt), _p(x), _p(v), C.byref(r))
        return x, v, r.as_dict()

    def linear_solve(self, x, b, dx0=None, **opts):
        x = np.ascontiguousarray(x, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        dx = np.zeros(self.N) if dx0 is None else np.ascontiguousarray(dx0, dtype=np.float64).copy()
        o = default_options(**opts)
        res = C.c_int32(); it = C.c_int64()
        lib().orc_linear_solve(self.h, C.byref(o), _p(x), _p(b), _p(dx), C.byref(res), C.byref(it))
        return dx, res.value, it.value

    def set_staging(self, groups, num_stages=0, x_ini=None):
        """Staged boundary conditions (see orc_set_staging); the stage goes back to 0."""
        arr, keep = stage_groups(groups)
        xi = np.ascontiguousarray(self.rest() if x_ini is None else x_ini, dtype=np.float64)
        if lib().orc_set_staging(self.h, len(groups), arr, int(num_stages), _p(xi)) != 0:
            raise ValueError("oracle rejected the staging")
        del keep

    def stage(self) -> int:
        return int(lib().orc_stage(self.h))

    def set_soft(self, k, t):
        """Soft records of the nodes that have one: stiffness k[n], targets t[3n]."""
        k = np.ascontiguousarray(k, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        if lib().orc_set_soft(self.h, _p(k), _p(t)) != 0:
            raise ValueError("the mesh has no soft records")

    def last_log(self):
        n = lib().orc_last_log(self.h, None, None, None, None, 0)
        obj = np.zeros(n); opt = np.zeros(n); bis = np.zeros(n, dtype=np.int32); step = np.zeros(n)
        lib().orc_last_log(self.h, _p(obj), _p(opt), _p(bis), _p(step), n)
        return {"obj": obj, "opt": opt, "bis": bis, "step": step}


def sample_grid(X0, T, x, field, shape, origin, delta, fill=0.0, E=None):
    """Restatement of the device grid sampler (field_oracle.cpp): values and owning tets of a
    grid of `shape` cells, x fastest, as flat arrays."""
    X0 = np.ascontiguousarray(X0, dtype=np.float64).ravel()
    T = np.ascontiguousarray(T, dtype=np.int32).ravel()
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    E = None if E is None else np.ascontiguousarray(E, dtype=np.float64)
    sh = np.asarray(shape, dtype=np.int32)
    org = np.asarray(origin, dtype=np.float64)
    dl = np.asarray(delta, dtype=np.float64)
    count = int(np.prod(sh.astype(np.int64)))
    vals = np.empty(count, dtype=np.float64)
    own = np.empty(count, dtype=np.int32)
    rc = lib().orc_sample_grid(len(X0) // 3, len(T) // 4, _p(X0), _p(T), _p(x), _p(E), int(field), _p(sh),
                               _p(org), _p(dl), float(fill), _p(vals), _p(own))
    if rc != 0:
        raise ValueError("orc_sample_grid: bad field or missing energies")
    return vals, own
