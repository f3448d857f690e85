"""physim_gb300 -- GB300-native tet-FEM Newton path behind PhySim's solver interface.

The compute path is libphx.so (hand-written sm_103a CUDA + a C ABI, see
include/phx.h).  This module is a thin ctypes binding over that ABI; it has
no compute of its own and no fallback: if libphx.so cannot be loaded, every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

import numpy as np

from . import mesh  # noqa: F401  (re-exported)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libphx.so")

PREC_FP64 = 0
PREC_FP32_REFINE = 1
OS_NAMES = {0: "ONGOING", 1: "SUCCESS", 2: "MINSTEP", 3: "MINIMPR", 4: "FAILURE", 5: "MAXITER", 6: "NONDESC"}

PHX_OK, PHX_EINVAL, PHX_ENOMEM, PHX_ETIMEOUT, PHX_ECUDA, PHX_EBUSY, PHX_ENOTFOUND = 0, -1, -2, -3, -4, -5, -6

# every entry point include/phx.h declares
EXPORTS = [
    "phx_version", "phx_last_error", "phx_default_options", "phx_context_create", "phx_context_destroy",
    "phx_context_memory", "phx_instance_create", "phx_instances_create", "phx_instance_destroy", "phx_instance_sizes",
    "phx_instance_reset", "phx_instance_set_positions", "phx_instance_get_positions", "phx_instance_set_velocities",
    "phx_instance_get_velocities", "phx_instance_update_load", "phx_instance_set_staging", "phx_instance_stage", "phx_energy_gradient", "phx_hessian",
    "phx_hessian_pattern", "phx_scatter_map", "phx_element_local", "phx_solve_static", "phx_solve_step", "phx_solve_log",
    "phx_dynamic_step", "phx_batch_solve", "phx_batch_dynamic_step", "phx_server_create", "phx_server_destroy",
    "phx_server_submit", "phx_server_submit_step", "phx_server_submit_mesh", "phx_server_stats",
    "phx_server_progress", "phx_server_poll", "phx_profile_enable", "phx_profile_read",
    "phx_profile_reset", "phx_profile_bytes", "phx_kernel_launches", "phx_timer_mark", "phx_timer_elapsed",
    "phx_hessian_blocks_noalloc", "phx_debug_unmet_barrier", "phx_context_launch_settings", "phx_tune_batch",
    "phx_scene_load", "phx_scene_destroy", "phx_scene_info", "phx_scene_mesh", "phx_scene_options",
    "phx_scene_staging", "phx_scene_instance", "phx_svl_write", "phx_svl_read_header", "phx_svl_read",
    "phx_instance_sample_grid",
]


class PhxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"phx error {code}: {msg}")
        self.code = code


class Mesh_(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_tets", C.c_int32), ("X0", C.c_void_p), ("tets", C.c_void_p),
                ("lame", C.c_void_p), ("rho", C.c_void_p), ("model", C.c_void_p), ("fixed", C.c_void_p),
                ("force", C.c_void_p), ("gravity", C.c_double * 3), ("soft_k", C.c_void_p),
                ("soft_target", C.c_void_p)]


class LaunchSettings_(C.Structure):
    """phx_launch_settings: scheduling of a context's batch solves (changes no result)."""
    _fields_ = [("graph", C.c_int32), ("wait_rounds", C.c_int32), ("wait_share", C.c_int32), ("rounds", C.c_int32),
                ("pcg_grid", C.c_int32), ("slice_share", C.c_int32), ("slice_min", C.c_int32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class Options(C.Structure):
    """phx_options: OptimSolverOptions (include/PhySim/Solvers/OptimSolver.h:47-70) + GPU settings."""
    _fields_ = [("qp_solver", C.c_int32), ("tol_max_error", C.c_double), ("tol_min_step", C.c_double),
                ("min_step_max_count", C.c_int32), ("tol_min_impr", C.c_double),
                ("min_impr_max_count", C.c_int32), ("num_max_iters", C.c_int32), ("try_steepest", C.c_int32),
                ("max_step_size", C.c_double), ("ls_solver", C.c_int32), ("ls_num_max_iters", C.c_int32),
                ("ls_tol_max_error", C.c_double), ("ls_num_reg_trials", C.c_int32), ("lsearch_type", C.c_int32),
                ("lsearch_alpha", C.c_double), ("lsearch_num_try", C.c_int32),
                ("lsearch_wolfe1", C.c_double), ("lsearch_wolfe2", C.c_double), ("precision", C.c_int32),
                ("precond", C.c_int32), ("inner_tol", C.c_double), ("max_refine_sweeps", C.c_int32),
                ("warm_guess", C.c_int32), ("pcg_chunk", C.c_int32), ("tol_rel", C.c_double),
                ("pcg_cluster", C.c_int32), ("fp64_finish", C.c_int32),
                ("lsearch_parallel", C.c_int32), ("negative_curvature", C.c_int32)]


class StageGroup_(C.Structure):
    """phx_stage_group: one BC_FixDoF group loaded over stages with animated targets."""
    _fields_ = [("num_stages", C.c_int32), ("soft", C.c_int32), ("k_start", C.c_double), ("k_end", C.c_double),
                ("move", C.c_double * 9), ("shift", C.c_double * 3), ("num_nodes", C.c_int32),
                ("nodes", C.c_void_p)]


class Grid_(C.Structure):
    """phx_grid: a ScalarField_Grid's shape, origin and cell size."""
    _fields_ = [("shape", C.c_int32 * 3), ("origin", C.c_double * 3), ("delta", C.c_double * 3)]


# SVL value types (Serializer_Field.cpp's "char", "short", "int", "float", "double") and numpy's
SVL_DTYPES = {0: np.int8, 1: np.int16, 2: np.int32, 3: np.float32, 4: np.float64}
FIELD_DISPLACEMENT_X, FIELD_DISPLACEMENT_Y, FIELD_DISPLACEMENT_Z = 0, 1, 2
FIELD_DISPLACEMENT_NORM, FIELD_VOLUME_RATIO, FIELD_ENERGY_DENSITY = 3, 4, 5


class Report(C.Structure):
    _fields_ = [("result", C.c_int32), ("iterations", C.c_int32), ("bisections", C.c_int32),
                ("reg_trials", C.c_int32), ("pcg_iterations", C.c_int64), ("refine_sweeps", C.c_int32),
                ("status", C.c_int32), ("obj", C.c_double), ("opt", C.c_double), ("opt0", C.c_double),
                ("seconds", C.c_double), ("hessian_evals", C.c_int32), ("fp64_iterations", C.c_int32),
                ("pcg_slices", C.c_int32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["result_name"] = OS_NAMES.get(self.result, str(self.result))
        return d


_lib = None


def lib():
    """Loads libphx.so; raises if the CUDA path is not built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA path first (physim_gb300.build.build())")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "phx_version": ([], C.c_int),
        "phx_last_error": ([], C.c_char_p),
        "phx_default_options": ([C.POINTER(Options)], None),
        "phx_context_create": ([i32, i64, C.POINTER(vp)], C.c_int),
        "phx_context_destroy": ([vp], C.c_int),
        "phx_context_memory": ([vp, C.POINTER(i64), C.POINTER(i64)], C.c_int),
        "phx_instance_create": ([vp, C.POINTER(Mesh_), C.POINTER(vp)], C.c_int),
        "phx_instances_create": ([vp, C.c_int32, C.POINTER(Mesh_), C.POINTER(vp)], C.c_int),
        "phx_instance_destroy": ([vp], C.c_int),
        "phx_instance_sizes": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)], C.c_int),
        "phx_instance_reset": ([vp], C.c_int),
        "phx_instance_set_positions": ([vp, vp], C.c_int),
        "phx_instance_get_positions": ([vp, vp], C.c_int),
        "phx_instance_set_velocities": ([vp, vp], C.c_int),
        "phx_instance_get_velocities": ([vp, vp], C.c_int),
        "phx_instance_update_load": ([vp, vp, vp], C.c_int),
        "phx_instance_set_staging": ([vp, i32, vp, i32], C.c_int),
        "phx_instance_stage": ([vp, C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "phx_energy_gradient": ([vp, vp, C.POINTER(dbl), vp, i32], C.c_int),
        "phx_hessian": ([vp, vp, i32, vp, i32], C.c_int),
        "phx_hessian_pattern": ([vp, vp, vp], C.c_int),
        "phx_scatter_map": ([vp, vp], C.c_int),
        "phx_element_local": ([vp, vp, i32, vp, vp, vp], C.c_int),
        "phx_solve_static": ([vp, C.POINTER(Options), vp, C.POINTER(Report)], C.c_int),
        "phx_solve_step": ([vp, C.POINTER(Options), vp, C.POINTER(Report)], C.c_int),
        "phx_solve_log": ([vp, vp, vp, vp, vp, i32], C.c_int),
        "phx_dynamic_step": ([vp, C.POINTER(Options), dbl, vp, vp, C.POINTER(Report)], C.c_int),
        "phx_batch_solve": ([vp, i32, vp, C.POINTER(Options), vp, vp], C.c_int),
        "phx_batch_dynamic_step": ([vp, i32, vp, C.POINTER(Options), dbl, vp], C.c_int),
        "phx_server_create": ([vp, i32, i64, C.POINTER(Options), C.POINTER(vp)], C.c_int),
        "phx_server_destroy": ([vp], C.c_int),
        "phx_server_submit": ([vp, vp, i64], C.c_int),
        "phx_server_submit_step": ([vp, vp, dbl, i64], C.c_int),
        "phx_server_submit_mesh": ([vp, C.POINTER(Mesh_), i64, C.POINTER(vp)], C.c_int),
        "phx_server_stats": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)], C.c_int),
        "phx_server_progress": ([vp, C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "phx_server_poll": ([vp, vp, vp, i32], C.c_int),
        "phx_profile_enable": ([vp, i32], C.c_int),
        "phx_profile_read": ([vp, C.c_char_p, C.POINTER(i64), C.POINTER(dbl)], C.c_int),
        "phx_profile_bytes": ([vp, C.c_char_p, C.POINTER(dbl)], C.c_int),
        "phx_profile_reset": ([vp], C.c_int),
        "phx_kernel_launches": ([vp], i64),
        "phx_timer_mark": ([vp, i32], C.c_int),
        "phx_timer_elapsed": ([vp, i32, i32, C.POINTER(dbl)], C.c_int),
        "phx_hessian_blocks_noalloc": ([i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp], C.c_int),
        "phx_debug_unmet_barrier": ([vp, i32, i64], C.c_int),
        "phx_context_launch_settings": ([vp, C.POINTER(LaunchSettings_), C.POINTER(LaunchSettings_)], C.c_int),
        "phx_tune_batch": ([vp, i32, vp, C.POINTER(Options), C.POINTER(LaunchSettings_), C.POINTER(dbl),
                            C.POINTER(dbl), C.POINTER(i32)], C.c_int),
        "phx_scene_load": ([C.c_char_p, C.POINTER(vp)], C.c_int),
        "phx_scene_destroy": ([vp], C.c_int),
        "phx_scene_info": ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(dbl), C.POINTER(i32),
                            C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "phx_scene_mesh": ([vp, C.POINTER(Mesh_), vp], C.c_int),
        "phx_scene_options": ([vp, C.POINTER(Options)], C.c_int),
        "phx_scene_staging": ([vp, vp, i32], C.c_int),
        "phx_scene_instance": ([vp, vp, C.POINTER(vp)], C.c_int),
        "phx_svl_write": ([C.c_char_p, C.POINTER(Grid_), i32, vp], C.c_int),
        "phx_svl_read_header": ([C.c_char_p, C.POINTER(Grid_), C.POINTER(i32)], C.c_int),
        "phx_svl_read": ([C.c_char_p, i32, vp, i64], C.c_int),
        "phx_instance_sample_grid": ([vp, vp, i32, C.POINTER(Grid_), dbl, vp, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int):
    if rc != PHX_OK:
        raise PhxError(rc, lib().phx_last_error().decode(errors="replace"))


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def options(**kw) -> Options:
    o = Options()
    lib().phx_default_options(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


def _grid(shape, origin, delta) -> Grid_:
    g = Grid_()
    for d in range(3):
        g.shape[d] = int(shape[d])
        g.origin[d] = float(origin[d])
        g.delta[d] = float(delta[d])
    return g


def write_svl(path: str, values: np.ndarray, origin=(0.0, 0.0, 0.0), delta=(1.0, 1.0, 1.0)):
    """Writes a 3-D array values[i, j, k] as an SVL grid (Serializer_Field::WriteGrid_SVL); the
    array's dtype picks the value type (int8, int16, int32, float32 or float64)."""
    values = np.asarray(values)
    if values.ndim != 3:
        raise ValueError("values must be a 3-D array indexed [i, j, k]")
    fmt = {np.dtype(t): f for f, t in SVL_DTYPES.items()}.get(values.dtype)
    if fmt is None:
        raise ValueError(f"SVL holds int8, int16, int32, float32 or float64 values, not {values.dtype}")
    flat = np.ascontiguousarray(values.ravel(order="F"))
    _check(lib().phx_svl_write(os.fsencode(path), C.byref(_grid(values.shape, origin, delta)), fmt, _p(flat)))


def read_svl_header(path: str):
    """(shape, origin, delta, value type) of an SVL grid file."""
    g = Grid_(); f = C.c_int32()
    _check(lib().phx_svl_read_header(os.fsencode(path), C.byref(g), C.byref(f)))
    return tuple(g.shape), tuple(g.origin), tuple(g.delta), int(f.value)


def read_svl(path: str, dtype=None):
    """Reads an SVL grid (Serializer_Field::ReadGrid_SVL) as values[i, j, k], origin, delta;
    dtype (one of the five SVL types) converts the values as the reference does, None keeps the
    file's type."""
    shape, origin, delta, fmt = read_svl_header(path)
    if dtype is not None:
        fmt = {np.dtype(t): f for f, t in SVL_DTYPES.items()}.get(np.dtype(dtype))
        if fmt is None:
            raise ValueError(f"SVL holds int8, int16, int32, float32 or float64 values, not {dtype}")
    flat = np.empty(int(np.prod(shape, dtype=np.int64)), dtype=SVL_DTYPES[fmt])
    _check(lib().phx_svl_read(os.fsencode(path), fmt, _p(flat), flat.size))
    return flat.reshape(shape, order="F"), origin, delta


class Context:
    """One GPU, one stream, one device-memory arena."""

    def __init__(self, device: int = 0, arena_bytes: int = 0):
        h = C.c_void_p()
        _check(lib().phx_context_create(int(device), int(arena_bytes), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().phx_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def memory(self):
        u = C.c_int64(); c = C.c_int64()
        _check(lib().phx_context_memory(self.h, C.byref(u), C.byref(c)))
        return u.value, c.value

    def create_instances(self, meshes):
        """Instances of many meshes at once (phx_instances_create: host parts in parallel)."""
        meshes = list(meshes)
        if not meshes:
            return []
        descs, keeps = zip(*(_mesh_desc(m) for m in meshes))
        arr = (Mesh_ * len(meshes))(*descs)
        hs = (C.c_void_p * len(meshes))()
        _check(lib().phx_instances_create(self.h, len(meshes), arr, hs))
        del keeps
        return [Instance(self, m, _handle=C.c_void_p(h)) for m, h in zip(meshes, hs)]

    def mark(self, slot: int):
        """Records CUDA event `slot` on the library's stream."""
        _check(lib().phx_timer_mark(self.h, int(slot)))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_double()
        _check(lib().phx_timer_elapsed(self.h, int(a), int(b), C.byref(ms)))
        return ms.value

    def debug_unmet_barrier(self, tag: int, limit_cycles: int = 0):
        """Test hook: engine grid barrier `tag` waits for an arrival that never comes and gives
        up after limit_cycles (tag 0: off)."""
        _check(lib().phx_debug_unmet_barrier(self.h, int(tag), int(limit_cycles)))

    def launch_settings(self, **changes) -> dict:
        """The context's default launch settings (graph, wait_rounds, wait_share, rounds, pcg_grid); keyword
        arguments change them.  Returns the settings in force after the call."""
        cur = LaunchSettings_()
        _check(lib().phx_context_launch_settings(self.h, C.byref(cur), None))
        if changes:
            for k, v in changes.items():
                if k not in cur.as_dict():
                    raise KeyError(k)
                setattr(cur, k, int(v))
            _check(lib().phx_context_launch_settings(self.h, None, C.byref(cur)))
        return cur.as_dict()

    def tune_batch(self, insts: Sequence["Instance"], opts: "Options") -> dict:
        """Tunes the launch settings for this batch (cached under its mix key); the instances are
        left as they were.  Returns the chosen settings, the default and best batch times."""
        n = len(insts)
        arr = (C.c_void_p * n)(*[i.h.value for i in insts])
        ch, td, tb, nt = LaunchSettings_(), C.c_double(), C.c_double(), C.c_int32()
        _check(lib().phx_tune_batch(self.h, n, arr, C.byref(opts), C.byref(ch), C.byref(td), C.byref(tb), C.byref(nt)))
        return {"chosen": ch.as_dict(), "default_seconds": td.value, "best_seconds": tb.value, "trials": nt.value}

    def kernel_launches(self) -> int:
        return int(lib().phx_kernel_launches(self.h))

    def profile(self, on: bool = True):
        _check(lib().phx_profile_enable(self.h, int(on)))

    def profile_reset(self):
        _check(lib().phx_profile_reset(self.h))

    def profile_bytes(self, kind: str) -> float:
        b = C.c_double()
        _check(lib().phx_profile_bytes(self.h, kind.encode(), C.byref(b)))
        return b.value

    def profile_read(self, kind: str):
        n = C.c_int64(); ms = C.c_double()
        _check(lib().phx_profile_read(self.h, kind.encode(), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def batch_solve(self, insts: Sequence["Instance"], opts: Options, xs: Optional[List[np.ndarray]] = None,
                    inplace: bool = False):
        """Solves the instances together.  xs: starting positions, returned solved (copies,
        or with inplace=True the caller's float64 contiguous arrays themselves, e.g. pinned)."""
        n = len(insts)
        arr = (C.c_void_p * n)(*[i.h.value for i in insts])
        reps = (Report * n)()
        if xs is not None:
            if inplace:
                for x in xs:
                    if x.dtype != np.float64 or not x.flags.c_contiguous:
                        raise ValueError("inplace positions must be float64 and contiguous")
                xs = [x.reshape(-1) for x in xs]
            else:
                xs = [np.array(x, dtype=np.float64, copy=True).ravel() for x in xs]
            xp = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        else:
            xp = None
        _check(lib().phx_batch_solve(self.h, n, arr, C.byref(opts), xp, reps))
        return [r.as_dict() for r in reps], xs

    def batch_dynamic_step(self, insts: Sequence["Instance"], opts: Options, dt: float):
        n = len(insts)
        arr = (C.c_void_p * n)(*[i.h.value for i in insts])
        reps = (Report * n)()
        _check(lib().phx_batch_dynamic_step(self.h, n, arr, C.byref(opts), float(dt), reps))
        return [r.as_dict() for r in reps]


def _mesh_desc(m):
    """phx_mesh of a mesh, and the arrays it points into (keep them alive for the call)."""
    keep = [np.ascontiguousarray(m.X0, dtype=np.float64).ravel(),
            np.ascontiguousarray(m.T, dtype=np.int32).ravel(),
            np.ascontiguousarray(m.lame, dtype=np.float64).ravel(),
            np.ascontiguousarray(m.rho, dtype=np.float64).ravel(),
            np.ascontiguousarray(m.model, dtype=np.uint8).ravel(),
            np.ascontiguousarray(m.fixed, dtype=np.uint8).ravel(),
            np.ascontiguousarray(m.force, dtype=np.float64).ravel()]
    d = Mesh_()
    d.num_nodes = m.n
    d.num_tets = m.m
    d.X0, d.tets, d.lame, d.rho, d.model, d.fixed, d.force = [a.ctypes.data for a in keep]
    for c in range(3):
        d.gravity[c] = float(m.gravity[c])
    if getattr(m, "soft_k", None) is not None:
        keep.append(np.ascontiguousarray(m.soft_k, dtype=np.float64).ravel())
        d.soft_k = keep[-1].ctypes.data
        if getattr(m, "soft_target", None) is not None:
            keep.append(np.ascontiguousarray(m.soft_target, dtype=np.float64).ravel())
            d.soft_target = keep[-1].ctypes.data
    return d, keep


class Instance:
    """One FEM volume on the device (Simulable_FEM + boundary conditions)."""

    def __init__(self, ctx: Context, m, _handle=None):
        self.ctx = ctx
        self.mesh = m
        if _handle is None:
            d, keep = _mesh_desc(m)
            h = C.c_void_p()
            _check(lib().phx_instance_create(ctx.h, C.byref(d), C.byref(h)))
            _handle = h
        self.h = _handle
        self.N = 3 * m.n

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            lib().phx_instance_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sizes(self):
        a, b, c, d = (C.c_int64() for _ in range(4))
        _check(lib().phx_instance_sizes(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"ndof": a.value, "nnz": b.value, "lower_blocks": c.value, "full_blocks": d.value}

    def reset(self):
        """Positions back to rest, velocities and the warm-start step to zero (device-side copies)."""
        _check(lib().phx_instance_reset(self.h))

    def set_positions(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check(lib().phx_instance_set_positions(self.h, _p(x)))

    def positions(self):
        x = np.zeros(self.N)
        _check(lib().phx_instance_get_positions(self.h, _p(x)))
        return x

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        _check(lib().phx_instance_set_velocities(self.h, _p(v)))

    def velocities(self):
        v = np.zeros(self.N)
        _check(lib().phx_instance_get_velocities(self.h, _p(v)))
        return v

    def update_load(self, force=None, gravity=None):
        f = None if force is None else np.ascontiguousarray(force, dtype=np.float64)
        g = None if gravity is None else np.ascontiguousarray(gravity, dtype=np.float64)
        _check(lib().phx_instance_update_load(self.h, _p(f), _p(g)))

    def set_staging(self, groups, num_stages=0):
        """Staged boundary conditions: groups are dicts (num_stages, soft, k_start, k_end, move,
        shift, nodes); their targets start from the current positions.  The stage goes to 0."""
        keep = []
        arr = (StageGroup_ * max(1, len(groups)))()
        for g, d in zip(arr, groups):
            nodes = np.ascontiguousarray(d["nodes"], dtype=np.int32)
            keep.append(nodes)
            g.num_stages = int(d.get("num_stages", 1))
            g.soft = int(d.get("soft", 0))
            g.k_start = float(d.get("k_start", 1e9))
            g.k_end = float(d.get("k_end", 1e9))
            mv = np.asarray(d.get("move", np.zeros((3, 3))), dtype=np.float64).ravel()
            sh = np.asarray(d.get("shift", np.zeros(3)), dtype=np.float64)
            for k in range(9):
                g.move[k] = mv[k]
            for k in range(3):
                g.shift[k] = sh[k]
            g.num_nodes = len(nodes)
            g.nodes = nodes.ctypes.data
        _check(lib().phx_instance_set_staging(self.h, len(groups), arr, int(num_stages)))
        del keep

    def stage(self):
        a = C.c_int32(); b = C.c_int32()
        _check(lib().phx_instance_stage(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def energy_gradient(self, x=None, fix=True):
        xx = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        e = C.c_double()
        g = np.zeros(self.N)
        _check(lib().phx_energy_gradient(self.h, _p(xx), C.byref(e), _p(g), int(fix)))
        return e.value, g

    def hessian(self, x=None, precision=PREC_FP64, fix=True):
        xx = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        v = np.zeros(self.sizes()["nnz"])
        _check(lib().phx_hessian(self.h, _p(xx), int(precision), _p(v), int(fix)))
        return v

    def pattern(self):
        s = self.sizes()
        cp = np.zeros(self.N + 1, dtype=np.int32)
        ri = np.zeros(s["nnz"], dtype=np.int32)
        _check(lib().phx_hessian_pattern(self.h, _p(cp), _p(ri)))
        return cp, ri

    def scatter_map(self):
        mp = np.zeros((self.mesh.m, 10), dtype=np.int32)
        _check(lib().phx_scatter_map(self.h, _p(mp)))
        return mp

    def element_local(self, x=None, precision=PREC_FP64):
        xx = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        m = self.mesh.m
        E = np.zeros(m); g = np.zeros((m, 12)); H = np.zeros((m, 12, 12))
        _check(lib().phx_element_local(self.h, _p(xx), int(precision), _p(E), _p(g), _p(H)))
        return E, g, H

    def sample_grid(self, field: int, shape, origin, delta, x=None, fill: float = 0.0):
        """A field of the solve on the cell centres of a grid over the rest shape
        (phx_instance_sample_grid): values[i, j, k] and the owning tet of each (-1: outside)."""
        xx = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        count = int(np.prod(np.asarray(shape, dtype=np.int64)))
        vals = np.empty(count, dtype=np.float64)
        own = np.empty(count, dtype=np.int32)
        _check(lib().phx_instance_sample_grid(self.h, _p(xx), int(field), C.byref(_grid(shape, origin, delta)),
                                              float(fill), _p(vals), _p(own)))
        return vals.reshape(tuple(shape), order="F"), own.reshape(tuple(shape), order="F")

    def solve_static(self, opts: Options, x=None):
        xx = None if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        r = Report()
        _check(lib().phx_solve_static(self.h, C.byref(opts), _p(xx), C.byref(r)))
        return (self.positions() if xx is None else xx), r.as_dict()

    def solve_step(self, opts: Options, x=None):
        xx = None if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        r = Report()
        _check(lib().phx_solve_step(self.h, C.byref(opts), _p(xx), C.byref(r)))
        return (self.positions() if xx is None else xx), r.as_dict()

    def solve_log(self):
        """Per-iteration trace of the last solve: obj, opt, bisections, step."""
        n = lib().phx_solve_log(self.h, None, None, None, None, 0)
        if n < 0:
            _check(n)
        k = min(n, 256)
        obj = np.zeros(k); opt = np.zeros(k); bis = np.zeros(k, dtype=np.int32); step = np.zeros(k)
        lib().phx_solve_log(self.h, _p(obj), _p(opt), _p(bis), _p(step), k)
        return {"obj": obj, "opt": opt, "bis": bis, "step": step, "iterations": n}

    def dynamic_step(self, opts: Options, dt: float, x=None, v=None):
        xx = None if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64).copy()
        r = Report()
        _check(lib().phx_dynamic_step(self.h, C.byref(opts), float(dt), _p(xx), _p(vv), C.byref(r)))
        if xx is None:
            xx = self.positions()
        if vv is None:
            vv = self.velocities()
        return xx, vv, r.as_dict()


class Server:
    """Continuous batching over the device engine (phx_server_*)."""

    def __init__(self, ctx: Context, max_slots: int, budget_bytes: int, opts: Options):
        h = C.c_void_p()
        _check(lib().phx_server_create(ctx.h, int(max_slots), int(budget_bytes), C.byref(opts), C.byref(h)))
        self.h = h
        self.ctx = ctx

    def close(self):
        if getattr(self, "h", None):
            lib().phx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, inst: Instance, tag: int):
        """A static solve of a live instance from its current positions (warm re-solve)."""
        _check(lib().phx_server_submit(self.h, inst.h, int(tag)))

    def submit_step(self, inst: Instance, dt: float, tag: int):
        """One implicit-Euler step of a live instance."""
        _check(lib().phx_server_submit_step(self.h, inst.h, float(dt), int(tag)))

    def submit_mesh(self, m, tag: int) -> Instance:
        """A cold request: the server builds the instance of mesh m at admission, then solves it
        from rest.  Returns the instance (destroy it when done with it)."""
        d, keep = _mesh_desc(m)
        h = C.c_void_p()
        _check(lib().phx_server_submit_mesh(self.h, C.byref(d), int(tag), C.byref(h)))
        del keep  # the server copied the mesh
        return Instance(self.ctx, m, _handle=h)

    def stats(self):
        a, b, c, d = (C.c_int64() for _ in range(4))
        _check(lib().phx_server_stats(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"in_use": a.value, "peak": b.value, "resident": c.value, "evictions": d.value}

    def progress(self):
        a = C.c_int32(); q = C.c_int32()
        _check(lib().phx_server_progress(self.h, C.byref(a), C.byref(q)))
        return a.value, q.value

    def poll(self, cap: int = 1024):
        tags = np.zeros(cap, dtype=np.int64)
        reps = (Report * cap)()
        n = lib().phx_server_poll(self.h, _p(tags), reps, cap)
        if n < 0:
            _check(n)
        return [(int(tags[i]), reps[i].as_dict()) for i in range(n)]


class Scene:
    """A scene file in the reference's XML vocabulary (phx_scene_*): the model, the problem,
    the solver options and the boundary conditions, with TetGen volume meshes."""

    def __init__(self, path: str):
        h = C.c_void_p()
        _check(lib().phx_scene_load(os.fsencode(path), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().phx_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        n, m, dyn, ng, ns, fl = (C.c_int32() for _ in range(6))
        dt = C.c_double()
        _check(lib().phx_scene_info(self.h, C.byref(n), C.byref(m), C.byref(dyn), C.byref(dt), C.byref(ng),
                                    C.byref(ns), C.byref(fl)))
        return {"nodes": n.value, "tets": m.value, "dynamic": bool(dyn.value), "dt": dt.value, "groups": ng.value,
                "num_stages": ns.value, "reoriented": fl.value}

    def mesh(self):
        """(mesh, x_init): the model as a physim_gb300.mesh.Mesh (copies) and its start positions."""
        d = Mesh_()
        info = self.info()
        x = np.zeros(3 * info["nodes"])
        _check(lib().phx_scene_mesh(self.h, C.byref(d), _p(x)))
        n, m = d.num_nodes, d.num_tets

        def arr(ptr, count, ctype, dtype):
            if not ptr:
                return None
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).astype(dtype).copy()

        out = mesh.Mesh(X0=arr(d.X0, 3 * n, C.c_double, np.float64).reshape(n, 3),
                        T=arr(d.tets, 4 * m, C.c_int32, np.int32).reshape(m, 4),
                        lame=arr(d.lame, 2 * m, C.c_double, np.float64).reshape(m, 2),
                        rho=arr(d.rho, m, C.c_double, np.float64),
                        model=arr(d.model, m, C.c_uint8, np.uint8),
                        fixed=arr(d.fixed, 3 * n, C.c_uint8, np.uint8),
                        force=np.zeros(3 * n), gravity=np.array([d.gravity[k] for k in range(3)]),
                        dims=None, name="scene")
        if d.soft_k:
            out.soft_k = arr(d.soft_k, n, C.c_double, np.float64)
            out.soft_target = arr(d.soft_target, 3 * n, C.c_double, np.float64)
        return out, x

    def options(self) -> Options:
        o = Options()
        _check(lib().phx_scene_options(self.h, C.byref(o)))
        return o

    def staging(self):
        """The animated FixPosition groups as dicts (num_stages, soft, k_start, k_end, move, shift, nodes)."""
        k = lib().phx_scene_staging(self.h, None, 0)
        if k < 0:
            _check(k)
        arr = (StageGroup_ * max(1, k))()
        lib().phx_scene_staging(self.h, arr, k)
        out = []
        for g in arr[:k]:
            nodes = np.ctypeslib.as_array(C.cast(g.nodes, C.POINTER(C.c_int32)), shape=(g.num_nodes,)).copy() \
                if g.num_nodes else np.zeros(0, dtype=np.int32)
            out.append({"num_stages": g.num_stages, "soft": g.soft, "k_start": g.k_start, "k_end": g.k_end,
                        "move": np.array(list(g.move)).reshape(3, 3), "shift": np.array(list(g.shift)),
                        "nodes": nodes})
        return out

    def instance(self, ctx: Context) -> "Instance":
        """The scene's instance on the device: mesh, start positions and staging."""
        m, _ = self.mesh()
        h = C.c_void_p()
        _check(lib().phx_scene_instance(ctx.h, self.h, C.byref(h)))
        return Instance(ctx, m, _handle=h)
