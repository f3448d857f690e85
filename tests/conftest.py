import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NATIVE = os.path.join(ROOT, "tests", "native")
CSRC = os.path.join(ROOT, "physim_gb300", "csrc")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a path)")


def _build_shim(name, srcs):
    out_dir = os.path.join(NATIVE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, f"lib{name}.so")
    deps = [os.path.join(NATIVE, s) if not os.path.isabs(s) else s for s in srcs]
    deps_all = deps + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    if not os.path.exists(out) or any(os.path.getmtime(d) > os.path.getmtime(out) for d in deps_all):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", CSRC, "-o", out] + deps
        subprocess.check_call(cmd)
    return out


@pytest.fixture(scope="session")
def pattern_shim():
    import ctypes as C
    path = _build_shim("pattern_shim", ["pattern_shim.cpp", os.path.join(CSRC, "pattern.cpp")])
    return C.CDLL(path)


@pytest.fixture(scope="session")
def ctl_shim():
    import ctypes as C
    path = _build_shim("ctl_shim", ["ctl_shim.cpp"])
    return C.CDLL(path)


@pytest.fixture(scope="session")
def admission_shim():
    import ctypes as C
    path = _build_shim("admission_shim", ["admission_shim.cpp"])
    L = C.CDLL(path)
    L.adm_decide.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_longlong, C.c_int, C.c_void_p,
                             C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
    return L


@pytest.fixture(scope="session")
def gpu_ctx():
    import physim_gb300 as px
    from physim_gb300 import build
    build.build()
    ctx = px.Context(0, arena_bytes=24 << 30)
    yield ctx
    ctx.close()


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))
