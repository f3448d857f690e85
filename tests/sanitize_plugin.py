"""pytest plugin: the host tests against AddressSanitizer + UndefinedBehaviorSanitizer builds.

The oracle, the product's pattern builder (physim_gb300/csrc/pattern.cpp) and its Newton
state machine (physim_gb300/csrc/newton_control.h, through tests/native/ctl_shim.cpp)
are rebuilt with -fsanitize=address,undefined into tests/native/_build, and the session
loads those instead of the optimised builds.  The sanitizer runtimes must be preloaded
into the Python process:

    LD_PRELOAD="$(gcc -print-file-name=libasan.so) $(gcc -print-file-name=libubsan.so)" \\
    ASAN_OPTIONS=detect_leaks=0 UBSAN_OPTIONS=print_stacktrace=1 PYTHONPATH=tests \\
    python -m pytest -p sanitize_plugin tests/test_pattern_host.py tests/test_control_host.py \\
        tests/test_oracle.py -q -s

A sanitizer report is printed to stderr ("runtime error" / "AddressSanitizer").
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "native", "_build")
CSRC = os.path.join(ROOT, "physim_gb300", "csrc")
FLAGS = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-g", "-O1", "-std=c++17", "-fPIC", "-shared"]


def _build(name, srcs, extra=()):
    os.makedirs(OUT, exist_ok=True)
    out = os.path.join(OUT, f"lib{name}_san.so")
    if not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in srcs):
        subprocess.check_call(["g++"] + FLAGS + list(extra) + ["-I", CSRC, "-o", out] + srcs)
    return out


def pytest_sessionstart(session):
    import oracle.build as ob
    orc = _build("oracle", [os.path.join(ROOT, "oracle", "phx_oracle.cpp")], ["-fopenmp"])
    ob.build_oracle = lambda force=False: orc
    native = os.path.join(HERE, "native")
    paths = {
        "pattern_shim": _build("pattern_shim", [os.path.join(native, "pattern_shim.cpp"),
                                                os.path.join(CSRC, "pattern.cpp")]),
        "ctl_shim": _build("ctl_shim", [os.path.join(native, "ctl_shim.cpp")]),
    }
    conftest = sys.modules["conftest"]
    conftest._build_shim = lambda name, srcs: paths[name]
