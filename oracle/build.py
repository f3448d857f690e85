"""Build recipe for the CPU oracle (test infrastructure only).

* ``liboracle.so``  -- the C++ restatement in phx_oracle.cpp and the grid sampler's in
  field_oracle.cpp (always built).
* ``_ref/libref_mcg.so`` -- the reference's own generated material code, compiled
  from the reference tree when it is present (it is not on the GPU host).  The
  tree is the directory named by the environment variable PHYSIM_REFERENCE, or
  by ``--reference DIR`` on the command line, or /root/reference by default.
  It is only used to regenerate and re-check tests/golden/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load these.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REFERENCE = "/root/reference"
AUTO_SUBDIR = os.path.join("include", "PhySim", "Utils", "Auto")
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_mcg.so")


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    """liboracle.so from phx_oracle.cpp and field_oracle.cpp.  The grid sampler's file is
    compiled with -ffp-contract=off: each product and sum rounds on its own, as the device
    sampler's explicitly rounded operations do, so the two agree bit for bit on any host."""
    srcs = [os.path.join(HERE, f) for f in ("phx_oracle.cpp", "field_oracle.cpp", "phx_oracle.h")]
    if force or _stale(LIB, srcs):
        obj = os.path.join(HERE, "_field_oracle.o")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-c",
                               "-o", obj, srcs[1]])
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                               "-o", LIB, srcs[0], obj])
        os.remove(obj)
    return LIB


def reference_root(arg: str | None = None) -> str:
    """The reference tree: an explicit argument, else $PHYSIM_REFERENCE, else the default."""
    return arg or os.environ.get("PHYSIM_REFERENCE") or DEFAULT_REFERENCE


def build_ref(force: bool = False, reference: str | None = None) -> str | None:
    auto = os.path.join(reference_root(reference), AUTO_SUBDIR)
    if not os.path.isdir(auto):
        return None
    os.makedirs(os.path.dirname(REF_LIB), exist_ok=True)
    src = os.path.join(HERE, "ref_mcg_shim.cpp")
    if force or _stale(REF_LIB, [src]):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-I", auto,
               "-o", REF_LIB, src]
        subprocess.check_call(cmd)
    return REF_LIB


def build_all(force: bool = False, reference: str | None = None):
    return build_oracle(force), build_ref(force, reference)


if __name__ == "__main__":
    ref = None
    if "--reference" in sys.argv:
        ref = sys.argv[sys.argv.index("--reference") + 1]
    print(build_all(force="--force" in sys.argv, reference=ref))
