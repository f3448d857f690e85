"""Build recipe for the CPU oracle (test infrastructure only).

* ``liboracle.so``  -- the C++ restatement in phx_oracle.cpp (always built).
* ``_ref/libref_mcg.so`` -- the reference's own generated material code, compiled
  from the reference tree when it is present on this machine (it is not on the
  GPU host).  It is only used to regenerate and re-check tests/golden/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load these.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_AUTO = "/root/reference/include/PhySim/Utils/Auto"
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_mcg.so")


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "phx_oracle.cpp"), os.path.join(HERE, "phx_oracle.h")]
    if force or _stale(LIB, srcs):
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
               "-o", LIB, srcs[0]]
        subprocess.check_call(cmd)
    return LIB


def build_ref(force: bool = False) -> str | None:
    if not os.path.isdir(REF_AUTO):
        return None
    os.makedirs(os.path.dirname(REF_LIB), exist_ok=True)
    src = os.path.join(HERE, "ref_mcg_shim.cpp")
    if force or _stale(REF_LIB, [src]):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-I", REF_AUTO,
               "-o", REF_LIB, src]
        subprocess.check_call(cmd)
    return REF_LIB


def build_all(force: bool = False):
    return build_oracle(force), build_ref(force)


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
