"""The ctypes mirrors of the public structs have the C layout of include/phx.h.

A small C program compiled here against the header prints sizeof and the offset of every
field of phx_mesh, phx_options, phx_report, phx_launch_settings, phx_stage_group and phx_grid;
the Python structures must agree field by field, so that a field added to one side only is
caught without a GPU.
"""
import ctypes as C
import os
import shutil
import subprocess

import pytest

import physim_gb300 as px

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MIRRORS = {
    "phx_mesh": px.Mesh_,
    "phx_options": px.Options,
    "phx_report": px.Report,
    "phx_launch_settings": px.LaunchSettings_,
    "phx_stage_group": px.StageGroup_,
    "phx_grid": px.Grid_,
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "phx.h"', "int main(void) {"]
    for name, cls in MIRRORS.items():
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.check_call([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        struct, key, value = line.split()
        out[(struct, key)] = int(value)
    return out


@pytest.mark.parametrize("name", sorted(MIRRORS))
def test_struct_layout_matches_header(c_layout, name):
    cls = MIRRORS[name]
    assert C.sizeof(cls) == c_layout[(name, "size")], name
    for field, _ in cls._fields_:
        assert getattr(cls, field).offset == c_layout[(name, field)], (name, field)
