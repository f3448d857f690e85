"""Restatement of the SVL scalar-grid file format (test infrastructure only).

Serializer_Field (source/PhySim/Utils/Serializer_Field.cpp) writes, in writeGridSVL
(:114-140): the grid's shape as 3 int, its origin and delta as 3 double each, the value type
as an int (SVLFormatMapping, :23-46: char 0, short 1, int 2, float 3, double 4), then the
values in the storage order of the grid's Eigen tensor (column-major: x fastest), all in
native byte order with no padding.  readGridSVL (:50-112) reads the same layout and casts
value by value when the file's type differs from the grid's (IOUtils::readBinaryArrayWithCast,
include/PhySim/Utils/IOUtils.h:51-57).  The tests compare the library's files and reads with
these byte strings.
"""
from __future__ import annotations

import struct

import numpy as np

TYPES = {0: np.int8, 1: np.int16, 2: np.int32, 3: np.float32, 4: np.float64}


def pack(values: np.ndarray, origin, delta, fmt: int) -> bytes:
    """The bytes writeGridSVL produces for values[i, j, k] of SVL type fmt."""
    values = np.asarray(values)
    head = struct.pack("=3i3d3di", *values.shape, *[float(v) for v in origin], *[float(v) for v in delta], fmt)
    return head + np.asarray(values, dtype=TYPES[fmt]).ravel(order="F").tobytes()


def parse(data: bytes):
    """(values[i, j, k] in the file's type, origin, delta, type) of an SVL byte string."""
    sx, sy, sz, ox, oy, oz, dx, dy, dz, fmt = struct.unpack_from("=3i3d3di", data, 0)
    count = sx * sy * sz
    vals = np.frombuffer(data, dtype=TYPES[fmt], count=count, offset=struct.calcsize("=3i3d3di"))
    return vals.reshape((sx, sy, sz), order="F"), (ox, oy, oz), (dx, dy, dz), fmt
