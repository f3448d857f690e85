"""Field output on the host: SVL grid files through the library, and the grid sampler's
restatement in the oracle.

* The library writes the bytes of the format's restatement (oracle/svl.py, from
  Serializer_Field.cpp) for every value type, and reads them back; converting reads follow
  readBinaryArrayWithCast (truncation toward zero into integers) and refuse values the
  target type cannot hold; malformed files are refused with a status, not read.
* The sampler's restatement (oracle/field_oracle.cpp): a centre on a mesh node belongs to
  the lowest-index tet at that node, every centre inside the box has an owner and every
  centre outside gets the fill value, a linear displacement field is interpolated exactly
  (up to rounding), and J = 1, u = 0 at rest.
"""
import os
import struct

import numpy as np
import pytest

import oracle
from oracle import svl
import physim_gb300 as px
from physim_gb300 import mesh as M


def _arr(fmt, shape, seed):
    rng = np.random.default_rng(seed)
    t = svl.TYPES[fmt]
    if np.issubdtype(t, np.integer):
        info = np.iinfo(t)
        return rng.integers(info.min, info.max, size=shape, endpoint=True).astype(t)
    return rng.standard_normal(shape).astype(t)


@pytest.mark.parametrize("fmt", [0, 1, 2, 3, 4])
def test_svl_bytes_and_round_trip(tmp_path, fmt):
    vals = _arr(fmt, (5, 3, 2), fmt)
    origin, delta = (-1.5, 0.25, 3.0), (0.5, 0.125, 2.0)
    p = str(tmp_path / "g.svl")
    px.write_svl(p, vals, origin, delta)
    data = open(p, "rb").read()
    assert data == svl.pack(vals, origin, delta, fmt)
    assert len(data) == 64 + vals.size * vals.itemsize
    back, o, d = px.read_svl(p)
    assert back.dtype == vals.dtype and back.shape == vals.shape and np.array_equal(back, vals)
    assert o == origin and d == delta
    assert px.read_svl_header(p) == ((5, 3, 2), origin, delta, fmt)
    # x varies fastest in the file
    v2, *_ = svl.parse(data)
    assert np.array_equal(v2, vals)
    flat = np.frombuffer(data[64:], dtype=vals.dtype)
    assert flat[1] == vals[1, 0, 0] and flat[5] == vals[0, 1, 0] and flat[15] == vals[0, 0, 1]


def test_svl_char_is_signed(tmp_path):
    p = str(tmp_path / "c.svl")
    open(p, "wb").write(svl.pack(np.array([-5, 127, -128], dtype=np.int8).reshape(3, 1, 1), (0, 0, 0), (1, 1, 1), 0))
    v, *_ = px.read_svl(p, dtype=np.float64)
    assert v.ravel().tolist() == [-5.0, 127.0, -128.0]


def test_svl_converting_reads(tmp_path):
    p = str(tmp_path / "f.svl")
    f = np.array([1.9, -1.9, 0.5, -0.5, 32767.2, -32768.9], dtype=np.float32).reshape(6, 1, 1)
    open(p, "wb").write(svl.pack(f, (0, 0, 0), (1, 1, 1), 3))
    # float -> short truncates toward zero (the reference's TBuffer(value))
    s, *_ = px.read_svl(p, dtype=np.int16)
    assert s.ravel().tolist() == [1, -1, 0, 0, 32767, -32768]
    d, *_ = px.read_svl(p, dtype=np.float64)
    assert np.array_equal(d.ravel(), f.ravel().astype(np.float64))
    # int -> float and int -> double are exact for these values
    q = str(tmp_path / "i.svl")
    i = np.array([-(2 ** 24), 3, 2 ** 24], dtype=np.int32).reshape(1, 3, 1)
    open(q, "wb").write(svl.pack(i, (0, 0, 0), (1, 1, 1), 2))
    assert px.read_svl(q, dtype=np.float32)[0].ravel().tolist() == [-(2.0 ** 24), 3.0, 2.0 ** 24]


@pytest.mark.parametrize("vals,fmt,to", [
    (np.array([1e10], dtype=np.float64), 4, np.int32),    # out of range
    (np.array([np.nan], dtype=np.float32), 3, np.int16),  # NaN into an integer
    (np.array([300], dtype=np.int16), 1, np.int8),        # narrowing out of range
    (np.array([1e300], dtype=np.float64), 4, np.float32),
])
def test_svl_refuses_values_the_target_cannot_hold(tmp_path, vals, fmt, to):
    p = str(tmp_path / "r.svl")
    open(p, "wb").write(svl.pack(vals.reshape(-1, 1, 1), (0, 0, 0), (1, 1, 1), fmt))
    with pytest.raises(px.PhxError) as ei:
        px.read_svl(p, dtype=to)
    assert ei.value.code == px.PHX_EINVAL


def test_svl_nan_and_inf_stay_floating(tmp_path):
    p = str(tmp_path / "n.svl")
    v = np.array([np.nan, np.inf, -np.inf], dtype=np.float64).reshape(3, 1, 1)
    open(p, "wb").write(svl.pack(v, (0, 0, 0), (1, 1, 1), 4))
    f, *_ = px.read_svl(p, dtype=np.float32)
    assert np.isnan(f[0, 0, 0]) and f[1, 0, 0] == np.inf and f[2, 0, 0] == -np.inf


def test_svl_malformed_files(tmp_path):
    good = svl.pack(np.arange(8, dtype=np.float64).reshape(2, 2, 2), (0, 0, 0), (1, 1, 1), 4)
    cases = {
        "short_header": good[:40],
        "short_values": good[:-8],
        "bad_type": good[:60] + struct.pack("=i", 7) + good[64:],
        "zero_shape": struct.pack("=3i", 0, 2, 2) + good[12:],
    }
    for name, data in cases.items():
        p = str(tmp_path / f"{name}.svl")
        open(p, "wb").write(data)
        with pytest.raises(px.PhxError) as ei:
            px.read_svl(p)
        assert ei.value.code == px.PHX_EINVAL, name
    with pytest.raises(px.PhxError) as ei:
        px.read_svl(str(tmp_path / "missing.svl"))
    assert ei.value.code == px.PHX_ENOTFOUND
    # room for fewer values than the grid holds
    p = str(tmp_path / "ok.svl")
    open(p, "wb").write(good)
    buf = np.empty(7)
    assert px.lib().phx_svl_read(os.fsencode(p), 4, buf.ctypes.data, 7) == px.PHX_EINVAL
    # writing: unknown type, shape below 1
    g = px._grid((1, 1, 1), (0, 0, 0), (1, 1, 1))
    assert px.lib().phx_svl_write(os.fsencode(p), g, 9, buf.ctypes.data) == px.PHX_EINVAL
    g = px._grid((1, 0, 1), (0, 0, 0), (1, 1, 1))
    assert px.lib().phx_svl_write(os.fsencode(p), g, 4, buf.ctypes.data) == px.PHX_EINVAL
    with pytest.raises(ValueError):
        px.write_svl(p, np.zeros((2, 2, 2), dtype=np.uint16))


def _unit_box(n):
    X0, T = M.box_grid(n, n, n, (1.0, 1.0, 1.0))
    return X0, T


def test_sampler_owner_at_nodes_is_lowest_incident_tet():
    n = 4
    X0, T = _unit_box(n)
    h = 1.0 / n
    # cell centres on the nodes: origin -h/2, delta h (exact binary fractions)
    vals, own = oracle.sample_grid(X0, T, X0, px.FIELD_DISPLACEMENT_X, (n + 1,) * 3, (-h / 2,) * 3, (h,) * 3, fill=-7.0)
    lowest = np.full(len(X0), np.iinfo(np.int32).max)
    np.minimum.at(lowest, T.ravel(), np.repeat(np.arange(len(T)), 4))
    # node (i, j, k) is value i + (n+1)(j + (n+1) k): the node numbering
    assert np.array_equal(own, lowest.astype(np.int32))
    assert np.all(vals == 0.0)


def test_sampler_covers_the_box_and_fills_outside():
    n = 3
    X0, T = _unit_box(n)
    shape = (11, 9, 10)
    origin = (-0.2, -0.1, -0.15)
    delta = (1.4 / 11, 1.2 / 9, 1.3 / 10)
    vals, own = oracle.sample_grid(X0, T, X0, px.FIELD_VOLUME_RATIO, shape, origin, delta, fill=-1.0)
    vals = vals.reshape(shape, order="F"); own = own.reshape(shape, order="F")
    c = [origin[d] + (np.arange(shape[d]) + 0.5) * delta[d] for d in range(3)]
    inside = ((c[0][:, None, None] > 1e-9) & (c[0][:, None, None] < 1 - 1e-9) &
              (c[1][None, :, None] > 1e-9) & (c[1][None, :, None] < 1 - 1e-9) &
              (c[2][None, None, :] > 1e-9) & (c[2][None, None, :] < 1 - 1e-9))
    outside = ((c[0][:, None, None] < -1e-9) | (c[0][:, None, None] > 1 + 1e-9) |
               (c[1][None, :, None] < -1e-9) | (c[1][None, :, None] > 1 + 1e-9) |
               (c[2][None, None, :] < -1e-9) | (c[2][None, None, :] > 1 + 1e-9))
    assert inside.sum() > 100 and outside.sum() > 100
    assert np.all(own[inside] >= 0) and np.all(vals[inside] == 1.0)
    assert np.all(own[outside] == -1) and np.all(vals[outside] == -1.0)
    # each owner holds its centre (barycentric weights from numpy, loose)
    idx = np.argwhere(inside)
    for i, j, k in idx[:: max(1, len(idx) // 200)]:
        t = T[own[i, j, k]]
        A = np.stack([X0[t[1]] - X0[t[0]], X0[t[2]] - X0[t[0]], X0[t[3]] - X0[t[0]]], axis=1)
        mu = np.linalg.solve(A, np.array([c[0][i], c[1][j], c[2][k]]) - X0[t[0]])
        assert mu.min() > -1e-9 and mu.sum() < 1 + 1e-9


def test_sampler_interpolates_a_linear_field():
    m = M.cantilever(3, 3, 8)
    X0 = m.X0
    A = np.array([[0.01, -0.02, 0.003], [0.004, 0.02, -0.01], [0.0, 0.005, -0.015]])
    b = np.array([1e-3, -2e-3, 5e-4])
    x = X0 + X0 @ A.T + b
    shape, origin, delta = (7, 6, 20), (0.0, 0.0, 0.0), (0.1 / 7, 0.1 / 6, 0.4 / 20)
    c = np.stack(np.meshgrid(*[origin[d] + (np.arange(shape[d]) + 0.5) * delta[d] for d in range(3)],
                             indexing="ij"), axis=-1).reshape(-1, 3, order="F")
    want = c @ A.T + b
    for f in range(3):
        vals, own = oracle.sample_grid(X0, m.T, x, f, shape, origin, delta)
        assert np.all(own >= 0)
        assert np.max(np.abs(vals - want[:, f])) < 1e-14
    nrm, _ = oracle.sample_grid(X0, m.T, x, px.FIELD_DISPLACEMENT_NORM, shape, origin, delta)
    assert np.max(np.abs(nrm - np.linalg.norm(want, axis=1))) < 1e-14
    J, _ = oracle.sample_grid(X0, m.T, x, px.FIELD_VOLUME_RATIO, shape, origin, delta)
    assert np.max(np.abs(J - np.linalg.det(np.eye(3) + A))) < 1e-12


def test_sampler_energy_density_is_energy_over_rest_volume():
    m = M.cantilever(2, 2, 4)
    orc = oracle.Oracle(m)
    x = m.X0.ravel() + 1e-3 * np.sin(np.arange(3 * m.n))
    E, _, _ = orc.element_local(x)
    shape, origin, delta = (4, 4, 8), (0.0, 0.0, 0.0), (0.025, 0.025, 0.05)
    vals, own = oracle.sample_grid(m.X0, m.T, x, px.FIELD_ENERGY_DENSITY, shape, origin, delta, E=E)
    vol = np.abs(M.signed_volumes(m.X0, m.T))
    assert np.all(own >= 0)
    np.testing.assert_allclose(vals, E[own] / vol[own], rtol=1e-12)
