"""Grid sampling of a solve's fields on the GPU (k_grid_init / k_grid_claim / k_grid_eval)
against the oracle's restatement, bit for bit: owners and values of every field, on grids
whose centres fall on nodes (shared by many tets), off the nodes, partly outside the mesh,
much finer than the mesh, and on a renumbered mesh; then the sampled field written as an
SVL file and read back."""
import numpy as np
import pytest

import oracle
import physim_gb300 as px
from physim_gb300 import mesh as M

pytestmark = pytest.mark.gpu

FIELDS = [px.FIELD_DISPLACEMENT_X, px.FIELD_DISPLACEMENT_Y, px.FIELD_DISPLACEMENT_Z,
          px.FIELD_DISPLACEMENT_NORM, px.FIELD_VOLUME_RATIO, px.FIELD_ENERGY_DENSITY]


def _same_as_oracle(inst, m, x, shape, origin, delta, fill=-3.0):
    E, _, _ = inst.element_local(x)
    for f in FIELDS:
        vals, own = inst.sample_grid(f, shape, origin, delta, x=x, fill=fill)
        ov, oo = oracle.sample_grid(m.X0, m.T, x, f, shape, origin, delta, fill=fill,
                                    E=E if f == px.FIELD_ENERGY_DENSITY else None)
        assert np.array_equal(own.ravel(order="F"), oo), f
        assert np.array_equal(vals.ravel(order="F"), ov, equal_nan=True), f
    return own


def test_sampled_fields_match_oracle_bitwise(gpu_ctx):
    m = M.cantilever(4, 4, 16)
    inst = px.Instance(gpu_ctx, m)
    o = px.options(precision=px.PREC_FP64, tol_rel=1e-8, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)
    x, r = inst.solve_static(o, m.X0.ravel().copy())
    assert r["result_name"] == "SUCCESS"
    h = (0.025, 0.025, 0.025)
    grids = [
        ((5, 5, 17), (-h[0] / 2, -h[1] / 2, -h[2] / 2), h),            # centres on the nodes
        ((9, 7, 30), (0.0, 0.0, 0.0), (0.1 / 9, 0.1 / 7, 0.4 / 30)),   # off the nodes
        ((12, 12, 25), (-0.05, -0.03, -0.1), (0.02, 0.015, 0.025)),    # partly outside
        ((40, 40, 160), (0.0, 0.0, 0.0), (0.0025, 0.0025, 0.0025)),    # ~10 cells per tet edge
        ((1, 1, 1), (0.0, 0.0, 0.0), (0.1, 0.1, 0.4)),
    ]
    for shape, origin, delta in grids:
        own = _same_as_oracle(inst, m, x, shape, origin, delta)
        if shape == (12, 12, 25):
            assert (own == -1).any() and (own >= 0).any()
    inst.close()


def test_sampling_on_a_renumbered_mesh(gpu_ctx):
    m = M.renumbered(M.cantilever(3, 3, 8), 11)
    inst = px.Instance(gpu_ctx, m)
    x = m.X0.ravel() + 2e-3 * np.cos(np.arange(3 * m.n))
    _same_as_oracle(inst, m, x, (8, 8, 20), (0.0, 0.0, 0.0), (0.1 / 8, 0.1 / 8, 0.4 / 20))
    inst.close()


def test_sampled_field_to_svl_file(gpu_ctx, tmp_path):
    m = M.cantilever(3, 3, 8)
    inst = px.Instance(gpu_ctx, m)
    x = m.X0.ravel() + 1e-3 * np.sin(np.arange(3 * m.n))
    shape, origin, delta = (6, 6, 16), (0.0, 0.0, 0.0), (0.1 / 6, 0.1 / 6, 0.4 / 16)
    vals, own = inst.sample_grid(px.FIELD_DISPLACEMENT_NORM, shape, origin, delta, x=x)
    assert np.all(own >= 0)
    p = str(tmp_path / "u.svl")
    px.write_svl(p, vals, origin, delta)
    back, o, d = px.read_svl(p)
    assert np.array_equal(back, vals) and o == origin and d == delta
    # the positions given became the instance's
    assert np.array_equal(inst.positions(), x)
    # argument checks
    for bad in (dict(field=6), dict(shape=(0, 1, 1)), dict(delta=(0.0, 1.0, 1.0))):
        kw = dict(field=0, shape=(2, 2, 2), origin=(0, 0, 0), delta=(1.0, 1.0, 1.0))
        kw.update(bad)
        with pytest.raises(px.PhxError) as ei:
            inst.sample_grid(kw["field"], kw["shape"], kw["origin"], kw["delta"])
        assert ei.value.code == px.PHX_EINVAL
    inst.close()
