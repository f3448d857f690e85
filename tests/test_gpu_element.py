"""Element kernels, assembly, pattern and scatter map on the GPU against the CPU oracle.

Tolerances: FP64 kernels within 1e-12 relative (the reference's own arithmetic
is FP64; differences are summation order only).  FP32 Hessian kernels within
2e-5 relative to each block's (or the matrix's) largest entry.
"""
import numpy as np
import pytest

import oracle
import physim_gb300 as px
from physim_gb300 import mesh as M
from conftest import rel

pytestmark = pytest.mark.gpu

CASES = {
    "conh_cantilever": lambda: M.cantilever(4, 3, 9),
    "stvk_traction": lambda: M.make_box(3, 4, 5, (0.03, 0.04, 0.05), 3e5, 0.4, 1000.0, M.MODEL_STVK,
                                        (0.0, -9.81, 0.0), clamp_face=0, load_face=1, traction=(50.0, 80.0, -20.0)),
    "batch_instance": lambda: M.batch_instance(3, 7),
}


def perturbed(m, scale, seed=1):
    rng = np.random.default_rng(seed)
    h = np.min(np.linalg.norm(m.X0[m.T[:, 1]] - m.X0[m.T[:, 0]], axis=1))
    return (m.X0 + scale * h * rng.standard_normal(m.X0.shape)).ravel()


@pytest.mark.parametrize("name", list(CASES))
def test_element_local_fp64(gpu_ctx, name):
    m = CASES[name]()
    inst = px.Instance(gpu_ctx, m)
    orc = oracle.Oracle(m)
    x = perturbed(m, 0.05)
    E, g, H = inst.element_local(x, px.PREC_FP64)
    Eo, go, Ho = orc.element_local(x)
    assert np.max(np.abs(E - Eo) / np.maximum(np.abs(Eo), 1e-300)) < 1e-11
    assert np.max(np.abs(g - go)) <= 1e-12 * np.abs(go).max()
    for e in range(0, m.m, 5):
        assert np.abs(H[e] - Ho[e]).max() <= 1e-11 * np.abs(Ho[e]).max()


@pytest.mark.parametrize("name", list(CASES))
def test_element_hessian_fp32(gpu_ctx, name):
    m = CASES[name]()
    inst = px.Instance(gpu_ctx, m)
    orc = oracle.Oracle(m)
    x = perturbed(m, 0.05, seed=2)
    _, _, H = inst.element_local(x, px.PREC_FP32_REFINE)
    _, _, Ho = orc.element_local(x)
    err = np.abs(H - Ho).max(axis=(1, 2)) / np.abs(Ho).max(axis=(1, 2))
    assert err.max() < 2e-5


@pytest.mark.parametrize("name", list(CASES))
def test_energy_gradient(gpu_ctx, name):
    m = CASES[name]()
    inst = px.Instance(gpu_ctx, m)
    orc = oracle.Oracle(m)
    for seed in (3, 4):
        x = perturbed(m, 0.03, seed)
        for fix in (True, False):
            E, g = inst.energy_gradient(x, fix=fix)
            assert abs(E - orc.energy(x)) <= 1e-12 * max(abs(E), 1e-300) + 1e-15 * np.abs(orc.element_local(x)[0]).sum()
            go = orc.gradient(x, fix=fix)
            assert np.abs(g - go).max() <= 1e-12 * np.abs(go).max()


def test_inverted_element_gives_infinite_energy(gpu_ctx):
    m = CASES["conh_cantilever"]()
    inst = px.Instance(gpu_ctx, m)
    x = m.X0.copy()
    t = m.T[10]
    x[t[0]] = x[t[1]] + 2 * (x[t[1]] - x[t[0]])
    E, g = inst.energy_gradient(x.ravel())
    assert np.isinf(E) and E > 0
    Ee, _, _ = inst.element_local(x.ravel())
    assert np.isinf(Ee[10])


@pytest.mark.parametrize("name", list(CASES))
def test_pattern_and_scatter_map_bit_exact(gpu_ctx, name):
    m = CASES[name]()
    inst = px.Instance(gpu_ctx, m)
    orc = oracle.Oracle(m)
    cp, ri = inst.pattern()
    cpo, rio = orc.pattern()
    assert np.array_equal(cp, cpo) and np.array_equal(ri, rio)
    assert np.array_equal(inst.scatter_map(), orc.scatter_map())
    s = inst.sizes()
    assert s["nnz"] == len(rio) and s["lower_blocks"] == m.n + len(M.unique_edges(m.T))


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("fix", [True, False])
def test_assembled_hessian(gpu_ctx, name, fix):
    m = CASES[name]()
    inst = px.Instance(gpu_ctx, m)
    orc = oracle.Oracle(m)
    x = perturbed(m, 0.05, seed=5)
    Ho = orc.hessian(x, fix=fix)
    H64 = inst.hessian(x, px.PREC_FP64, fix=fix)
    assert np.abs(H64 - Ho).max() <= 1e-12 * np.abs(Ho).max()
    H32 = inst.hessian(x, px.PREC_FP32_REFINE, fix=fix)
    assert np.abs(H32 - Ho).max() <= 2e-5 * np.abs(Ho).max()
    if fix:
        cp, ri = orc.pattern()
        cols = np.repeat(np.arange(len(cp) - 1), np.diff(cp))
        fx = m.fixed.astype(bool)[ri] | m.fixed.astype(bool)[cols]
        assert np.all(H64[fx] == np.where(ri[fx] == cols[fx], 1.0, 0.0))


def test_bad_mesh_rejected_through_the_abi(gpu_ctx):
    m = CASES["conh_cantilever"]()
    bad = m.copy()
    bad.T[5, [1, 2]] = bad.T[5, [2, 1]]
    with pytest.raises(px.PhxError) as ei:
        px.Instance(gpu_ctx, bad)
    assert ei.value.code == px.PHX_EINVAL and "rest volume" in str(ei.value)
    bad = m.copy()
    bad.T[0, 0] = -1
    with pytest.raises(px.PhxError):
        px.Instance(gpu_ctx, bad)


def test_bad_options_rejected(gpu_ctx):
    m = M.cantilever(2, 2, 2)
    inst = px.Instance(gpu_ctx, m)
    with pytest.raises(px.PhxError):
        inst.solve_static(px.options(precision=7))
    with pytest.raises(px.PhxError):
        inst.solve_static(px.options(lsearch_type=5))
    with pytest.raises(px.PhxError):
        inst.solve_static(px.options(lsearch_type=3, lsearch_wolfe1=0.5, lsearch_wolfe2=0.4))
