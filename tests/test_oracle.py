"""The CPU oracle against the reference's own material code, known answers and FD checks.

Golden vectors: tests/golden/material_golden.npz, produced by the reference's
generated .mcg code (see tests/golden/gen_golden.py).  FD checks mirror
EnergyElement::TestLocalGradient/TestLocalHessian (source/PhySim/Physics/
Elements/EnergyElement.cpp:244-329): central differences, eps = 1e-6,
pass if ||analytic - FD|| / ||FD|| <= 1e-6.
"""
import os

import numpy as np
import pytest

import oracle
from physim_gb300 import mesh as M
from conftest import rel

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("model,name", [(0, "conh"), (1, "stvk")])
def test_material_matches_reference_mcg(model, name):
    g = np.load(os.path.join(GOLD, "material_golden.npz"))
    F, lame = g[f"{name}_F"], g[f"{name}_lame"]
    for k in range(F.shape[0]):
        psi, P, D = oracle.material(model, lame[k, 0], lame[k, 1], F[k])
        assert abs(psi - g[f"{name}_psi"][k]) <= 1e-12 * max(1.0, abs(g[f"{name}_psi"][k])) + 1e-9 * lame[k].max() * 1e-12
        assert rel(P, g[f"{name}_P"][k]) < 1e-12
        assert rel(D, g[f"{name}_dPdF"][k]) < 1e-12


@pytest.mark.parametrize("model,name", [(0, "conh"), (1, "stvk")])
def test_material_extremes_match_reference_mcg(model, name):
    """Strong compression, strong stretch, near-identity and large random deformation
    gradients against the reference's generated code.  Within 1e-6 of the identity the
    reference forms P and psi with cancellation, so there the bound is the stress scale
    (lambda + mu) times a few ulps rather than |P| itself."""
    g = np.load(os.path.join(GOLD, "material_extreme_golden.npz"))
    F, lame, kind = g[f"{name}_F"], g[f"{name}_lame"], g[f"{name}_kind"]
    assert sorted(set(kind.tolist())) == [0, 1, 2, 3]
    for k in range(F.shape[0]):
        psi, P, D = oracle.material(model, lame[k, 0], lame[k, 1], F[k])
        scale = lame[k].sum()
        gp, gP, gD = g[f"{name}_psi"][k], g[f"{name}_P"][k], g[f"{name}_dPdF"][k]
        assert abs(psi - gp) <= 1e-13 * abs(gp) + 1e-15 * scale, (k, kind[k])
        assert np.abs(P - gP).max() <= 1e-13 * np.abs(gP).max() + 1e-15 * scale, (k, kind[k])
        assert np.abs(D - gD).max() <= 1e-13 * np.abs(gD).max(), (k, kind[k])


@pytest.mark.skipif(oracle.ref_lib() is None, reason="reference sources not present")
def test_golden_file_matches_reference_build():
    """Re-derive a few golden entries from the reference build itself (where it exists)."""
    g = np.load(os.path.join(GOLD, "material_golden.npz"))
    R = oracle.ref_lib()
    for name, fn in (("conh", R.ref_conh), ("stvk", R.ref_stvk)):
        for k in range(0, 200, 37):
            Fv = np.ascontiguousarray(g[f"{name}_F"][k])
            U = np.zeros(1); P = np.zeros(9); H = np.zeros(81)
            fn(g[f"{name}_lame"][k, 0], g[f"{name}_lame"][k, 1], Fv.ctypes.data, U.ctypes.data, P.ctypes.data,
               H.ctypes.data)
            assert U[0] == g[f"{name}_psi"][k]
            assert np.array_equal(P, g[f"{name}_P"][k])


@pytest.mark.parametrize("model", [0, 1])
def test_rest_state_is_stress_free(model):
    psi, P, D = oracle.material(model, 3e4, 1e4, np.eye(3).T.ravel())
    assert abs(psi) < 1e-12 and np.abs(P).max() < 1e-9
    # linearised: dP/dF at rest = mu (I + T) + lambda vec(I) vec(I)^T
    lam, mu = 3e4, 1e4
    I9 = np.eye(9)
    Tm = np.zeros((9, 9))
    for i in range(3):
        for j in range(3):
            Tm[i + 3 * j, j + 3 * i] = 1.0
    vI = np.eye(3).T.ravel()
    assert np.allclose(D, mu * (I9 + Tm) + lam * np.outer(vI, vI), rtol=1e-12, atol=1e-9)


def test_uniaxial_known_answers():
    lam, mu, s = 2e5, 7e4, 1.3
    F = np.diag([s, 1.0, 1.0])
    psi, P, _ = oracle.material(0, lam, mu, F.T.ravel())
    ls = np.log(s)
    assert np.isclose(psi, mu / 2 * (s * s - 1 - 2 * ls) + lam / 2 * ls * ls, rtol=1e-13)
    assert np.isclose(P[0], mu * s + (lam * ls - mu) / s, rtol=1e-13)
    psi, P, _ = oracle.material(1, lam, mu, F.T.ravel())
    e = 0.5 * (s * s - 1)
    assert np.isclose(psi, lam / 2 * e * e + mu * e * e, rtol=1e-13)
    assert np.isclose(P[0], s * (lam * e + 2 * mu * e), rtol=1e-13)


@pytest.mark.parametrize("model", [0, 1])
def test_rotation_invariance(model):
    rng = np.random.default_rng(5)
    for _ in range(20):
        F = np.eye(3) + 0.3 * rng.standard_normal((3, 3))
        if np.linalg.det(F) < 0:
            F[:, 0] *= -1
        Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        if np.linalg.det(Q) < 0:
            Q[:, 0] *= -1
        a, _, _ = oracle.material(model, 1e5, 4e4, F.T.ravel())
        b, _, _ = oracle.material(model, 1e5, 4e4, (Q @ F).T.ravel())
        assert abs(a - b) <= 1e-9 * abs(a)


def _small(model=0):
    m = M.make_box(2, 2, 2, (0.02, 0.02, 0.02), 1e5, 0.3, 1000.0, model, (0.0, -9.81, 0.0), clamp_face=4)
    return m


@pytest.mark.parametrize("model", [0, 1])
def test_element_fd_like_reference(model):
    m = _small(model)
    o = oracle.Oracle(m)
    rng = np.random.default_rng(3)
    x = o.rest() + 2e-3 * rng.standard_normal(o.N)
    E, g, H = o.element_local(x)
    eps = 1e-6
    for e in range(0, m.m, 7):
        nodes = m.T[e]
        gfd = np.zeros(12)
        Hfd = np.zeros((12, 12))
        for d in range(12):
            xp = x.copy(); xm = x.copy()
            xp[3 * nodes[d // 3] + d % 3] += eps
            xm[3 * nodes[d // 3] + d % 3] -= eps
            Ep, gp, _ = o.element_local(xp)
            Em, gm, _ = o.element_local(xm)
            gfd[d] = (Ep[e] - Em[e]) / (2 * eps)
            Hfd[:, d] = (gp[e] - gm[e]) / (2 * eps)
        assert np.linalg.norm(g[e] - gfd) / np.linalg.norm(gfd) <= 1e-6
        assert np.linalg.norm(H[e] - Hfd) / np.linalg.norm(Hfd) <= 1e-6
        assert np.allclose(H[e], H[e].T, rtol=0, atol=1e-9 * np.abs(H[e]).max())


def test_inverted_element_energy_is_huge():
    m = _small()
    o = oracle.Oracle(m)
    x = o.rest().reshape(-1, 3)
    t = m.T[0]
    x[t[0]] = x[t[1]] + 2 * (x[t[1]] - x[t[0]])  # push node 0 through the opposite side
    E, _, _ = o.element_local(x.ravel())
    assert np.isinf(E[0]) and np.isinf(o.energy(x.ravel()))


def test_global_gradient_fd():
    m = _small()
    o = oracle.Oracle(m)
    rng = np.random.default_rng(2)
    x = o.rest() + 1e-3 * rng.standard_normal(o.N)
    g = o.gradient(x, fix=False)
    eps = 1e-6
    for d in range(0, o.N, 5):
        xp = x.copy(); xm = x.copy()
        xp[d] += eps; xm[d] -= eps
        fd = (o.energy(xp) - o.energy(xm)) / (2 * eps)
        assert abs(fd - g[d]) <= 1e-6 * max(1.0, np.abs(g).max())


def test_pattern_is_eigen_lower_with_full_diagonal_blocks():
    m = M.cantilever(2, 2, 3)
    o = oracle.Oracle(m)
    cp, ri = o.pattern()
    E = len(M.unique_edges(m.T))
    assert cp[-1] == 9 * (m.n + E)
    for c in range(o.N):
        rows = ri[cp[c]:cp[c + 1]]
        assert np.all(np.diff(rows) > 0)
        assert rows[0] == 3 * (c // 3)  # the full diagonal block starts the column
        assert np.all(rows >= 3 * (c // 3))


def test_fixed_dofs_in_matrix_and_vector():
    m = M.cantilever(2, 2, 3)
    o = oracle.Oracle(m)
    x = o.rest()
    g = o.gradient(x, fix=True)
    assert np.all(g[m.fixed.astype(bool)] == 0)
    H = o.hessian(x, fix=True)
    cp, ri = o.pattern()
    for c in range(o.N):
        for q in range(cp[c], cp[c + 1]):
            r = ri[q]
            if m.fixed[r] or m.fixed[c]:
                assert H[q] == (1.0 if r == c else 0.0)


def test_small_cantilever_regression():
    gold = np.load(os.path.join(GOLD, "cantilever_small.npz"))
    m = M.cantilever(2, 2, 8)
    o = oracle.Oracle(m)
    x0 = o.rest()
    g0 = np.linalg.norm(o.gradient(x0))
    assert np.isclose(g0, gold["g0"], rtol=1e-14)
    x, rep = o.solve_static(x0, tol_max_error=1e-10 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    assert rep["result_name"] == "SUCCESS"
    assert rel(x - x0, gold["x"] - x0) < 1e-10
    cp, ri = o.pattern()
    assert np.array_equal(cp, gold["colptr"]) and np.array_equal(ri, gold["rowidx"])
    assert np.array_equal(o.scatter_map(), gold["scatter"])


def test_ldlt_and_cg_agree():
    m = M.cantilever(2, 2, 8)
    o = oracle.Oracle(m)
    x0 = o.rest()
    g0 = np.linalg.norm(o.gradient(x0))
    kw = dict(tol_max_error=1e-10 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    xl, rl = o.solve_static(x0, **kw)
    xc, rc = o.solve_static(x0, ls_solver=1, cg_block_jacobi=1, **kw)
    assert rl["result_name"] == rc["result_name"] == "SUCCESS"
    assert rel(xc - x0, xl - x0) < 1e-8


def test_parallel_cg_matches_serial_cg():
    """The row-parallel CG (full rows, blocked inner products) runs the same iteration as the
    serial one in another summation order: the same Newton path to the CG tolerance's scale,
    and the same bits for any thread count."""
    m = M.cantilever(3, 3, 10)
    o = oracle.Oracle(m)
    x0 = o.rest()
    g0 = np.linalg.norm(o.gradient(x0))
    kw = dict(tol_max_error=1e-9 * g0, tol_min_impr=0.0, tol_min_step=0.0, ls_solver=1, ls_tol_max_error=1e-10)
    xs, rs = o.solve_static(x0, **kw)
    xp, rp = o.solve_static(x0, cg_parallel=1, threads=4, **kw)
    xq, rq = o.solve_static(x0, cg_parallel=1, threads=1, **kw)
    assert rs["result_name"] == rp["result_name"] == "SUCCESS"
    assert rel(xp - x0, xs - x0) < 1e-8
    assert abs(rp["lin_iterations"] - rs["lin_iterations"]) <= 0.02 * rs["lin_iterations"] + 2
    assert np.array_equal(xp, xq) and rp["lin_iterations"] == rq["lin_iterations"]


def test_dynamic_step_conserves_at_rest():
    # no load, no velocity: the implicit step must keep the rest state
    m = M.make_box(2, 2, 2, (0.02, 0.02, 0.02), 1e5, 0.3, clamp_face=2)
    o = oracle.Oracle(m)
    x0 = o.rest()
    x, v, rep = o.solve_dynamic(x0, np.zeros(o.N), 1e-3)
    assert rep["result_name"] == "SUCCESS"
    assert np.abs(x - x0).max() == 0 and np.abs(v).max() == 0


def test_dynamic_step_against_explicit_energy():
    m = M.make_box(2, 2, 3, (0.02, 0.02, 0.03), 1e5, 0.3, 1000.0, 0, (0.0, -9.81, 0.0), clamp_face=2)
    o = oracle.Oracle(m)
    x0 = o.rest()
    v0 = np.zeros(o.N)
    v0[1::3] = 0.1
    v0[m.fixed.astype(bool)] = 0
    dt = 1e-3
    x, v, rep = o.solve_dynamic(x0, v0, dt, tol_max_error=1e-12, tol_min_impr=0.0, tol_min_step=0.0)
    assert rep["result_name"] == "SUCCESS"
    # stationarity of the incremental potential: g(x) + M a = 0 on free DoFs
    g = o.gradient(x, fix=True)
    mass = np.zeros(m.n)
    vol = M.signed_volumes(m.X0, m.T)
    for e in range(m.m):
        mass[m.T[e]] += m.rho[e] * vol[e] / 4
    a = (x - x0) / dt ** 2 - v0 / dt
    r = g + np.repeat(mass, 3) * a
    r[m.fixed.astype(bool)] = 0
    assert np.linalg.norm(r) < 1e-9
    assert np.allclose(v, (x - x0) / dt)


def test_soft_fixed_position_fd_and_stiff_limit():
    """BC_FixDoF soft mode (EnergyElement_SoftConstraint): the gradient and the Hessian's
    diagonal term match finite differences of the energy with the reference's eps, and a
    stiff soft clamp approaches the hard clamp's equilibrium."""
    base = M.cantilever(2, 2, 4)
    m = M.soft_clamped(base, 1e6, target_shift=(1e-3, 0.0, -2e-3))
    o = oracle.Oracle(m)
    rng = np.random.default_rng(5)
    x = o.rest() + 1e-3 * rng.standard_normal(o.N)
    g = o.gradient(x, fix=False)
    eps = 1e-6
    soft_dofs = np.flatnonzero(np.repeat(m.soft_k > 0, 3))
    for d in list(soft_dofs[:9]) + [soft_dofs[-1] + 3]:
        xp = x.copy(); xm = x.copy()
        xp[d] += eps; xm[d] -= eps
        fd = (o.energy(xp) - o.energy(xm)) / (2 * eps)
        assert abs(fd - g[d]) <= 1e-6 * max(1.0, np.abs(g).max())
        # the diagonal Hessian entry against the gradient's difference
        cp, ri = o.pattern()
        vals = o.hessian(x, fix=False)
        q = [i for i in range(cp[d], cp[d + 1]) if ri[i] == d][0]
        hfd = (o.gradient(xp, fix=False)[d] - o.gradient(xm, fix=False)[d]) / (2 * eps)
        assert abs(hfd - vals[q]) <= 1e-5 * abs(vals[q])
    # stiff limit: soft clamp with k -> large approaches the hard clamp
    hard = oracle.Oracle(base)
    x0 = hard.rest()
    g0 = np.linalg.norm(hard.gradient(x0))
    xh, rh = hard.solve_static(x0, tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    errs = []
    for k in (1e5, 1e7):
        stiff = oracle.Oracle(M.soft_clamped(base, k))
        xs, rs = stiff.solve_static(x0, tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0)
        assert rh["result_name"] == "SUCCESS" and rs["result_name"] == "SUCCESS"
        errs.append(np.linalg.norm(xs - xh) / np.linalg.norm(xh - x0))
    assert errs[1] < 1e-3 and errs[1] < errs[0] / 50  # the gap closes like 1/k
