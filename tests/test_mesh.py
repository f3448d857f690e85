"""Structured 6-tet box meshes and the seeded workloads (host only)."""
import numpy as np

from physim_gb300 import mesh as M


def test_cantilever_counts():
    m = M.cantilever()
    assert (m.n, m.m) == (2673, 12288)
    assert len(M.unique_edges(m.T)) == 16112
    assert m.fixed.sum() == 3 * 81  # z = 0 face clamped


def test_large_counts_without_building_materials():
    X0, T = M.box_grid(48, 48, 192, M.CANTILEVER_SIZE)
    assert (X0.shape[0], T.shape[0]) == (463393, 2654208)


def test_positive_orientation_and_volume():
    for dims in [(1, 1, 1), (3, 4, 5)]:
        X0, T = M.box_grid(*dims, size=(1.0, 2.0, 3.0))
        vol = M.signed_volumes(X0, T)
        assert vol.min() > 0
        assert abs(vol.sum() - 6.0) < 1e-12


def test_conforming_faces():
    # every interior triangle is shared by exactly two tets, boundary ones by one
    X0, T = M.box_grid(3, 2, 2)
    faces = {}
    for t in T:
        for f in ([0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]):
            key = tuple(sorted(t[f]))
            faces[key] = faces.get(key, 0) + 1
    assert set(faces.values()) <= {1, 2}
    nb = sum(1 for v in faces.values() if v == 1)
    assert nb == 2 * 2 * (3 * 2 + 3 * 2 + 2 * 2)  # 2 triangles per boundary quad


def test_traction_total_force():
    t = np.array([10.0, -20.0, 5.0])
    m = M.make_box(3, 4, 5, (0.3, 0.4, 0.5), 1e5, 0.3, load_face=5, traction=t)
    total = -m.force.reshape(-1, 3).sum(0)  # f = -F_phys
    assert np.allclose(total, t * 0.3 * 0.4, rtol=1e-12)


def test_workloads_deterministic():
    a = M.batch_instance(3, 17)
    b = M.batch_instance(3, 17)
    assert a.name == b.name and np.array_equal(a.force, b.force) and np.array_equal(a.lame, b.lame)
    batch = M.batch_workload(512)
    sizes = np.array([x.m for x in batch])
    assert sizes.min() >= 324 and sizes.max() <= 41472
    models = np.array([x.model[0] for x in batch])
    assert 0.4 < models.mean() < 0.6


def test_large_cantilever_material_draw():
    m = M.cantilever(2, 2, 4, seed=11)
    E = m.lame[:, 1] * 2 * 1.3
    assert E.min() >= 1e4 * (1 - 1e-12) and E.max() <= 1e6 * (1 + 1e-12)
    assert len(np.unique(E)) > 10
