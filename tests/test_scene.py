"""Scene files in the reference's XML vocabulary, with TetGen volume meshes (host only).

The loader (physim_gb300/csrc/scene.cpp) reads the elements of the reference's per-component
loaders (source/PhySim/Utils/Serializer_XML.cpp): LoadSimulable_VolumeFEM, LoadOptimProblem,
LoadOptimSolver and LoadBoundary.  Each test writes a scene and its .node/.ele files and pins
one part of what the loader must produce, from the reference's definitions: the Lame
parameters of InitLinearFromYoungPoisson, the mesh transform of LoadMesh_TetVolume, the
distributions' element maps, the selections of the geometry filters, the animators' targets.
"""
import os

import numpy as np
import pytest

import physim_gb300 as px
from physim_gb300 import mesh as M


def write_tetgen(base, X, T, first=1, flip=()):
    with open(base + ".node", "w") as f:
        f.write("# nodes written by the test\n")
        f.write(f"{len(X)} 3 1 1\n")
        for k, p in enumerate(X):
            f.write(f"{k + first}  {p[0]:.17g} {p[1]:.17g} {p[2]:.17g}  0.5  0\n")
    with open(base + ".ele", "w") as f:
        f.write(f"{len(T)} 4 0\n")
        for e, t in enumerate(T):
            t = list(t)
            if e in flip:
                t[1], t[2] = t[2], t[1]
            f.write(f"{e + first} " + " ".join(str(v + first) for v in t) + "\n")


SIM = """<simulable type="VolumeFEM">
    <meshInit type="FILEVOLUME" path="{mesh}">{tf}</meshInit>{rest}
    <discretization type="TET4"/>
    <shapeFunction type="CONSTANT"><shapeFunction type="TET_LIN"/></shapeFunction>
    <quadrature type="CONSTANT"><quadrature type="TET_1"/></quadrature>
    {model}
    {param}
  </simulable>"""
CONH = '<materialModel type="CONSTANT"><materialModel type="CONH" dimSpace="3" dimBasis="3"/></materialModel>'
PARAM = ('<materialParam type="CONSTANT"><materialParam><parameter name="YOUNG" value="{E}"/>'
         '<parameter name="POISSON" value="{nu}"/><parameter name="DENSITY" value="{rho}"/></materialParam></materialParam>')


def scene_xml(mesh="bar", tf="", rest="", model=CONH, param=None, problem='<problem type="Static"/>', solver="",
              boundary=""):
    param = param or PARAM.format(E=1e5, nu=0.3, rho=1000)
    return ("<?xml version='1.0'?>\n<!-- a scene -->\n<scene>\n  " +
            SIM.format(mesh=mesh, tf=tf, rest=rest, model=model, param=param) +
            f"\n  {problem}\n  {solver}\n  <boundary>{boundary}</boundary>\n</scene>\n")


def load(tmp_path, xml, m=None, name="bar", **kw):
    if m is not None:
        write_tetgen(os.path.join(tmp_path, name), m.X0, m.T, **kw)
    p = os.path.join(tmp_path, "scene.xml")
    with open(p, "w") as f:
        f.write(xml)
    return px.Scene(p)


CLAMP = ('<bc type="FixPosition" soft="false"><selection type="BoxNodes" field="Pos0">'
         '<minCorner>-1e-9, -1e-9, -1e-9</minCorner><maxCorner>1, 1, 1e-9</maxCorner></selection></bc>')
GRAV = '<bc type="Gravity"><gravity>0.0, -9.81, 0.0</gravity></bc>'


def test_cantilever_scene_gives_the_generator_mesh(tmp_path):
    ref = M.cantilever(2, 2, 4)
    sc = load(tmp_path, scene_xml(boundary=CLAMP + GRAV), ref)
    m, x = sc.mesh()
    assert sc.info() == {"nodes": ref.n, "tets": ref.m, "dynamic": False, "dt": 0.0, "groups": 0, "num_stages": 1,
                         "reoriented": 0}
    assert np.array_equal(m.X0, ref.X0) and np.array_equal(m.T, ref.T) and np.array_equal(x, ref.X0.ravel())
    # ParameterSet::InitLinearFromYoungPoisson (ParameterSet.cpp:54-70)
    assert np.allclose(m.lame, ref.lame, rtol=1e-15, atol=0) and np.all(m.rho == 1000.0)
    assert np.all(m.model == M.MODEL_CONH)
    assert np.array_equal(m.fixed, ref.fixed)
    assert np.array_equal(m.gravity, [0.0, -9.81, 0.0])
    o = sc.options()
    d = px.options()
    assert (o.num_max_iters, o.tol_max_error, o.lsearch_type, o.qp_solver) == \
        (d.num_max_iters, d.tol_max_error, d.lsearch_type, d.qp_solver)


def test_gravity_default_and_solver_attributes(tmp_path):
    ref = M.cantilever(1, 1, 2)
    solver = ('<solver maxIters="37" maxError="1e-7" qpStep="Steepest"><linear type="EigenCG" maxIters="500" '
              'maxError="1e-10"/><lsearch type="WolfeStrong" iters="20" alpha="0.6" wolfe1="0.001" wolfe2="0.8"/>'
              '</solver>')
    sc = load(tmp_path, scene_xml(solver=solver, boundary='<bc type="Gravity"/>',
                                  problem='<problem type="Dynamic" step="0.002"/>'), ref)
    m, _ = sc.mesh()
    assert np.array_equal(m.gravity, [0.0, -9.8, 0.0])  # BC_Gravity's default acceleration
    info = sc.info()
    assert info["dynamic"] and info["dt"] == 0.002
    o = sc.options()
    assert (o.num_max_iters, o.tol_max_error, o.qp_solver) == (37, 1e-7, 0)
    assert (o.ls_num_max_iters, o.ls_tol_max_error) == (500, 1e-10)
    assert (o.lsearch_type, o.lsearch_num_try, o.lsearch_alpha) == (4, 20, 0.6)
    assert (o.lsearch_wolfe1, o.lsearch_wolfe2) == (0.001, 0.8)


def test_zero_based_indices_and_reoriented_tets(tmp_path):
    ref = M.cantilever(2, 1, 2)
    sc = load(tmp_path, scene_xml(), ref, first=0, flip=(0, 3, 5))
    m, _ = sc.mesh()
    assert sc.info()["reoriented"] == 3
    assert np.array_equal(m.T, ref.T)  # flipped back to positive volumes
    assert np.all(M.signed_volumes(m.X0, m.T) > 0)


def test_mesh_transform_and_rest_mesh(tmp_path):
    """LoadMesh_TetVolume: V' = R S V + t, R = Rz Ry Rx from degrees (GeometryUtils.cpp:79-114);
    meshRest gives the rest shape, meshInit the start positions."""
    ref = M.cantilever(1, 1, 3)
    write_tetgen(os.path.join(tmp_path, "rest"), ref.X0, ref.T)
    tf = "<position>1, 2, 3</position><scale>2, 1, 0.5</scale><rotation>10, 20, 30</rotation>"
    rest = '\n    <meshRest type="FILEVOLUME" path="rest"/>'
    sc = load(tmp_path, scene_xml(tf=tf, rest=rest), ref)
    m, x = sc.mesh()
    a = np.deg2rad([10.0, 20.0, 30.0])
    Rx = np.array([[1, 0, 0], [0, np.cos(a[0]), -np.sin(a[0])], [0, np.sin(a[0]), np.cos(a[0])]])
    Ry = np.array([[np.cos(a[1]), 0, np.sin(a[1])], [0, 1, 0], [-np.sin(a[1]), 0, np.cos(a[1])]])
    Rz = np.array([[np.cos(a[2]), -np.sin(a[2]), 0], [np.sin(a[2]), np.cos(a[2]), 0], [0, 0, 1]])
    want = (Rz @ Ry @ Rx @ np.diag([2.0, 1.0, 0.5]) @ ref.X0.T).T + [1.0, 2.0, 3.0]
    assert np.allclose(x.reshape(-1, 3), want, rtol=0, atol=1e-14)
    assert np.array_equal(m.X0, ref.X0)


def test_variable_distributions(tmp_path):
    """VARIABLE distributions map each element to one of their objects (DomainDistribution_Variable)."""
    ref = M.cantilever(1, 1, 2)
    dist = ", ".join(str(e % 2) for e in range(ref.m))
    model = ('<materialModel type="VARIABLE"><materialModel type="CONH" dimSpace="3" dimBasis="3"/>'
             '<materialModel type="STVK" dimSpace="3" dimBasis="3"/><distribution>' + dist + '</distribution>'
             '</materialModel>')
    param = ('<materialParam type="VARIABLE"><materialParam><parameter name="LAME1" value="100"/>'
             '<parameter name="LAME2" value="50"/><parameter name="DENSITY" value="900"/></materialParam>'
             '<materialParam><parameter name="YOUNG" value="2e5"/><parameter name="POISSON" value="0.25"/>'
             '<parameter name="DENSITY" value="1100"/></materialParam><distribution>' + dist + '</distribution>'
             '</materialParam>')
    sc = load(tmp_path, scene_xml(model=model, param=param), ref)
    m, _ = sc.mesh()
    assert np.array_equal(m.model, np.arange(ref.m) % 2)
    lam1, mu1 = M.lame_from_young_poisson(2e5, 0.25)
    for e in range(ref.m):
        want = (100.0, 50.0, 900.0) if e % 2 == 0 else (lam1, mu1, 1100.0)
        assert np.allclose([m.lame[e, 0], m.lame[e, 1], m.rho[e]], want, rtol=1e-15)


def test_selections(tmp_path):
    ref = M.make_box(2, 2, 2, (1.0, 1.0, 1.0), 1e5, 0.3)
    interior = np.where(np.all(np.isclose(ref.X0, 0.5), axis=1))[0]
    cases = {
        '<selection type="AllNodes"/>': np.arange(ref.n),
        '<selection type="BoundaryNodes"/>': np.setdiff1d(np.arange(ref.n), interior),
        '<selection type="IndexNodes"><indices>3, 5, 7</indices></selection>': np.array([3, 5, 7]),
        ('<selection type="BoxNodes" field="PosX"><minCorner>0.4, -1, -1</minCorner>'
         '<maxCorner>2, 2, 0.6</maxCorner></selection>'):
            np.where((ref.X0[:, 0] >= 0.4) & (ref.X0[:, 2] <= 0.6))[0],
    }
    for sel, nodes in cases.items():
        sc = load(tmp_path, scene_xml(boundary=f'<bc type="FixPosition" soft="false">{sel}</bc>'), ref)
        m, _ = sc.mesh()
        want = np.zeros(ref.n, dtype=np.uint8)
        want[nodes] = 1
        assert np.array_equal(m.fixed.reshape(-1, 3), np.repeat(want[:, None], 3, axis=1)), sel


def test_soft_clamp_and_staged_animation(tmp_path):
    """Soft FixPosition: BC_FixDoF soft mode at its default stiffness 1e9, targets at the start
    positions.  Transform3D animation over numStep stages: VectorAnimator_LerpT3D holds R S and
    t (R from radians here), and a stage applies a t + (I + a R S) v.  A gravity condition with
    numStep 6 sets the stage count."""
    ref = M.cantilever(2, 2, 3)
    anim = ('<animation type="Transform3D"><position>0.01, 0, 0</position><rotation>0, 0, 0.2</rotation>'
            '<scale>1, 1, 1</scale></animation>')
    bc = ('<bc type="FixPosition" soft="true" numStep="4"><selection type="BoxNodes" field="Pos0">'
          '<minCorner>-1e-9, -1e-9, -1e-9</minCorner><maxCorner>1, 1, 1e-9</maxCorner></selection>' + anim + '</bc>'
          '<bc type="Gravity" numStep="6"/>')
    sc = load(tmp_path, scene_xml(boundary=bc), ref)
    m, x = sc.mesh()
    clamp = np.where(ref.fixed.reshape(-1, 3).all(axis=1))[0]
    assert not m.fixed.any()
    assert np.array_equal(np.where(m.soft_k > 0)[0], clamp) and np.all(m.soft_k[clamp] == 1e9)
    assert np.array_equal(m.soft_target.reshape(-1, 3), x.reshape(-1, 3))
    info = sc.info()
    assert info["groups"] == 1 and info["num_stages"] == 6
    (g,) = sc.staging()
    c, s = np.cos(0.2), np.sin(0.2)
    assert g["num_stages"] == 4 and g["soft"] == 1 and g["k_start"] == g["k_end"] == 1e9
    assert np.allclose(g["move"], [[c, -s, 0], [s, c, 0], [0, 0, 1]], rtol=0, atol=1e-16)
    assert np.array_equal(g["shift"], [0.01, 0.0, 0.0]) and np.array_equal(g["nodes"], clamp)


@pytest.mark.parametrize("xml,msg", [
    (scene_xml().replace('"TET4"', '"TET10"'), "discretization TET10"),
    (scene_xml().replace('type="FILEVOLUME" path="bar"', 'type="FILESURFACE" path="bar.obj"'), "FILESURFACE"),
    (scene_xml(boundary='<bc type="CollPlane" soft="true"/>'), "CollPlane"),
    (scene_xml(boundary='<bc type="Force"/>'), "creates no condition"),
    (scene_xml(model=CONH.replace('"CONH"', '"COMR"')), "COMR"),
    (scene_xml().replace("<quadrature type=\"TET_1\"/>", "<quadrature type=\"TET_4\"/>"), "TET_4"),
    (scene_xml().replace("</scene>", ""), "not closed"),
    (scene_xml().replace('<discretization type="TET4"/>', ""), "discretization"),
    (scene_xml(param='<materialParam type="CONSTANT"><materialParam><parameter name="YOUNG" value="1"/>'
                     '</materialParam></materialParam>'), "YOUNG, POISSON and DENSITY"),
])
def test_refusals(tmp_path, xml, msg):
    ref = M.cantilever(1, 1, 2)
    with pytest.raises(px.PhxError) as ei:
        load(tmp_path, xml, ref)
    assert ei.value.code == px.PHX_EINVAL and msg in str(ei.value)


def test_ten_node_tets_refused(tmp_path):
    ref = M.cantilever(1, 1, 2)
    base = os.path.join(tmp_path, "bar")
    write_tetgen(base, ref.X0, ref.T)
    with open(base + ".ele", "w") as f:
        f.write(f"{ref.m} 10 0\n")
        for e, t in enumerate(ref.T):
            f.write(f"{e + 1} " + " ".join(str(v + 1) for v in list(t) * 3)[: 40] + "\n")
    with pytest.raises(px.PhxError) as ei:
        load(tmp_path, scene_xml())
    assert "10-node" in str(ei.value)
