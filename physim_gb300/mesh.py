"""Structured tetrahedral box meshes and the synthetic workloads built on them.

The reference meshes a structured hex grid with 5 tets per hex
(source/PhySim/Utils/MeshUtils.cpp:927-991) and leaves the 6-tet split
unimplemented (MeshUtils.cpp:437-439).  The workloads here need 6 tets per
hex, so this module writes its own generator: every hex is cut into the six
Kuhn (Freudenthal) tets that share the hex main diagonal v000 -> v111.  The
split is translation invariant, so neighbouring hexes cut shared faces along
the same diagonal and the mesh is conforming.  Every tet is emitted with a
positive signed volume (det Dm > 0), matching Cell_Tetra::VolumeSpace
(source/PhySim/Geometry/Polytopes/Cell_Tetra.cpp:27-36).

Node numbering is lexicographic with x fastest: node(i, j, k) =
i + (nx+1) * (j + (ny+1) * k).  DoF d of node v is 3*v + d, which is the order
KinematicsTree::Init assigns offsets in (source/PhySim/Kinematics/
KinematicsTree.cpp:25-40) for a mesh of particles.

All random draws come from a counter-based splitmix64 stream keyed by one
seed per workload, so every workload is reproducible bit for bit on any host.
"""
from __future__ import annotations

import dataclasses
import itertools
import math
from typing import List, Optional, Sequence

import numpy as np

MODEL_CONH = 0  # compressible Neo-Hookean (MaterialModels.h:235-299)
MODEL_STVK = 1  # Saint-Venant Kirchhoff (MaterialModels.h:166-230)

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """Vectorised splitmix64 finaliser over uint64 counters (wrapping)."""
    z = np.asarray(x, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


class Stream:
    """Counter-based uniform stream: draw k of stream `key` is splitmix64(key*2^32 + k)."""

    def __init__(self, seed: int, key: int = 0):
        self.base = np.uint64((int(seed) * 0x100000001B3 + int(key) * 0x9E3779B1) & 0xFFFFFFFFFFFFFFFF)
        self.count = 0

    def uniform(self, n: Optional[int] = None) -> np.ndarray | float:
        m = 1 if n is None else int(n)
        ctr = self.base + np.arange(self.count, self.count + m, dtype=np.uint64)
        self.count += m
        u = (splitmix64(ctr) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return float(u[0]) if n is None else u

    def integers(self, lo: int, hi: int, n: Optional[int] = None):
        """Uniform integers in [lo, hi] inclusive."""
        u = self.uniform(n)
        v = np.floor(np.asarray(u) * (hi - lo + 1)).astype(np.int64) + lo
        v = np.minimum(v, hi)
        return int(v) if n is None else v


@dataclasses.dataclass
class Mesh:
    """One FEM volume instance: the inputs of Simulable_FEM + its boundary conditions."""

    X0: np.ndarray            # float64 [n, 3] rest positions
    T: np.ndarray             # int32 [m, 4] tets
    lame: np.ndarray          # float64 [m, 2] (lambda, mu) = (LAME1, LAME2)
    rho: np.ndarray           # float64 [m] density
    model: np.ndarray         # uint8 [m] MODEL_CONH / MODEL_STVK
    fixed: np.ndarray         # uint8 [3n] hard-fixed DoFs (BC_FixDoF hard mode)
    force: np.ndarray         # float64 [3n] EnergyElement_Force f (E = x.f, so f = -F_phys)
    gravity: np.ndarray       # float64 [3]
    dims: tuple = (0, 0, 0)   # hex grid dims when structured
    name: str = ""
    soft_k: np.ndarray = None        # float64 [n] BC_FixDoF soft mode stiffness per node (0: none), or None
    soft_target: np.ndarray = None   # float64 [n, 3] its targets, or None (rest positions)

    @property
    def n(self) -> int:
        return int(self.X0.shape[0])

    @property
    def m(self) -> int:
        return int(self.T.shape[0])

    @property
    def ndof(self) -> int:
        return 3 * self.n

    def copy(self) -> "Mesh":
        return dataclasses.replace(
            self, X0=self.X0.copy(), T=self.T.copy(), lame=self.lame.copy(), rho=self.rho.copy(),
            model=self.model.copy(), fixed=self.fixed.copy(), force=self.force.copy(),
            gravity=self.gravity.copy(),
            soft_k=None if self.soft_k is None else self.soft_k.copy(),
            soft_target=None if self.soft_target is None else self.soft_target.copy())


def lame_from_young_poisson(E, nu):
    """ParameterSet::InitLinearFromYoungPoisson (source/PhySim/Utils/ParameterSet.cpp:54-70)."""
    E = np.asarray(E, dtype=np.float64)
    nu = np.asarray(nu, dtype=np.float64)
    t0 = 1.0 + nu
    t1 = 1.0 - 2.0 * nu
    lam = (E * nu) / (t0 * t1)
    mu = E / (2.0 * t0)
    return lam, mu


def node_index(nx: int, ny: int, nz: int):
    def idx(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)
    return idx


def box_grid(nx: int, ny: int, nz: int, size=(1.0, 1.0, 1.0)):
    """Rest positions and the 6-tet Kuhn tets of an nx x ny x nz hex grid."""
    xs = np.linspace(0.0, size[0], nx + 1)
    ys = np.linspace(0.0, size[1], ny + 1)
    zs = np.linspace(0.0, size[2], nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    X0 = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.float64)

    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i = i.ravel(); j = j.ravel(); k = k.ravel()
    idx = node_index(nx, ny, nz)
    tets = []
    unit = np.eye(3, dtype=np.int64)
    for perm in itertools.permutations(range(3)):
        # path v000 -> +e_p0 -> +e_p1 -> +e_p2 (= v111)
        c0 = np.zeros(3, dtype=np.int64)
        c1 = c0 + unit[perm[0]]
        c2 = c1 + unit[perm[1]]
        c3 = c2 + unit[perm[2]]
        corners = [c0, c1, c2, c3]
        sign = np.linalg.det(np.stack([c1 - c0, c2 - c0, c3 - c0], axis=1).astype(np.float64))
        if sign < 0:
            corners = [c0, c1, c3, c2]
        tets.append(np.stack([idx(i + c[0], j + c[1], k + c[2]) for c in corners], axis=1))
    # hex-major order: the six tets of one hex are consecutive
    T = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return X0, T


def face_nodes(nx, ny, nz, face: int) -> np.ndarray:
    """Node ids on one box face. face = 2*axis + side (side 0 = min, 1 = max)."""
    axis, side = divmod(face, 2)
    dims = (nx, ny, nz)
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coord = (i, j, k)[axis]
    sel = coord.ravel() == (0 if side == 0 else dims[axis])
    return np.nonzero(sel)[0].astype(np.int64)


def face_triangles(nx, ny, nz, face: int) -> np.ndarray:
    """Boundary triangles [nt, 3] of one box face, cut like the Kuhn tets cut it."""
    axis, side = divmod(face, 2)
    dims = (nx, ny, nz)
    a1, a2 = [a for a in range(3) if a != axis]
    idx = node_index(nx, ny, nz)
    fix = 0 if side == 0 else dims[axis]
    u, v = np.meshgrid(np.arange(dims[a1]), np.arange(dims[a2]), indexing="ij")
    u = u.ravel(); v = v.ravel()

    def node(du, dv):
        c = [None, None, None]
        c[axis] = np.full_like(u, fix)
        c[a1] = u + du
        c[a2] = v + dv
        return idx(c[0], c[1], c[2])

    n00, n10, n01, n11 = node(0, 0), node(1, 0), node(0, 1), node(1, 1)
    # Kuhn tets cut every face along its (0,0)-(1,1) diagonal
    t1 = np.stack([n00, n10, n11], axis=1)
    t2 = np.stack([n00, n11, n01], axis=1)
    return np.concatenate([t1, t2], axis=0)


def traction_forces(X0, tris, traction) -> np.ndarray:
    """Lump a uniform traction t onto nodes: each triangle adds area*t/3 to its 3 nodes.

    The reference has no traction condition; nodal loads enter through
    EnergyElement_Force (source/PhySim/Elements/EnergyElement_Force.cpp:43-56)
    whose energy is x.f, so the returned f is minus the physical nodal force.
    """
    n = X0.shape[0]
    F = np.zeros((n, 3), dtype=np.float64)
    p0 = X0[tris[:, 0]]; p1 = X0[tris[:, 1]]; p2 = X0[tris[:, 2]]
    area = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0), axis=1)
    contrib = (area / 3.0)[:, None] * np.asarray(traction, dtype=np.float64)[None, :]
    for c in range(3):
        np.add.at(F, tris[:, c], contrib)
    return -F.ravel()


def make_box(nx, ny, nz, size, E, nu, rho=1000.0, model=MODEL_CONH, gravity=(0.0, 0.0, 0.0),
             clamp_face: Optional[int] = 4, load_face: Optional[int] = None, traction=None,
             name="") -> Mesh:
    X0, T = box_grid(nx, ny, nz, size)
    m = T.shape[0]
    E = np.broadcast_to(np.asarray(E, dtype=np.float64), (m,)).copy()
    nu = np.broadcast_to(np.asarray(nu, dtype=np.float64), (m,)).copy()
    lam, mu = lame_from_young_poisson(E, nu)
    fixed = np.zeros(3 * X0.shape[0], dtype=np.uint8)
    if clamp_face is not None:
        fn = face_nodes(nx, ny, nz, clamp_face)
        fixed[3 * fn] = 1; fixed[3 * fn + 1] = 1; fixed[3 * fn + 2] = 1
    force = np.zeros(3 * X0.shape[0], dtype=np.float64)
    if load_face is not None and traction is not None:
        force = traction_forces(X0, face_triangles(nx, ny, nz, load_face), traction)
    return Mesh(X0=X0, T=T, lame=np.stack([lam, mu], axis=1), rho=np.full(m, float(rho)),
                model=np.full(m, model, dtype=np.uint8), fixed=fixed, force=force,
                gravity=np.asarray(gravity, dtype=np.float64), dims=(nx, ny, nz), name=name)


# ---------------------------------------------------------------------------
# The five synthetic workloads
# ---------------------------------------------------------------------------

CANTILEVER_SIZE = (0.1, 0.1, 0.4)
GRAVITY_Y = (0.0, -9.81, 0.0)


def cantilever(nx=8, ny=8, nz=32, E=1e5, nu=0.3, rho=1000.0, seed: Optional[int] = None) -> Mesh:
    """Neo-Hookean cantilever: box 0.1 x 0.1 x 0.4 m, z = 0 clamped, gravity along -y.

    With seed=None, E is uniform (the 8x8x32 case); with a seed, per-element E is
    drawn log-uniform in [1e4, 1e6] Pa (the 48x48x192 case).
    """
    m = 6 * nx * ny * nz
    if seed is not None:
        s = Stream(seed, key=2)
        E = 10.0 ** (4.0 + 2.0 * s.uniform(m))
    return make_box(nx, ny, nz, CANTILEVER_SIZE, E, nu, rho, MODEL_CONH, GRAVITY_Y,
                    clamp_face=4, name=f"cantilever_{nx}x{ny}x{nz}")


def unit_direction(s: Stream) -> np.ndarray:
    z = 2.0 * s.uniform() - 1.0
    phi = 2.0 * math.pi * s.uniform()
    r = math.sqrt(max(0.0, 1.0 - z * z))
    return np.array([r * math.cos(phi), r * math.sin(phi), z])


def batch_instance(seed: int, index: int, h: float = 0.01) -> Mesh:
    """One instance of the batched uneven workload (512 boxes, hex edge 1 cm)."""
    s = Stream(seed, key=1000 + index)
    nx = s.integers(3, 12); ny = s.integers(3, 12); nz = s.integers(6, 48)
    model = MODEL_CONH if s.uniform() < 0.5 else MODEL_STVK
    E = 10.0 ** (4.0 + 2.0 * s.uniform())
    nu = 0.2 + 0.25 * s.uniform()
    clamp = s.integers(0, 5)
    load = clamp ^ 1  # opposite face
    tmag = 1e2 + 9e2 * s.uniform()
    t = tmag * unit_direction(s)
    return make_box(nx, ny, nz, (nx * h, ny * h, nz * h), E, nu, 1000.0, model, (0.0, 0.0, 0.0),
                    clamp_face=clamp, load_face=load, traction=t,
                    name=f"batch{index}_{nx}x{ny}x{nz}")


def batch_workload(count: int = 512, seed: int = 3) -> List[Mesh]:
    return [batch_instance(seed, i) for i in range(count)]


def serving_request(seed: int, index: int) -> Mesh:
    """One request of the serving stream: 1:1:4 box with tet count log-uniform in [1e3, 2e5]."""
    s = Stream(seed, key=5000 + index)
    T = 10.0 ** (3.0 + (math.log10(2e5) - 3.0) * s.uniform())
    n = max(2, int(round((T / 24.0) ** (1.0 / 3.0))))
    E = 10.0 ** (4.0 + 2.0 * s.uniform())
    face = [0, 1, 2, 3, 5][s.integers(0, 4)]  # any face but the clamped z = 0
    t = (1e3 * s.uniform()) * unit_direction(s)
    return make_box(n, n, 4 * n, CANTILEVER_SIZE, E, 0.3, 1000.0, MODEL_CONH, GRAVITY_Y,
                    clamp_face=4, load_face=face, traction=t, name=f"req{index}_{n}x{n}x{4*n}")


def perturb_load(mesh: Mesh, seed: int, index: int, amount: float = 0.1) -> Mesh:
    """Warm re-solve: the same instance with its nodal load scaled by up to +-amount."""
    s = Stream(seed, key=9000 + index)
    out = mesh.copy()
    out.force = mesh.force * (1.0 + amount * (2.0 * s.uniform() - 1.0))
    out.gravity = mesh.gravity * (1.0 + amount * (2.0 * s.uniform() - 1.0))
    return out


def slab_block(seed: int, index: int, n: int = 32, L: float = 0.32) -> Mesh:
    """Near-incompressible block for implicit dynamics: 4-cell slabs alternating 1e4 / 1e8 Pa."""
    s = Stream(seed, key=7000 + index)
    axis = s.integers(0, 2)
    mesh = make_box(n, n, n, (L, L, L), 1.0, 0.495, 1000.0, MODEL_CONH, GRAVITY_Y,
                    clamp_face=2, name=f"slab{index}_{n}^3_axis{axis}")
    hexes = np.arange(n * n * n)
    hi = hexes % n; hj = (hexes // n) % n; hk = hexes // (n * n)
    cell = (hi, hj, hk)[axis]
    E_hex = np.where((cell // 4) % 2 == 0, 1e4, 1e8)
    E = np.repeat(E_hex, 6)
    lam, mu = lame_from_young_poisson(E, 0.495)
    mesh.lame = np.stack([lam, mu], axis=1)
    return mesh


def slab_initial_velocity(mesh: Mesh, L: float = 0.32) -> np.ndarray:
    v = np.zeros((mesh.n, 3))
    v[:, 1] = 0.5 * np.sin(math.pi * mesh.X0[:, 0] / L)
    v = v.ravel()
    v[mesh.fixed.astype(bool)] = 0.0
    return v


def unique_edges(T: np.ndarray) -> np.ndarray:
    pairs = np.concatenate([T[:, [a, b]] for a, b in itertools.combinations(range(4), 2)], axis=0)
    pairs = np.sort(pairs, axis=1).astype(np.int64)
    key = np.unique(pairs[:, 0] * (int(T.max()) + 1) + pairs[:, 1])
    return key


def signed_volumes(X, T) -> np.ndarray:
    p0 = X[T[:, 0]]
    d = np.stack([X[T[:, 1]] - p0, X[T[:, 2]] - p0, X[T[:, 3]] - p0], axis=2)
    return np.linalg.det(d) / 6.0


def soft_clamped(m: Mesh, k: float, target_shift=(0.0, 0.0, 0.0)) -> Mesh:
    """The mesh with its hard-fixed nodes held instead by soft fixed-position conditions of
    stiffness k (BC_FixDoF soft mode), targets at their rest positions plus target_shift."""
    out = m.copy()
    fixed_nodes = m.fixed.reshape(-1, 3).any(axis=1)
    out.fixed = np.zeros_like(m.fixed)
    out.soft_k = np.where(fixed_nodes, float(k), 0.0)
    out.soft_target = m.X0 + np.where(fixed_nodes[:, None], np.asarray(target_shift, dtype=np.float64), 0.0)
    return out



def renumbered(m: Mesh, seed: int) -> Mesh:
    """The same mesh with unstructured numbering: nodes renumbered, tets reordered and each
    tet's corners rotated by an even permutation (orientation kept), all from the seed."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(m.n)          # new id of old node v
    inv = np.argsort(perm)               # old id of new node
    order = rng.permutation(m.m)
    even = np.array([[0, 1, 2, 3], [1, 2, 0, 3], [2, 0, 1, 3], [0, 2, 3, 1], [0, 3, 1, 2], [1, 0, 3, 2],
                     [2, 3, 0, 1], [3, 2, 1, 0], [1, 3, 2, 0], [3, 0, 2, 1], [2, 1, 3, 0], [3, 1, 0, 2]])
    T = perm[m.T[order]]
    T = np.take_along_axis(T, even[rng.integers(0, 12, m.m)], axis=1).astype(np.int32)
    out = m.copy()
    out.X0 = m.X0[inv].copy()
    out.T = T
    out.lame = m.lame[order].copy()
    out.rho = m.rho[order].copy()
    out.model = m.model[order].copy()
    out.fixed = m.fixed.reshape(-1, 3)[inv].ravel().copy()
    out.force = m.force.reshape(-1, 3)[inv].ravel().copy()
    if m.soft_k is not None:
        out.soft_k = m.soft_k[inv].copy()
    if m.soft_target is not None:
        out.soft_target = m.soft_target[inv].copy()
    return out
