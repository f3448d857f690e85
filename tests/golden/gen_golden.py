"""Regenerates the golden vectors under tests/golden/.

material_golden.npz: psi, P = dpsi/dF and dP/dF of the reference's own
generated material code (include/PhySim/Utils/Auto/FEMVol_{CoNH,StVK}_
{Energy,Gradient,Hessian}.mcg), compiled by oracle/build.py into
oracle/_ref/libref_mcg.so, on seeded deformation gradients (column-major
Fv, as MaterialModel_3Din3D_* vectorises F).  Needs the reference tree, so it
only runs where the reference is present; the committed file is what the
tests read.

material_extreme_golden.npz: the same code at strong compression, strong stretch,
within 1e-6 of the identity, and I + N(0, 1), 40 of each per model.

cantilever_small.npz: the oracle's converged static solve of a 2x2x8
Neo-Hookean cantilever (LDLT Newton to ||g||/||g0|| < 1e-10), its Hessian
pattern and scatter map -- a regression fixture for the oracle itself.

Usage: python tests/golden/gen_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from physim_gb300 import mesh as M  # noqa: E402


def material_golden(count=200, seed=20240611):
    R = oracle.ref_lib()
    if R is None:
        raise SystemExit("reference sources not present: cannot regenerate material_golden.npz")
    rng = np.random.default_rng(seed)
    out = {}
    for model, fn, name in ((0, R.ref_conh, "conh"), (1, R.ref_stvk, "stvk")):
        Fs, lams, mus, psis, Ps, Ds = [], [], [], [], [], []
        for k in range(count):
            scale = [0.02, 0.2, 0.6][k % 3]
            F = np.eye(3) + scale * rng.standard_normal((3, 3))
            if np.linalg.det(F) <= 0:
                F[:, 0] *= -1.0
            Fv = np.ascontiguousarray(F.T.ravel())  # column-major
            lam = 10.0 ** rng.uniform(3, 7)
            mu = 10.0 ** rng.uniform(3, 7)
            U = np.zeros(1); P = np.zeros(9); H = np.zeros(81)
            fn(lam, mu, Fv.ctypes.data, U.ctypes.data, P.ctypes.data, H.ctypes.data)
            Fs.append(Fv); lams.append(lam); mus.append(mu); psis.append(U[0]); Ps.append(P); Ds.append(H)
        out[f"{name}_F"] = np.array(Fs)
        out[f"{name}_lame"] = np.stack([lams, mus], axis=1)
        out[f"{name}_psi"] = np.array(psis)
        out[f"{name}_P"] = np.array(Ps)
        out[f"{name}_dPdF"] = np.array(Ds).reshape(-1, 9, 9)
    np.savez_compressed(os.path.join(HERE, "material_golden.npz"), **out)


def cantilever_golden():
    m = M.cantilever(2, 2, 8)
    o = oracle.Oracle(m)
    x0 = o.rest()
    g0 = np.linalg.norm(o.gradient(x0))
    x, rep = o.solve_static(x0, tol_max_error=1e-10 * g0, tol_min_impr=0.0, tol_min_step=0.0)
    cp, ri = o.pattern()
    np.savez_compressed(os.path.join(HERE, "cantilever_small.npz"), x=x, obj=rep["obj"], opt=rep["opt"],
                        iterations=rep["iterations"], colptr=cp, rowidx=ri, scatter=o.scatter_map(),
                        g0=g0)


def material_extreme_golden(per_kind=40, seed=20261204):
    """The reference's material code at four kinds of deformation gradient: strong
    compression (singular values 1e-2..1), strong stretch (1..10^1.5), within 1e-6 of the
    identity, and I + N(0, 1) -- each with a random rotation on both sides."""
    R = oracle.ref_lib()
    if R is None:
        raise SystemExit("reference sources not present: cannot regenerate material_extreme_golden.npz")
    rng = np.random.default_rng(seed)
    out = {}
    for fn, name in ((R.ref_conh, "conh"), (R.ref_stvk, "stvk")):
        Fs, lames, kinds, psis, Ps, Ds = [], [], [], [], [], []
        for kind in range(4):
            for _ in range(per_kind):
                if kind < 2:
                    U, _ = np.linalg.qr(rng.standard_normal((3, 3)))
                    V, _ = np.linalg.qr(rng.standard_normal((3, 3)))
                    s = 10.0 ** (rng.uniform(-2, 0, 3) if kind == 0 else rng.uniform(0, 1.5, 3))
                    F = U @ np.diag(s) @ V.T
                elif kind == 2:
                    F = np.eye(3) + 1e-6 * rng.standard_normal((3, 3))
                else:
                    F = np.eye(3) + rng.standard_normal((3, 3))
                if np.linalg.det(F) <= 0:
                    F[:, 0] *= -1.0
                Fv = np.ascontiguousarray(F.T.ravel())  # column-major
                lam, mu = 10.0 ** rng.uniform(3, 7), 10.0 ** rng.uniform(3, 7)
                U1 = np.zeros(1); P = np.zeros(9); H = np.zeros(81)
                fn(lam, mu, Fv.ctypes.data, U1.ctypes.data, P.ctypes.data, H.ctypes.data)
                Fs.append(Fv); lames.append((lam, mu)); kinds.append(kind)
                psis.append(U1[0]); Ps.append(P); Ds.append(H)
        out[f"{name}_F"] = np.array(Fs)
        out[f"{name}_lame"] = np.array(lames)
        out[f"{name}_kind"] = np.array(kinds, dtype=np.int8)
        out[f"{name}_psi"] = np.array(psis)
        out[f"{name}_P"] = np.array(Ps)
        out[f"{name}_dPdF"] = np.array(Ds).reshape(-1, 9, 9)
    np.savez_compressed(os.path.join(HERE, "material_extreme_golden.npz"), **out)


if __name__ == "__main__":
    # python tests/golden/gen_golden.py [material cantilever extreme]  (default: all)
    oracle.build.build_all()
    which = set(sys.argv[1:]) or {"material", "cantilever", "extreme"}
    if "material" in which:
        material_golden()
    if "cantilever" in which:
        cantilever_golden()
    if "extreme" in which:
        material_extreme_golden()
    print("wrote", os.listdir(HERE))
