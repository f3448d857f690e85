"""Regenerates the golden vectors under tests/golden/.

material_golden.npz: psi, P = dpsi/dF and dP/dF of the reference's own
generated material code (include/PhySim/Utils/Auto/FEMVol_{CoNH,StVK}_
{Energy,Gradient,Hessian}.mcg), compiled by oracle/build.py into
oracle/_ref/libref_mcg.so, on seeded deformation gradients (column-major
Fv, as MaterialModel_3Din3D_* vectorises F).  Needs the reference tree, so it
only runs where the reference is present; the committed file is what the
tests read.

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


if __name__ == "__main__":
    oracle.build.build_all()
    material_golden()
    cantilever_golden()
    print("wrote", os.listdir(HERE))
