"""Host-side driver of the product's Newton state machine (tests only).

The device phases (vector ops, energy/gradient, Hessian + PCG) are emulated
with numpy and the CPU oracle so that physim_gb300/csrc/newton_control.h can
be checked against the oracle's SolveFull without a GPU.
"""
import ctypes as C

import numpy as np
import scipy.sparse as sp

PH_DONE, PH_START, PH_VEC, PH_EVAL, PH_EVAL_DONE, PH_ITER, PH_HESS, PH_JACOBI, PH_LINSETUP, PH_RESID, PH_PCG, \
    PH_ACCUM, PH_LIN_DONE, PH_EVALK, PH_EVALK2 = range(15)
VO_RESTORE, VO_ACCEPT, VO_SAVE, VO_STEEP, VO_TRIAL, VO_VEL, VO_PRED, VO_GCOPY, VO_ZERODX = \
    1, 2, 4, 8, 16, 32, 64, 128, 256
VO_STAGE, VO_GNEW = 1024, 2048
LIN_RUNNING, LIN_CONVERGED, LIN_MAXITER, LIN_BREAKDOWN = range(4)


class NState(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "phase", "next_phase", "vecop", "purpose", "result", "it", "steepest", "min_impr_count",
        "min_step_count", "num_bis", "total_bis", "reg_trial", "total_reg", "sweeps", "total_sweeps",
        "lin_status", "pcg_iter", "pcg_parity", "error", "first_step", "step_result", "nofix", "hess_count", "pad3")] + \
        [("pcg_total", C.c_int64)] + [(n, C.c_double) for n in (
            "obj", "opt", "opt0", "obj_new", "alpha_trial", "factor", "scale", "dx_norm", "b_dot_dx", "E_el",
            "E_eval", "gg_eval", "normA2", "shift", "regT", "bb", "rr64", "rz", "rr", "pq", "alpha", "beta",
            "thr_inner", "thr_final", "tol_eff", "lin_tol", "eta", "opt_prev", "log_step", "dg", "dg_eval")] + \
        [("log_pending", C.c_int32), ("log_count", C.c_int32), ("lsk", C.c_int32), ("pcg_resume", C.c_int32),
         ("ls_a", C.c_double * 8), ("ls_e", C.c_double * 8), ("ls_eel", C.c_double * 8),
         ("stage", C.c_int32), ("iter_staged", C.c_int32),
         ("pcg_slices", C.c_int32), ("pad_sl", C.c_int32)]


class DevOpts(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "qp_solver", "min_step_max_count", "min_impr_max_count", "num_max_iters", "try_steepest",
        "ls_num_max_iters", "ls_num_reg_trials", "lsearch_num_try", "precision", "precond",
        "max_refine_sweeps", "warm_guess", "dynamic", "ls_parallel", "lsearch_type", "pad_o")] + \
        [(n, C.c_double) for n in (
            "tol_max_error", "tol_min_step", "tol_min_impr", "max_step_size", "ls_tol_max_error",
            "lsearch_alpha", "inner_tol", "dt", "tol_rel", "lsearch_wolfe1", "lsearch_wolfe2")] + \
        [("num_stages", C.c_int32), ("stage_values", C.c_int32), ("curv_through", C.c_int32),
         ("pad_cv", C.c_int32)]


def make_opts(**kw):
    o = DevOpts(qp_solver=1, min_step_max_count=3, min_impr_max_count=3, num_max_iters=100, try_steepest=1,
                ls_num_max_iters=1000, ls_num_reg_trials=10, lsearch_num_try=32, precision=0, precond=1,
                max_refine_sweeps=1, warm_guess=1, dynamic=0, tol_max_error=1e-6, tol_min_step=1e-5,
                tol_min_impr=1e-9, max_step_size=1000.0, ls_tol_max_error=1e-9, lsearch_alpha=0.5,
                inner_tol=1e-3, dt=0.0, tol_rel=0.0, lsearch_type=1, lsearch_wolfe1=1e-4, lsearch_wolfe2=0.9)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def block_jacobi(H, n):
    Hd = H.toarray() if H.shape[0] <= 3000 else None
    inv = np.zeros((n, 3, 3))
    for v in range(n):
        B = (Hd[3 * v:3 * v + 3, 3 * v:3 * v + 3] if Hd is not None
             else H[3 * v:3 * v + 3, 3 * v:3 * v + 3].toarray())
        d = np.linalg.det(B)
        inv[v] = np.linalg.inv(B) if d != 0 and np.isfinite(d) else np.eye(3)
    return inv


def pcg(A, b, x, thr, maxit, Minv, eigen=True):
    """The device PCG.  eigen=True (the FP64 path): like Eigen's ConjugateGradient, a
    negative p.q gives a negative step and the iteration goes on; only p.q = 0 or a
    non-finite value stops it."""
    n = Minv.shape[0]
    apply = lambda r: np.einsum("vab,vb->va", Minv, r.reshape(n, 3)).ravel()
    r = b - A @ x
    rr = r @ r
    if rr < thr:
        return x, 0, LIN_CONVERGED
    z = apply(r)
    p = z.copy()
    rz = r @ z
    it = 0
    while it < maxit:
        q = A @ p
        pq = p @ q
        if not (pq > 0 or (eigen and pq < 0)):
            return x, it, LIN_BREAKDOWN
        alpha = rz / pq
        x = x + alpha * p
        r = r - alpha * q
        it += 1
        if r @ r < thr:
            return x, it, LIN_CONVERGED
        z = apply(r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return x, it, LIN_MAXITER


stats = {"evalk": 0}  # PH_EVALK visits of the last run


def stage_values(groups, ini, stage):
    """The staged targets and soft stiffness of every group node at `stage`, as the device's
    stage_node computes them: {node: (target[3], soft, k)}."""
    out = {}
    for g in groups:
        N = int(g.get("num_stages", 1))
        a = min(stage, N) / N
        M = np.asarray(g.get("move", np.zeros((3, 3))), dtype=np.float64).reshape(3, 3)
        b = np.asarray(g.get("shift", np.zeros(3)), dtype=np.float64)
        k0, k1 = float(g.get("k_start", 1e9)), float(g.get("k_end", 1e9))
        for i in g["nodes"]:
            v = ini[3 * i:3 * i + 3]
            t = np.array([a * b[r] + v[r] + a * (M[r, 0] * v[0] + M[r, 1] * v[1] + M[r, 2] * v[2]) for r in range(3)])
            out[int(i)] = (t, int(g.get("soft", 0)), k0 + a * (k1 - k0))
    return out


def run(shim, orc, x0, opts, dynamic=False, v0=None, max_steps=200000, staging=None, stage=0):
    """Drives ctl_advance_c until PH_DONE; returns (x, v, NState).  staging: (groups, x_ini)
    of staged boundary conditions (opts.num_stages and opts.stage_values set by the caller),
    stage: the stage the solve starts from."""
    sizes = (C.c_int * 2)()
    shim.ctl_sizes(sizes)
    assert sizes[0] == C.sizeof(NState) and sizes[1] == C.sizeof(DevOpts), "struct layout mismatch"
    shim.ctl_advance_c.argtypes = [C.POINTER(NState), C.POINTER(DevOpts)]
    m = orc.mesh
    n, N = m.n, 3 * m.n
    cp, ri = orc.pattern()
    fixed = m.fixed.astype(bool)
    mass = np.zeros(m.n)
    vol = np.array([np.linalg.det(np.stack([m.X0[t[c + 1]] - m.X0[t[0]] for c in range(3)], 1)) / 6 for t in m.T])
    for e in range(m.m):
        mass[m.T[e]] += m.rho[e] * vol[e] / 4
    mdof = np.repeat(mass, 3)
    x = x0.copy(); xs = x.copy(); dx = np.zeros(N); g = np.zeros(N); gn = np.zeros(N); dxprev = np.zeros(N)
    v = np.zeros(N) if v0 is None else v0.copy()
    xo = np.zeros(N); vo = np.zeros(N)
    s = NState()
    stats["evalk"] = 0
    s.phase = PH_START
    s.opt0 = -1.0
    s.stage = stage
    soft_k = None if getattr(m, "soft_k", None) is None else np.array(m.soft_k, dtype=np.float64)
    soft_t = None
    if soft_k is not None:
        st0 = getattr(m, "soft_target", None)
        soft_t = np.array(m.X0.ravel() if st0 is None else st0, dtype=np.float64).ravel()
    o = opts
    A = None
    Minv = None
    b = None
    dt = o.dt
    for _ in range(max_steps):
        shim.ctl_advance_c(C.byref(s), C.byref(o))
        ph = s.phase
        if ph == PH_DONE:
            break
        if ph == PH_VEC:
            ops, a = s.vecop, s.alpha_trial
            if ops & VO_PRED:
                xo = x.copy(); vo = v.copy(); x = xo + dt * vo
            if ops & VO_RESTORE:
                x = xs.copy()
            if ops & VO_STAGE:
                groups, ini = staging
                for i, (t, soft, k) in stage_values(groups, ini, s.stage).items():
                    if soft:
                        soft_t[3 * i:3 * i + 3] = t
                        soft_k[i] = k
                    elif not dynamic:
                        dxprev[3 * i:3 * i + 3] += t - x[3 * i:3 * i + 3]
                        x[3 * i:3 * i + 3] = t
                if soft_k is not None:
                    orc.set_soft(soft_k, soft_t)
            if ops & (VO_ACCEPT | VO_GCOPY | VO_GNEW):
                g = gn.copy()
            if ops & VO_ACCEPT:
                dxprev = a * dx
            if ops & VO_SAVE:
                xs = x.copy()
            if ops & VO_ZERODX:
                dx = np.zeros(N)
            if ops & VO_STEEP:
                dx = -g
            if ops & VO_TRIAL:
                x = xs + a * dx
            if ops & VO_VEL:
                v = (x - xo) / dt
            s.phase = s.next_phase
            s.vecop = 0
        elif ph == PH_EVALK:
            # several line-search trials at once: energies only, then the scan
            stats["evalk"] += 1
            for k in range(s.lsk):
                xk = xs + s.ls_a[k] * dx
                E = orc.energy(xk)
                if dynamic:
                    acc = (xk - xo) / dt ** 2 - vo / dt
                    E += dt * dt / 2 * np.sum(acc * mdof * acc)
                s.ls_e[k] = E
            s.phase = PH_EVAL_DONE
        elif ph == PH_EVAL:
            E = orc.energy(x)
            gg = orc.gradient(x, fix=False)
            if dynamic:
                acc = (x - xo) / dt ** 2 - vo / dt
                gg = gg + mdof * acc
                E += dt * dt / 2 * np.sum(acc * mdof * acc)
            gg[fixed] = 0
            gn = gg
            s.E_eval = E
            s.gg_eval = gn @ gn
            s.dg_eval = dx @ gn
            s.phase = PH_EVAL_DONE
        elif ph in (PH_HESS, PH_JACOBI):
            if ph == PH_HESS:
                vals = orc.hessian(x, fix=not dynamic)
                if dynamic:
                    L = sp.csc_matrix((vals, ri, cp), shape=(N, N)).tolil()
                    for i in range(N):
                        L[i, i] = L[i, i] + mdof[i] / dt ** 2
                    Lc = L.tocsc()
                    Lc.sort_indices()
                    Lc = Lc.tocoo()
                    keep = []
                    vals2 = np.array(sp.csc_matrix((vals, ri, cp), shape=(N, N)).toarray()[ri, np.repeat(np.arange(N), np.diff(cp))])
                    vals = vals2 + np.where(ri == np.repeat(np.arange(N), np.diff(cp)), mdof[ri] / dt ** 2, 0.0)
                    cc = np.repeat(np.arange(N), np.diff(cp))
                    fx = fixed[ri] | fixed[cc]
                    vals = np.where(fx, np.where(ri == cc, 1.0, 0.0), vals)
                s.normA2 = float(vals @ vals)
                s.regT = 1e-6 * np.sqrt(s.normA2)
                Lo = sp.csc_matrix((vals, ri, cp), shape=(N, N))
                cc = np.repeat(np.arange(N), np.diff(cp))
                low = sp.csc_matrix((np.where(ri >= cc, vals, 0.0), ri, cp), shape=(N, N))
                A0 = (low + low.T - sp.diags(low.diagonal())).tocsr()
            A = (A0 + s.shift * sp.identity(N)).tocsr()
            Minv = block_jacobi(A, n)
            s.phase = PH_LINSETUP
        elif ph == PH_LINSETUP:
            b = -g
            dx = dxprev.copy() if o.warm_guess else np.zeros(N)
            s.bb = b @ b
            s.thr_final = max(s.lin_tol ** 2 * s.bb, 2.2250738585072014e-308)
            s.sweeps = 0
            s.lin_status = LIN_RUNNING
            if s.bb == 0:
                s.lin_status = LIN_CONVERGED; s.b_dot_dx = 0; s.dx_norm = 0
                s.vecop = VO_ZERODX; s.next_phase = PH_LIN_DONE; s.phase = PH_VEC
            else:
                s.phase = PH_RESID
        elif ph == PH_RESID:
            dx, it, st = pcg(A, b, dx, s.thr_final, o.ls_num_max_iters, Minv, eigen=o.precision == 0)
            s.pcg_total += it
            s.lin_status = st
            s.b_dot_dx = b @ dx
            s.dx_norm = np.linalg.norm(dx)
            s.phase = PH_LIN_DONE
        else:
            raise AssertionError(f"unexpected phase {ph}")
    else:
        raise AssertionError("state machine did not finish")
    return x, v, s
