"""The product's host pattern builder (physim_gb300/csrc/pattern.cpp) against the oracle.

Bit-exact requirements: the lower block pattern (Eigen's stored CSC, expanded
per DoF), and the scatter map of every tet's 10 local node pairs onto it.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from physim_gb300 import mesh as M


def build(shim, m):
    arrs = [np.ascontiguousarray(m.X0, dtype=np.float64).ravel(), np.ascontiguousarray(m.T, dtype=np.int32).ravel(),
            np.ascontiguousarray(m.lame, dtype=np.float64).ravel(), np.ascontiguousarray(m.rho, dtype=np.float64),
            np.ascontiguousarray(m.model, dtype=np.uint8), np.ascontiguousarray(m.fixed, dtype=np.uint8),
            np.ascontiguousarray(m.force, dtype=np.float64), np.ascontiguousarray(m.gravity, dtype=np.float64)]
    shim.pat_build.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 8
    shim.pat_error.restype = C.c_char_p
    rc = shim.pat_build(m.n, m.m, *[a.ctypes.data for a in arrs])
    if rc != 0:
        return None, shim.pat_error().decode()
    sz = np.zeros(5, dtype=np.int64)
    shim.pat_sizes(sz.ctypes.data_as(C.c_void_p))
    n, mm, nlo, nch, nslots = (int(v) for v in sz)
    out = {"n": n, "m": mm, "nlo": nlo, "nchunks": nch, "nslots": nslots}

    def get(name, count, dtype):
        a = np.zeros(count, dtype=dtype)
        getattr(shim, "pat_" + name)(a.ctypes.data_as(C.c_void_p))
        return a

    out["lo_rc"] = get("lo_rc", 2 * nlo, np.int32).reshape(-1, 2)
    out["lo_colptr"] = get("lo_colptr", n + 1, np.int32)
    out["scatter"] = get("scatter", 10 * mm, np.int32).reshape(-1, 10)
    out["seg_ptr"] = get("seg_ptr", nlo + 1, np.int32)
    out["seg_c"] = get("seg_c", 10 * mm, np.int32)
    out["nseg_ptr"] = get("nseg_ptr", n + 1, np.int32)
    out["nseg_c"] = get("nseg_c", 4 * mm, np.int32)
    out["chunk_off"] = get("chunk_off", nch + 1, np.int32)
    out["slot_col"] = get("slot_col", nslots, np.int32)
    out["diag_slot"] = get("diag_slot", n, np.int32)
    out["lo_slot"] = get("lo_slot", nlo, np.int32)
    out["up_slot"] = get("up_slot", nlo, np.int32)
    out["rest64"] = get("rest64", 12 * mm, np.float64).reshape(-1, 12)
    out["mass"] = get("mass", n, np.float64)
    out["hlin"] = get("hlin", 4 * n, np.float64).reshape(-1, 4)
    out["fixmask"] = get("fixmask", n, np.uint8)
    return out, None


def csc_from_blocks(P):
    """Per-DoF lower CSC implied by the block pattern (column-major blocks)."""
    n = P["n"]
    colptr = [0]
    rows = []
    for Cn in range(n):
        ks = range(P["lo_colptr"][Cn], P["lo_colptr"][Cn + 1])
        for b in range(3):
            for k in ks:
                R = P["lo_rc"][k, 0]
                rows.extend([3 * R, 3 * R + 1, 3 * R + 2])
            colptr.append(len(rows))
    return np.array(colptr, dtype=np.int32), np.array(rows, dtype=np.int32)


MESHES = [
    lambda: M.cantilever(3, 2, 5),
    lambda: M.batch_instance(3, 4),
    lambda: M.make_box(1, 1, 1, (1.0, 1.0, 1.0), 1e5, 0.3),
]


@pytest.mark.parametrize("make", MESHES)
def test_pattern_and_scatter_bit_exact(pattern_shim, make):
    m = make()
    P, err = build(pattern_shim, m)
    assert err is None, err
    o = oracle.Oracle(m)
    cp, ri = o.pattern()
    mcp, mri = csc_from_blocks(P)
    assert np.array_equal(cp, mcp) and np.array_equal(ri, mri)
    assert np.array_equal(P["scatter"], o.scatter_map())
    assert P["nlo"] == m.n + len(M.unique_edges(m.T))


@pytest.mark.parametrize("make", MESHES)
def test_segments_and_sell_layout(pattern_shim, make):
    m = make()
    P, _ = build(pattern_shim, m)
    n, nlo = P["n"], P["nlo"]
    # segments: every (tet, pair) exactly once, grouped by target block, element order inside
    assert P["seg_ptr"][-1] == 10 * m.m
    flat = P["scatter"].ravel()
    for k in range(0, nlo, max(1, nlo // 200)):
        seg = P["seg_c"][P["seg_ptr"][k]:P["seg_ptr"][k + 1]]
        assert np.all(flat[seg] == k) and np.all(np.diff(seg) > 0)
    assert np.array_equal(np.sort(P["seg_c"]), np.arange(10 * m.m))
    # node segments
    assert np.array_equal(np.sort(P["nseg_c"]), np.arange(4 * m.m))
    for v in range(0, n, max(1, n // 100)):
        seg = P["nseg_c"][P["nseg_ptr"][v]:P["nseg_ptr"][v + 1]]
        assert np.all(m.T.ravel()[seg] == v) and np.all(np.diff(seg) > 0)
    # SELL: every full block (R,C) and (C,R) lands in a distinct slot of the right row/column
    def slot_row(s):
        chunk = np.searchsorted(P["chunk_off"], s, side="right") - 1
        return chunk * 32 + (s - P["chunk_off"][chunk]) % 32
    used = np.zeros(P["nslots"], dtype=np.int32)
    for k in range(nlo):
        R, Cn = P["lo_rc"][k]
        s = P["lo_slot"][k]
        assert slot_row(s) == R and P["slot_col"][s] == Cn
        used[s] += 1
        if R != Cn:
            u = P["up_slot"][k]
            assert slot_row(u) == Cn and P["slot_col"][u] == R
            used[u] += 1
        else:
            assert P["up_slot"][k] == -1 and P["diag_slot"][R] == s
    assert used.max() == 1 and used.sum() == 2 * nlo - n
    # rows sorted by column within the SELL order
    for v in range(0, n, max(1, n // 50)):
        c = v // 32
        L = (P["chunk_off"][c + 1] - P["chunk_off"][c]) // 32
        cols = [P["slot_col"][P["chunk_off"][c] + k * 32 + v % 32] for k in range(L)]
        real = [col for k, col in enumerate(cols) if used[P["chunk_off"][c] + k * 32 + v % 32]]
        assert real == sorted(real)


def test_rest_data_and_loads(pattern_shim):
    m = M.batch_instance(3, 9)
    P, _ = build(pattern_shim, m)
    vol = M.signed_volumes(m.X0, m.T)
    assert np.allclose(P["rest64"][:, 9], vol, rtol=1e-14)
    for e in range(0, m.m, 97):
        Dm = np.stack([m.X0[m.T[e, c + 1]] - m.X0[m.T[e, 0]] for c in range(3)], axis=1)
        assert np.allclose(P["rest64"][e, :9].reshape(3, 3).T @ Dm, np.eye(3), atol=1e-10)
    mass = np.zeros(m.n)
    for e in range(m.m):
        mass[m.T[e]] += m.rho[e] * vol[e] / 4
    assert np.allclose(P["mass"], mass, rtol=1e-13)
    h = m.force.reshape(-1, 3) - mass[:, None] * m.gravity[None, :]
    assert np.allclose(P["hlin"][:, :3], h, rtol=1e-14, atol=0)
    assert np.array_equal(P["fixmask"], m.fixed.reshape(-1, 3) @ np.array([1, 2, 4]))


def test_rejects_malformed_meshes(pattern_shim):
    base = M.cantilever(2, 1, 2)
    bad = base.copy(); bad.T[3, 1] = base.n + 5
    assert build(pattern_shim, bad)[1].startswith("mesh: node id out of range")
    bad = base.copy(); bad.T[2, [1, 2]] = bad.T[2, [2, 1]]
    assert "non-positive rest volume" in build(pattern_shim, bad)[1]
    bad = base.copy(); bad.T[0, 1] = bad.T[0, 0]
    assert "repeated node" in build(pattern_shim, bad)[1]
    bad = base.copy(); bad.X0 = np.vstack([bad.X0, [[9.0, 9.0, 9.0]]])
    bad.fixed = np.zeros(3 * (base.n + 1), dtype=np.uint8); bad.force = np.zeros(3 * (base.n + 1))
    assert "belongs to no tet" in build(pattern_shim, bad)[1]
    bad = base.copy(); bad.lame[4, 0] = np.nan
    assert "non-finite" in build(pattern_shim, bad)[1]


def _build_soft(shim, m, soft_k, soft_target):
    arrs = [np.ascontiguousarray(m.X0, dtype=np.float64).ravel(), np.ascontiguousarray(m.T, dtype=np.int32).ravel(),
            np.ascontiguousarray(m.lame, dtype=np.float64).ravel(), np.ascontiguousarray(m.rho, dtype=np.float64),
            np.ascontiguousarray(m.model, dtype=np.uint8), np.ascontiguousarray(m.fixed, dtype=np.uint8),
            np.ascontiguousarray(m.force, dtype=np.float64), np.ascontiguousarray(m.gravity, dtype=np.float64)]
    k = None if soft_k is None else np.ascontiguousarray(soft_k, dtype=np.float64)
    t = None if soft_target is None else np.ascontiguousarray(soft_target, dtype=np.float64).ravel()
    shim.pat_build_soft.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 10
    shim.pat_soft_size.restype = C.c_longlong
    shim.pat_error.restype = C.c_char_p
    rc = shim.pat_build_soft(m.n, m.m, *[a.ctypes.data for a in arrs], None if k is None else k.ctypes.data,
                             None if t is None else t.ctypes.data)
    if rc != 0:
        return None, shim.pat_error().decode()
    soft = np.zeros(int(shim.pat_soft_size()))
    shim.pat_soft(soft.ctypes.data_as(C.c_void_p))
    return soft.reshape(-1, 4) if soft.size else soft, ""


def test_soft_fixed_position_records(pattern_shim):
    """BC_FixDoF soft mode: one (target, k) record per node, the target the rest position
    unless given; no records when no node has a stiffness; bad stiffness rejected."""
    m = M.cantilever(2, 2, 3)
    k = np.zeros(m.n)
    k[[0, 5, m.n - 1]] = [10.0, 2.5, 7.0]
    soft, _ = _build_soft(pattern_shim, m, k, None)
    assert soft.shape == (m.n, 4)
    assert np.array_equal(soft[:, 3], k)
    assert np.array_equal(soft[:, :3], m.X0)
    tgt = m.X0 + 0.25
    soft, _ = _build_soft(pattern_shim, m, k, tgt)
    assert np.array_equal(soft[:, :3], tgt)
    soft, _ = _build_soft(pattern_shim, m, np.zeros(m.n), None)
    assert soft.size == 0
    for bad in (-1.0, np.nan, np.inf):
        kb = k.copy()
        kb[3] = bad
        soft, err = _build_soft(pattern_shim, m, kb, None)
        assert soft is None and "soft_k" in err


# (V + E lower blocks, V + 2E full blocks) of the 6-tet hex grids at their full sizes:
# the 8x8x32 cantilever, the 32^3 dynamics block, the 48x48x192 cantilever
FULL_SIZES = [
    ((8, 8, 32), 18785, 34897),
    ((32, 32, 32), 274625, 513313),
    ((48, 48, 192), 3622465, 6781537),
]


@pytest.mark.parametrize("dims,nlo_expect,nfull_expect", FULL_SIZES, ids=["8x8x32", "32^3", "48x48x192"])
def test_full_size_pattern_properties(pattern_shim, dims, nlo_expect, nfull_expect):
    """Size-independent checks of the pattern, scatter map, segments and SELL layout at the
    workloads' full sizes (the oracle comparison above covers small meshes bit for bit)."""
    nx, ny, nz = dims
    m = M.make_box(nx, ny, nz, M.CANTILEVER_SIZE, 1e5, 0.3, gravity=M.GRAVITY_Y, clamp_face=4)
    P, err = build(pattern_shim, m)
    assert err is None, err
    n, nlo, T = P["n"], P["nlo"], m.T
    assert (nlo, 2 * nlo - n) == (nlo_expect, nfull_expect)
    assert nlo == n + len(M.unique_edges(T))

    # Eigen lower CSC by node blocks: per column C the rows R >= C, ascending, diagonal first
    R, Cn = P["lo_rc"][:, 0].astype(np.int64), P["lo_rc"][:, 1].astype(np.int64)
    assert np.all(R >= Cn)
    assert np.array_equal(P["lo_colptr"], np.concatenate([[0], np.cumsum(np.bincount(Cn, minlength=n))]))
    same = Cn[1:] == Cn[:-1]
    assert np.all(Cn[1:] >= Cn[:-1]) and np.all(R[1:][same] > R[:-1][same])
    assert np.array_equal(R[P["lo_colptr"][:-1]], np.arange(n))

    # scatter: local pair (i, j <= i) of every tet lands on the block (max, min) of its nodes
    pi = np.array([0, 1, 1, 2, 2, 2, 3, 3, 3, 3])
    pj = np.array([0, 0, 1, 0, 1, 2, 0, 1, 2, 3])
    a, b = T[:, pi].astype(np.int64), T[:, pj].astype(np.int64)
    blk = P["scatter"]
    assert np.array_equal(R[blk], np.maximum(a, b)) and np.array_equal(Cn[blk], np.minimum(a, b))

    # segments: the inverse of the scatter map, element order inside each block's segment
    seg_c, seg_ptr = P["seg_c"].astype(np.int64), P["seg_ptr"]
    assert seg_ptr[-1] == 10 * m.m
    owner = np.repeat(np.arange(nlo), np.diff(seg_ptr))
    assert np.array_equal(blk.ravel()[seg_c], owner)
    assert np.all(seg_c[1:][owner[1:] == owner[:-1]] > seg_c[:-1][owner[1:] == owner[:-1]])
    assert np.array_equal(np.bincount(seg_c, minlength=10 * m.m), np.ones(10 * m.m, dtype=np.int64))
    nseg_c, nseg_ptr = P["nseg_c"].astype(np.int64), P["nseg_ptr"]
    nown = np.repeat(np.arange(n), np.diff(nseg_ptr))
    assert np.array_equal(T.ravel()[nseg_c], nown)
    assert np.all(nseg_c[1:][nown[1:] == nown[:-1]] > nseg_c[:-1][nown[1:] == nown[:-1]])
    assert np.array_equal(np.bincount(nseg_c, minlength=4 * m.m), np.ones(4 * m.m, dtype=np.int64))

    # SELL: each full block (R, C) and its mirror in a distinct slot of row R / row C
    off = P["chunk_off"]
    assert np.all(np.diff(off) % 32 == 0) and off[-1] == P["nslots"]

    def slot_row(s):
        c = np.searchsorted(off, s, side="right") - 1
        return c * 32 + (s - off[c]) % 32

    lo, up = P["lo_slot"].astype(np.int64), P["up_slot"].astype(np.int64)
    diag = R == Cn
    assert np.array_equal(slot_row(lo), R) and np.array_equal(P["slot_col"][lo], Cn)
    assert np.all(up[diag] == -1) and np.array_equal(P["diag_slot"], lo[diag])
    u = up[~diag]
    assert np.array_equal(slot_row(u), Cn[~diag]) and np.array_equal(P["slot_col"][u], R[~diag])
    used = np.bincount(np.concatenate([lo, u]), minlength=P["nslots"])
    assert used.max() == 1 and used.sum() == nfull_expect


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_pattern_bit_exact_on_renumbered_meshes(pattern_shim, seed):
    """Unstructured numbering: random node ids, tet order and corner order.  The lower
    pattern, the scatter map and the rest data still match the oracle bit for bit."""
    m = M.renumbered(M.batch_instance(3, 40 + seed), seed)
    assert np.all(M.signed_volumes(m.X0, m.T) > 0)
    P, err = build(pattern_shim, m)
    assert err is None, err
    o = oracle.Oracle(m)
    cp, ri = o.pattern()
    mcp, mri = csc_from_blocks(P)
    assert np.array_equal(cp, mcp) and np.array_equal(ri, mri)
    assert np.array_equal(P["scatter"], o.scatter_map())
    assert P["nlo"] == m.n + len(M.unique_edges(m.T))


@pytest.mark.parametrize("make", MESHES)
def test_base_block_layout_and_packing(pattern_shim, make):
    """An instance's device base block (one arena block, one copy, one memset): parts at
    256-byte offsets, in order, without overlap; the uploaded parts before the zeroed ones;
    the total is the sum of the parts rounded to 256 bytes (the serving admission's estimate);
    the packed upload holds the pattern arrays and the positions (4-wide, twice)."""
    m = make()
    P, err = build(pattern_shim, m)
    assert err is None
    out = np.zeros(90, dtype=np.int64)
    k = pattern_shim.pat_layout(out.ctypes.data_as(C.c_void_p))
    assert k == 85
    parts = out[:82].reshape(-1, 2)
    upload_end, zero_end, total = (int(v) for v in out[82:85])
    has_soft = parts[20, 1] > 0
    end = 0
    for i, (off, nb) in enumerate(parts):
        if i == 20 and not has_soft:  # no soft records: the part takes no room
            continue
        assert off % 256 == 0 and off == end and nb > 0
        end = off + ((nb + 255) // 256) * 256
        if i == 22:
            assert end == upload_end
        if i == 37:
            assert end == zero_end
    assert end == total
    n, mm = P["n"], P["m"]
    assert parts[0, 1] == 16 * mm and parts[21, 1] == 32 * n and parts[22, 1] == 32 * n
    buf = np.zeros(upload_end, dtype=np.uint8)
    X0 = np.ascontiguousarray(m.X0, dtype=np.float64).ravel()
    pattern_shim.pat_pack(X0.ctypes.data_as(C.c_void_p), buf.ctypes.data_as(C.c_void_p))

    def view(i, dtype, count):
        off = int(parts[i, 0])
        return np.frombuffer(buf[off:off + count * np.dtype(dtype).itemsize].tobytes(), dtype=dtype)

    assert np.array_equal(view(0, np.int32, 4 * mm), np.ascontiguousarray(m.T, dtype=np.int32).ravel())
    assert np.array_equal(view(1, np.float64, 12 * mm), P["rest64"].ravel())
    assert np.array_equal(view(14, np.int32, 10 * mm), P["seg_c"])
    assert np.array_equal(view(19, np.float64, 4 * n), P["hlin"].ravel())
    x4 = np.zeros((n, 4))
    x4[:, :3] = m.X0
    assert np.array_equal(view(21, np.float64, 4 * n), x4.ravel())
    assert np.array_equal(view(22, np.float64, 4 * n), x4.ravel())
