"""The entry point that allocates nothing: phx_hessian_blocks_noalloc.

It exists for callers that cannot allocate device memory (an engine that keeps
all GPU memory in its own pool, a runtime that forbids cudaMalloc while frames
run): they pass device pointers for every input and output, and the library's
only scratch is a fixed static device array.  This test allocates the caller's
buffers itself (with torch, standing in for the caller's pool), calls the entry
point twice in a row through the C ABI, and checks each result against the
regular allocating entry point (phx_hessian) at the same positions, with the
tolerance the other FP64 Hessian tests use.  It sits in a file of its own that
pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

import physim_gb300 as px
from physim_gb300 import mesh as M

pytestmark = pytest.mark.gpu

MAX_TETS = 32768  # PHX_NOALLOC_MAX_TETS in include/phx.h


def rest_records(m):
    """Per tet: column-major Dm^-1, rest volume, lambda, mu (the layout the entry point reads)."""
    X, T = m.X0, m.T
    Dm = np.stack([X[T[:, c + 1]] - X[T[:, 0]] for c in range(3)], axis=2)  # [m, 3(r), 3(c)]
    inv = np.linalg.inv(Dm)
    rec = np.zeros((m.m, 12))
    rec[:, :9] = inv.transpose(0, 2, 1).reshape(m.m, 9)  # column-major
    rec[:, 9] = np.linalg.det(Dm) / 6.0
    rec[:, 10:12] = m.lame
    return rec


def segments(scatter, nlo):
    """Invert the scatter map: contributions (tet*10 + pair) grouped by lower block, element order."""
    flat = scatter.ravel()
    order = np.argsort(flat, kind="stable").astype(np.int32)
    seg_ptr = np.zeros(nlo + 1, dtype=np.int32)
    np.cumsum(np.bincount(flat, minlength=nlo), out=seg_ptr[1:])
    return seg_ptr, order


def blocks_to_csc(blocks, colptr, n):
    """Lower 3x3 blocks (column-major block order, row-major entries) -> Eigen lower CSC values."""
    vals = np.zeros(colptr[-1])
    k = 0
    for Cn in range(n):
        length = (colptr[3 * Cn + 1] - colptr[3 * Cn]) // 3
        for j in range(length):
            for a in range(3):
                for b in range(3):
                    vals[colptr[3 * Cn + b] + 3 * j + a] = blocks[k, 3 * a + b]
            k += 1
    return vals


def test_noalloc_matches_the_allocating_entry_point(gpu_ctx):
    torch = pytest.importorskip("torch")
    m = M.batch_instance(3, 5)
    assert m.m <= MAX_TETS
    inst = px.Instance(gpu_ctx, m)
    colptr, _ = inst.pattern()
    scatter = inst.scatter_map()
    nlo = inst.sizes()["lower_blocks"]
    seg_ptr, seg_c = segments(scatter, nlo)

    dev = torch.device("cuda", 0)
    t_tets = torch.tensor(m.T.astype(np.int32).ravel(), device=dev)
    t_rest = torch.tensor(rest_records(m).ravel(), device=dev)
    t_model = torch.tensor(m.model.astype(np.uint8), device=dev)
    t_X0 = torch.tensor(m.X0.ravel(), device=dev)
    t_segp = torch.tensor(seg_ptr, device=dev)
    t_segc = torch.tensor(seg_c, device=dev)
    t_out = torch.empty(9 * nlo, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    rng = np.random.default_rng(7)
    h = 0.01
    for call in range(2):  # two calls in a row share the static scratch
        x = (m.X0 + 0.05 * h * rng.standard_normal(m.X0.shape)).ravel()
        t_x = torch.tensor(x, device=dev)
        rc = px.lib().phx_hessian_blocks_noalloc(
            m.n, m.m, nlo, t_tets.data_ptr(), t_rest.data_ptr(), t_model.data_ptr(), t_x.data_ptr(),
            t_X0.data_ptr(), t_segp.data_ptr(), t_segc.data_ptr(), t_out.data_ptr(), C.c_void_p(stream))
        assert rc == px.PHX_OK, px.lib().phx_last_error().decode()
        torch.cuda.synchronize(dev)
        got = blocks_to_csc(t_out.cpu().numpy().reshape(nlo, 9), colptr, m.n)
        want = inst.hessian(x, px.PREC_FP64, fix=False)
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_noalloc_rejects_meshes_beyond_its_scratch(gpu_ctx):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    dummy = torch.zeros(16, dtype=torch.float64, device=dev)
    p = dummy.data_ptr()
    rc = px.lib().phx_hessian_blocks_noalloc(10, MAX_TETS + 1, 10, p, p, None, p, p, p, p, p, None)
    assert rc == px.PHX_EINVAL
    assert "PHX_NOALLOC_MAX_TETS" in px.lib().phx_last_error().decode()
