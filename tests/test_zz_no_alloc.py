"""mft_weights_noalloc: the weight solve for callers that cannot allocate device memory.

Checks, through the C ABI, that two calls in a row give the same weights as the
allocating entry point mft_weights on the same stencils (the weight tests' tolerance:
bit for bit), and that oversized stencils are refused.  Collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.mft_weights_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                  C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    return f


def test_noalloc_weights_match_allocating_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, _h = W.vortex_cloud(40)
    n, k = pts.shape[0], 35
    ctx = L.Context(0)
    ctx.set_points(pts, per)
    idx, _, _, _ = ctx.knn(k)
    w_ref, _ = ctx.weights(L.OP_GRAD, 3, 3, 1, want_w=True)
    rowptr = np.arange(n + 1, dtype=np.int64) * k
    dev = torch.device("cuda:0")
    x_d = torch.from_numpy(pts.copy()).to(dev)
    rp_d = torch.from_numpy(rowptr).to(dev)
    ci_d = torch.from_numpy(idx.ravel().copy()).to(dev)
    per_h = np.ascontiguousarray(per, dtype=np.float64)
    f = _bind(L.load())
    err = C.create_string_buffer(512)
    for _call in range(2):
        w_d = torch.full((n * k * 2,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = f(2, n, x_d.data_ptr(), per_h.ctypes.data, rp_d.data_ptr(), ci_d.data_ptr(), k, 3, 3,
               1, w_d.data_ptr(), None, err, len(err))
        assert rc == 0, err.value.decode()
        w = w_d.cpu().numpy().reshape(n * k, 2)
        assert np.array_equal(w, w_ref)


def test_noalloc_rejects_oversized_stencils(gpu_lib):
    torch = pytest.importorskip("torch")
    from meshfree_gb300 import _lib as L
    f = _bind(L.load())
    dev = torch.device("cuda:0")
    pts = torch.rand((200, 2), dtype=torch.float64, device=dev)
    rp = torch.arange(201, dtype=torch.int64, device=dev) * 5
    ci = torch.zeros(1000, dtype=torch.int32, device=dev)
    w = torch.empty(2000, dtype=torch.float64, device=dev)
    err = C.create_string_buffer(512)
    rc = f(2, 200, pts.data_ptr(), None, rp.data_ptr(), ci.data_ptr(), 400, 3, 3, 1, w.data_ptr(),
           None, err, len(err))
    assert rc == L.MFT_ERR_ARG
    assert b"maximum" in err.value


def _knn_case(torch, L, W):
    pts, per, _h = W.vortex_cloud(24)
    n, k = pts.shape[0], 35
    ctx = L.Context(0)
    ctx.set_points(pts, per)
    idx, _, _, _ = ctx.knn(k + 1)
    ctx.close()
    return pts, per, n, k, idx


def test_noalloc_skips_a_stencil_longer_than_kmax(gpu_lib):
    """kmax = 35 with one stencil of 36 nodes: that stencil is reported (MFT_ERR_ARG) and
    left NaN, every other stencil still equals the allocating entry point's weights."""
    torch = pytest.importorskip("torch")
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, n, k, idx = _knn_case(torch, L, W)
    long_row = 7
    ks = np.full(n, k, dtype=np.int64)
    ks[long_row] = k + 1
    rowptr = np.zeros(n + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum(ks)
    cols = np.concatenate([idx[i, :ks[i]] for i in range(n)]).astype(np.int32)
    ctx = L.Context(0)
    ctx.set_points(pts, per)
    ctx.set_stencils(rowptr, cols)
    w_ref, _ = ctx.weights(L.OP_GRAD, 3, 3, 1, want_w=True)
    ctx.close()
    dev = torch.device("cuda:0")
    x_d = torch.from_numpy(pts.copy()).to(dev)
    rp_d = torch.from_numpy(rowptr).to(dev)
    ci_d = torch.from_numpy(cols).to(dev)
    per_h = np.ascontiguousarray(per, dtype=np.float64)
    f = _bind(L.load())
    err = C.create_string_buffer(512)
    w_d = torch.zeros((int(rowptr[-1]) * 2,), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = f(2, n, x_d.data_ptr(), per_h.ctypes.data, rp_d.data_ptr(), ci_d.data_ptr(), k, 3, 3, 1,
           w_d.data_ptr(), None, err, len(err))
    assert rc == L.MFT_ERR_ARG
    assert b"longer than kmax" in err.value
    w = w_d.cpu().numpy().reshape(-1, 2)
    skipped = np.zeros(int(rowptr[-1]), bool)
    skipped[rowptr[long_row]:rowptr[long_row + 1]] = True
    assert np.isnan(w[skipped]).all()
    assert np.array_equal(w[~skipped], w_ref[~skipped])


def test_noalloc_rejects_invalid_stencils_on_the_device(gpu_lib):
    """An empty stencil and a column index outside 0..n-1 are caught by the kernel's own
    checks before any coordinate is read: MFT_ERR_ARG, NaN weights for the bad rows, and
    the valid rows solved as usual."""
    torch = pytest.importorskip("torch")
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, n, k, idx = _knn_case(torch, L, W)
    ctx = L.Context(0)
    ctx.set_points(pts, per)
    ctx.knn(k)
    w_ref, _ = ctx.weights(L.OP_GRAD, 3, 3, 1, want_w=True)
    ctx.close()
    dev = torch.device("cuda:0")
    per_h = np.ascontiguousarray(per, dtype=np.float64)
    x_d = torch.from_numpy(pts.copy()).to(dev)
    f = _bind(L.load())
    err = C.create_string_buffer(512)
    for case in ("empty", "column"):
        ks = np.full(n, k, dtype=np.int64)
        cols2 = idx[:, :k].copy().astype(np.int32)
        bad = 11
        if case == "empty":
            ks[bad] = 0
        else:
            cols2[bad, 5] = n          # one past the last node
        rowptr = np.zeros(n + 1, dtype=np.int64)
        rowptr[1:] = np.cumsum(ks)
        cols = np.concatenate([cols2[i, :ks[i]] for i in range(n)]).astype(np.int32)
        w_d = torch.zeros((int(rowptr[-1]) * 2,), dtype=torch.float64, device=dev)
        rp_d = torch.from_numpy(rowptr).to(dev)
        ci_d = torch.from_numpy(cols).to(dev)
        torch.cuda.synchronize()
        rc = f(2, n, x_d.data_ptr(), per_h.ctypes.data, rp_d.data_ptr(), ci_d.data_ptr(), k, 3,
               3, 1, w_d.data_ptr(), None, err, len(err))
        assert rc == L.MFT_ERR_ARG, case
        assert b"outside" in err.value or b"empty" in err.value
        w = w_d.cpu().numpy().reshape(-1, 2)
        good_rows = np.ones(n, bool)
        good_rows[bad] = False
        e_good = np.repeat(good_rows, ks)
        e_ref = np.repeat(good_rows, np.full(n, k))
        assert np.array_equal(w[e_good], w_ref[e_ref]), case
        if case == "column":
            assert np.isnan(w[~e_good]).all()
