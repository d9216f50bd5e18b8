"""ctypes front end of the C restatement in mft_oracle.c (test infrastructure only).

Parity status: pinned against the reference's own known-answer/identity tests
(history_test.jl, divergence_test.jl, upwind_viscosity_test.jl), against LAPACK
dsytrf/dsytrs through scipy for the saddle-point solve, and by polynomial
reproduction on the reference fixture test/data/cyl_0_05.  Whole-rhs!/trajectory
parity against Julia itself is unpinned: no Julia toolchain exists here.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

_lib = None

I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
I64P = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")

EQ_EULER2D, EQ_ADVECTION, EQ_EULER3D = 0, 1, 2
BC_DIRICHLET, BC_SLIP_WALL, BC_DO_NOTHING = 0, 1, 2
SRC_RV, SRC_UPWIND, SRC_HV_TOMINEC, SRC_HV_FLYER, SRC_IGR = 0, 1, 2, 3, 4


class _Csr(C.Structure):
    _fields_ = [("n", C.c_int64), ("rp", C.c_void_p), ("ci", C.c_void_p), ("val", C.c_void_p),
                ("cp", C.c_void_p), ("ri", C.c_void_p), ("valt", C.c_void_p)]


class _Semi(C.Structure):
    _fields_ = [("dim", C.c_int), ("nvars", C.c_int), ("eq", C.c_int), ("gamma", C.c_double),
                ("adv", C.c_double * 3), ("n", C.c_int64), ("dop", _Csr * 3),
                ("n_bc", C.c_int), ("bc_kind", C.c_void_p), ("bc_ptr", C.c_void_p),
                ("bc_idx", C.c_void_p), ("bc_normal", C.c_void_p),
                ("n_src", C.c_int), ("src_kind", C.c_void_p),
                ("c_rv", C.c_double), ("c_uw", C.c_double), ("h", C.c_double),
                ("success_iter", C.c_int), ("approx_du", C.c_void_p),
                ("mean_mode", C.c_int), ("max_mode", C.c_int),
                ("hv", _Csr), ("hv_gamma", C.c_double),
                ("igr_alpha", C.c_double), ("igr_maxiter", C.c_int), ("igr_sigma", C.c_void_p)]


class _Diag(C.Structure):
    _fields_ = [("mean", C.c_double * 8), ("norms", C.c_double * 8)]


_variant = "parity"


def select_build(variant: str) -> None:
    """"parity" (default, no FMA contraction: the checker) or "speed" (-O3 with
    contraction: only for timing the CPU baseline).  Takes effect at the next lib()."""
    global _lib, _variant
    assert variant in ("parity", "speed")
    if variant != _variant:
        _variant = variant
        _lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build(variant=_variant)
        L = C.CDLL(str(path))
        L.mfto_pairwise_sum.restype = C.c_double
        L.mfto_pairwise_sum.argtypes = [F64P, C.c_int64, C.c_int64]
        L.mfto_knn.restype = C.c_int
        L.mfto_knn.argtypes = [C.c_int, C.c_int64, F64P, C.c_void_p, C.c_int, I32P, C.c_void_p,
                               C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
        L.mfto_weights.restype = C.c_int
        L.mfto_weights.argtypes = [C.c_int, C.c_int64, F64P, C.c_void_p, I64P, I32P, C.c_int,
                                   C.c_int, C.c_int, F64P, C.c_void_p, C.c_int]
        L.mfto_weights_rows.restype = C.c_int
        L.mfto_weights_rows.argtypes = [C.c_int, C.c_int64, F64P, C.c_void_p, I64P, I32P, C.c_int,
                                        C.c_int, C.c_int, F64P, C.c_int, C.c_int64, I64P]
        L.mfto_saddle_system.restype = C.c_int
        L.mfto_saddle_system.argtypes = [C.c_int, F64P, C.c_void_p, I64P, I32P, C.c_int, C.c_int,
                                         C.c_int, C.c_int64, F64P, F64P, F64P]
        L.mfto_bk_solve.restype = C.c_int
        L.mfto_bk_solve.argtypes = [C.c_int, F64P, C.c_int, F64P]
        L.mfto_rhs.restype = C.c_int
        L.mfto_rhs.argtypes = [C.POINTER(_Semi), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.POINTER(_Diag), C.c_int]
        L.mfto_rhs_adjoint.restype = C.c_int
        L.mfto_rhs_adjoint.argtypes = [C.POINTER(_Semi), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.mfto_limiter_zhang_shu.restype = C.c_int64
        L.mfto_limiter_zhang_shu.argtypes = [C.c_int64, C.c_int, C.c_double, I64P, I32P, C.c_int,
                                             C.c_double, C.c_void_p]
        L.mfto_calc_fluxes.restype = C.c_int
        L.mfto_calc_fluxes.argtypes = [C.POINTER(_Semi), C.c_void_p, C.c_void_p, C.c_int]
        for name in ("mfto_spmv_accum", "mfto_spmv_t_accum"):
            getattr(L, name).restype = None
            getattr(L, name).argtypes = [C.POINTER(_Csr), C.c_double, F64P, F64P, C.c_int]
        L.mfto_spmv.restype = None
        L.mfto_spmv.argtypes = [C.POINTER(_Csr), F64P, F64P, C.c_int]
        L.mfto_csr_to_csc.restype = None
        L.mfto_csr_to_csc.argtypes = [C.c_int64, I64P, I32P, F64P, I64P, I32P, F64P]
        L.mfto_ata.restype = C.c_int
        L.mfto_ata.argtypes = [C.POINTER(_Csr), I64P, C.c_void_p, C.c_void_p, C.c_int]
        L.mfto_time_deriv_weights.restype = C.c_int
        L.mfto_time_deriv_weights.argtypes = [C.c_int, F64P, F64P]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def pairwise_sum(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().mfto_pairwise_sum(x, x.size, 1)


# --------------------------------------------------------------------------
# A1 KNN
# --------------------------------------------------------------------------

def knn(points, k, period=None, nthreads=8):
    """Exact kNN, (d2, index) order, self first.  Returns idx, dists, dx_min, dx_avg."""
    x = np.ascontiguousarray(points, dtype=np.float64)
    n, dim = x.shape
    idx = np.empty((n, k), dtype=np.int32)
    dists = np.empty((n, k), dtype=np.float64)
    per = None if period is None else np.ascontiguousarray(period, dtype=np.float64)
    dmin, davg = C.c_double(), C.c_double()
    rc = lib().mfto_knn(dim, n, x, _ptr(per), k, idx, dists.ctypes.data, C.byref(dmin),
                        C.byref(davg), nthreads)
    if rc:
        raise RuntimeError("mfto_knn failed: %d" % rc)
    return idx, dists, dmin.value, davg.value


# --------------------------------------------------------------------------
# A2-A5 weights
# --------------------------------------------------------------------------

def weights(points, rowptr, stencil, rbf_pow=3, polydeg=3, deriv_order=1, period=None,
            want_resid=False, nthreads=8):
    """Per-node RBF-FD weights.  Returns w (nnz, dim) [and residuals (n,)]."""
    x = np.ascontiguousarray(points, dtype=np.float64)
    n, dim = x.shape
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    stencil = np.ascontiguousarray(stencil, dtype=np.int32)
    w = np.empty((int(rowptr[-1]), dim), dtype=np.float64)
    resid = np.empty(n, dtype=np.float64) if want_resid else None
    per = None if period is None else np.ascontiguousarray(period, dtype=np.float64)
    rc = lib().mfto_weights(dim, n, x, _ptr(per), rowptr, stencil, rbf_pow, polydeg,
                            deriv_order, w, _ptr(resid), nthreads)
    if rc:
        raise RuntimeError("mfto_weights: singular system at node %d" % (-rc - 1))
    return (w, resid) if want_resid else w


def weights_rows(points, rowptr, stencil, rows, rbf_pow=3, polydeg=3, deriv_order=1,
                 period=None, nthreads=8):
    """weights() for the listed rows only; other rows' entries are NaN."""
    x = np.ascontiguousarray(points, dtype=np.float64)
    n, dim = x.shape
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    stencil = np.ascontiguousarray(stencil, dtype=np.int32)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    w = np.full((int(rowptr[-1]), dim), np.nan)
    per = None if period is None else np.ascontiguousarray(period, dtype=np.float64)
    rc = lib().mfto_weights_rows(dim, n, x, _ptr(per), rowptr, stencil, rbf_pow, polydeg,
                                 deriv_order, w, nthreads, rows.size, rows)
    if rc:
        raise RuntimeError("mfto_weights_rows: singular system at node %d" % (-rc - 1))
    return w


def saddle_system(points, rowptr, stencil, e, rbf_pow=3, polydeg=3, deriv_order=1, period=None):
    """Node e's (M, b, s) as the weight computation assembles them."""
    x = np.ascontiguousarray(points, dtype=np.float64)
    dim = x.shape[1]
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    stencil = np.ascontiguousarray(stencil, dtype=np.int32)
    k = int(rowptr[e + 1] - rowptr[e])
    nn = k + math.comb(polydeg + dim, dim)
    m = np.zeros(nn * nn)
    b = np.zeros(nn * dim)
    s = np.zeros(dim)
    per = None if period is None else np.ascontiguousarray(period, dtype=np.float64)
    got = lib().mfto_saddle_system(dim, x, _ptr(per), rowptr, stencil, rbf_pow, polydeg,
                                   deriv_order, e, m, b, s)
    assert got == nn
    return m.reshape(nn, nn, order="F"), b.reshape(nn, dim, order="F"), s


def bk_solve(a, b):
    """Bunch-Kaufman solve of a symmetric system (upper triangle of a used)."""
    n = a.shape[0]
    af = np.asfortranarray(a, dtype=np.float64).ravel(order="F").copy()
    b2 = np.atleast_2d(np.asarray(b, dtype=np.float64).T).T
    bf = np.asfortranarray(b2).ravel(order="F").copy()
    info = lib().mfto_bk_solve(n, af, b2.shape[1], bf)
    if info:
        raise np.linalg.LinAlgError("exactly singular pivot %d" % info)
    return bf.reshape(b2.shape, order="F")


# --------------------------------------------------------------------------
# Sparse operators (SparseArrays.sparse semantics: duplicates summed)
# --------------------------------------------------------------------------

@dataclass
class Csr:
    n: int
    rp: np.ndarray
    ci: np.ndarray
    val: np.ndarray
    cp: np.ndarray
    ri: np.ndarray
    valt: np.ndarray
    _c: _Csr = field(default=None, repr=False)

    def cstruct(self):
        if self._c is None:
            self._c = _Csr(self.n, self.rp.ctypes.data, self.ci.ctypes.data, self.val.ctypes.data,
                           self.cp.ctypes.data, self.ri.ctypes.data, self.valt.ctypes.data)
        return self._c

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.ci, self.rp), shape=(self.n, self.n))


def csr_from_triplets(n, rows, cols, vals):
    """sparse(rows, cols, vals): duplicate (row, col) pairs are summed."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    order = np.lexsort((cols, rows))
    r, c, v = rows[order], cols[order], vals[order]
    if r.size:
        new = np.ones(r.size, dtype=bool)
        new[1:] = (r[1:] != r[:-1]) | (c[1:] != c[:-1])
        if not new.all():
            starts = np.flatnonzero(new)
            out = np.empty(starts.size)
            for m, s in enumerate(starts):
                e = starts[m + 1] if m + 1 < starts.size else r.size
                acc = v[s]
                for q in range(s + 1, e):
                    acc = acc + v[q]
                out[m] = acc
            r, c, v = r[starts], c[starts], out
    rp = np.zeros(n + 1, dtype=np.int64)
    rp[1:] = np.cumsum(np.bincount(r, minlength=n))
    return csr_from_sorted(n, rp, c.astype(np.int32), np.ascontiguousarray(v))


def csr_from_sorted(n, rp, ci, val):
    """Csr from CSR arrays whose rows hold ascending, distinct columns; the CSC view lists
    each column's rows ascending (a stable sort of the columns keeps row order)."""
    rp = np.ascontiguousarray(rp, dtype=np.int64)
    ci = np.ascontiguousarray(ci, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    cp = np.empty(n + 1, dtype=np.int64)
    ri = np.empty(ci.size, dtype=np.int32)
    valt = np.empty(ci.size, dtype=np.float64)
    lib().mfto_csr_to_csc(n, rp, ci, val, cp, ri, valt)
    return Csr(n, rp, ci, val, cp, ri, valt)


def operators_from_stencils(n, rowptr, stencil, w):
    """compute_operators.jl:443-452: one CSR per derivative direction (sparse(...) of the
    stencil triplets).  Stencils of one size without repeated nodes are sorted row by row;
    anything else goes through the general triplet path, which sums duplicates."""
    sizes = np.diff(rowptr)
    if n > 0 and np.all(sizes == sizes[0]):
        k = int(sizes[0])
        st = np.asarray(stencil, dtype=np.int64).reshape(n, k)
        order = np.argsort(st, axis=1, kind="stable")
        cs = np.take_along_axis(st, order, axis=1)
        if k < 2 or np.all(cs[:, 1:] != cs[:, :-1]):
            base = (np.arange(n, dtype=np.int64) * k)[:, None]
            perm = (base + order).ravel()
            ci = cs.ravel().astype(np.int32)
            return [csr_from_sorted(n, np.asarray(rowptr, dtype=np.int64).copy(), ci,
                                    np.ascontiguousarray(w[perm, d])) for d in range(w.shape[1])]
    rows = np.repeat(np.arange(n, dtype=np.int64), sizes)
    return [csr_from_triplets(n, rows, stencil, w[:, d]) for d in range(w.shape[1])]


def csr_add(ops):
    """sum(operators): elementwise + over an identical pattern, left to right."""
    base = ops[0]
    val = base.val.copy()
    for o in ops[1:]:
        assert np.array_equal(o.ci, base.ci) and np.array_equal(o.rp, base.rp)
        val = val + o.val
    return csr_from_sorted(base.n, base.rp.copy(), base.ci.copy(), val)


def ata(a: Csr, nthreads=8) -> Csr:
    """lap' * lap with SparseArrays' per-entry accumulation order (rows in parallel)."""
    L = lib()
    hrp = np.zeros(a.n + 1, dtype=np.int64)
    if L.mfto_ata(C.byref(a.cstruct()), hrp, None, None, nthreads):
        raise MemoryError("mfto_ata")
    nnz = int(hrp[-1])
    hci = np.empty(nnz, dtype=np.int32)
    hval = np.empty(nnz, dtype=np.float64)
    if L.mfto_ata(C.byref(a.cstruct()), hrp, hci.ctypes.data, hval.ctypes.data, nthreads):
        raise MemoryError("mfto_ata")
    return csr_from_sorted(a.n, hrp, hci, hval)


def spmv(a: Csr, x, nthreads=8):
    y = np.empty(a.n)
    lib().mfto_spmv(C.byref(a.cstruct()), np.ascontiguousarray(x, dtype=np.float64), y, nthreads)
    return y


def spmv_accum(a: Csr, alpha, x, y, nthreads=8):
    lib().mfto_spmv_accum(C.byref(a.cstruct()), alpha, np.ascontiguousarray(x, dtype=np.float64),
                          y, nthreads)


def spmv_t_accum(a: Csr, alpha, x, y, nthreads=8):
    lib().mfto_spmv_t_accum(C.byref(a.cstruct()), alpha,
                            np.ascontiguousarray(x, dtype=np.float64), y, nthreads)


def time_deriv_weights(t):
    t = np.ascontiguousarray(t, dtype=np.float64)
    w = np.empty_like(t)
    rc = lib().mfto_time_deriv_weights(t.size, t, w)
    if rc:
        raise RuntimeError("time_deriv_weights failed")
    return w


# --------------------------------------------------------------------------
# rhs! and the SSPRK33 + HistoryCallback driver
# --------------------------------------------------------------------------

class Semi:
    """Holds everything mfto_rhs needs.  `bcs` is a list of (kind, idx, normals,
    value_fn) in NamedTuple order; value_fn(x (m,dim), t) -> (m, nvars)."""

    def __init__(self, points, ops, eq="euler", gamma=1.4, adv=(1.0, 0.5), bcs=(), sources=(),
                 c_rv=1.0, c_uw=1.0, h=1.0, hv=None, hv_gamma=0.0, mean_mode=0, max_mode=0,
                 igr_alpha=1.0, igr_maxiter=20):
        self.points = np.ascontiguousarray(points, dtype=np.float64)
        self.n, self.dim = self.points.shape
        self.ops = list(ops)
        self.eq = {"euler": EQ_EULER2D, "advection": EQ_ADVECTION, "euler3d": EQ_EULER3D}[eq]
        self.nvars = {EQ_EULER2D: 4, EQ_ADVECTION: 1, EQ_EULER3D: 5}[self.eq]
        self.bcs = list(bcs)
        kinds, ptr, idx, nrm = [], [0], [], []
        for kind, ii, normals, _fn in self.bcs:
            kinds.append(kind)
            ii = np.asarray(ii, dtype=np.int32)
            idx.append(ii)
            nrm.append(np.zeros((ii.size, self.dim)) if normals is None
                       else np.asarray(normals, dtype=np.float64).reshape(ii.size, self.dim))
            ptr.append(ptr[-1] + ii.size)
        self.bc_kind = np.asarray(kinds or [0], dtype=np.int32)
        self.bc_ptr = np.asarray(ptr, dtype=np.int64)
        self.bc_idx = np.ascontiguousarray(np.concatenate(idx) if idx else np.zeros(1, np.int32))
        self.bc_normal = np.ascontiguousarray(np.concatenate(nrm) if nrm else np.zeros(1))
        self.src = np.asarray(list(sources) or [0], dtype=np.int32)
        self.approx_du = np.zeros(self.nvars * self.n)
        self.hv = hv
        s = _Semi()
        s.dim, s.nvars, s.eq, s.gamma = self.dim, self.nvars, self.eq, gamma
        for d in range(3):
            s.adv[d] = adv[d] if d < len(adv) else 0.0
        s.n = self.n
        for d, o in enumerate(self.ops):
            s.dop[d] = o.cstruct()
        s.n_bc = len(self.bcs)
        s.bc_kind, s.bc_ptr = self.bc_kind.ctypes.data, self.bc_ptr.ctypes.data
        s.bc_idx, s.bc_normal = self.bc_idx.ctypes.data, self.bc_normal.ctypes.data
        s.n_src = len(sources)
        s.src_kind = self.src.ctypes.data
        s.c_rv, s.c_uw, s.h = c_rv, c_uw, h
        s.success_iter = 0
        s.approx_du = self.approx_du.ctypes.data
        s.mean_mode, s.max_mode = mean_mode, max_mode
        if hv is not None:
            s.hv = hv.cstruct()
        s.hv_gamma = hv_gamma
        s.igr_alpha = igr_alpha
        s.igr_maxiter = igr_maxiter
        self.igr_sigma = np.zeros(self.n)
        s.igr_sigma = self.igr_sigma.ctypes.data
        self.s = s

    def dirichlet_values(self, t):
        total = int(self.bc_ptr[-1])
        if total == 0:
            return None
        out = np.zeros((total, self.nvars))
        for b, (kind, ii, _n, fn) in enumerate(self.bcs):
            if kind == BC_DIRICHLET:
                sl = slice(self.bc_ptr[b], self.bc_ptr[b + 1])
                out[sl] = np.asarray(fn(self.points[np.asarray(ii)], t)).reshape(-1, self.nvars)
        return np.ascontiguousarray(out)

    def rhs(self, u, t, nthreads=8, want_eps=False, diag=False):
        """du = rhs!(u, t); u (nvars, n) is mutated at boundary nodes."""
        assert u.shape == (self.nvars, self.n) and u.flags.c_contiguous
        du = np.empty_like(u)
        uptr = (C.c_void_p * self.nvars)(*[u[v].ctypes.data for v in range(self.nvars)])
        dptr = (C.c_void_p * self.nvars)(*[du[v].ctypes.data for v in range(self.nvars)])
        dv = self.dirichlet_values(t)
        eps = np.empty(self.n) if want_eps else None
        dg = _Diag()
        rc = lib().mfto_rhs(C.byref(self.s), t, _ptr(dv), C.cast(dptr, C.c_void_p),
                            C.cast(uptr, C.c_void_p), _ptr(eps), C.byref(dg), nthreads)
        if rc:
            raise RuntimeError("mfto_rhs failed: %d" % rc)
        out = [du]
        if want_eps:
            out.append(eps)
        if diag:
            out.append((np.array(dg.mean[:self.nvars]), np.array(dg.norms[:self.nvars])))
        return out[0] if len(out) == 1 else tuple(out)

    def rhs_adjoint(self, u, lam, nthreads=8):
        """(d rhs!(u)/du)^T lam (flux divergence, strong BCs, hyperviscosity); u is
        not mutated."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        assert u.shape == (self.nvars, self.n) and lam.shape == u.shape
        out = np.empty_like(u)
        ptrs = [(C.c_void_p * self.nvars)(*[a[v].ctypes.data for v in range(self.nvars)])
                for a in (u, lam, out)]
        rc = lib().mfto_rhs_adjoint(C.byref(self.s), C.cast(ptrs[0], C.c_void_p),
                                    C.cast(ptrs[1], C.c_void_p), C.cast(ptrs[2], C.c_void_p),
                                    nthreads)
        if rc:
            raise RuntimeError("mfto_rhs_adjoint failed: %d" % rc)
        return out

    def bc_project(self, lam):
        """Pi lam: the derivative of the strong-BC pass (Dirichlet entries zero,
        slip-wall momentum projected on the wall)."""
        out = np.array(lam, dtype=np.float64, copy=True)
        for kind, ii, normals, _fn in self.bcs:
            ii = np.asarray(ii, dtype=np.int64)
            if kind == BC_DIRICHLET:
                out[:, ii] = 0.0
            elif kind == BC_SLIP_WALL and self.nvars == 4:
                nr = np.asarray(normals, dtype=np.float64).reshape(ii.size, self.dim)
                nn = np.sqrt(nr[:, 0] * nr[:, 0] + nr[:, 1] * nr[:, 1])
                n1, n2 = nr[:, 0] / nn, nr[:, 1] / nn
                vn = out[1, ii] * n1 + out[2, ii] * n2
                out[1, ii] = out[1, ii] - vn * n1
                out[2, ii] = out[2, ii] - vn * n2
        return out


class History:
    """HistoryCallback (history.jl:15-152): ring of (t, u), newest first."""

    def __init__(self, semi: Semi, approx_order: int):
        self.semi = semi
        self.p = approx_order
        self.t = np.zeros(approx_order + 1)
        self.sol = np.zeros((approx_order + 1, semi.nvars, semi.n))
        self.success_iter = 0

    def push(self, t, u, success_iter):
        """modify_cache! :91-103 -> shift_soln_history! + update_approx_du!"""
        self.success_iter = success_iter
        self.semi.s.success_iter = success_iter
        self.t[1:] = self.t[:-1].copy()
        self.t[0] = t
        self.sol[1:] = self.sol[:-1].copy()
        self.sol[0] = u
        ad = self.semi.approx_du.reshape(self.semi.nvars, self.semi.n)
        ad[:] = 0.0
        m = min(success_iter + 1, self.p + 1)
        if success_iter > 0:
            w = time_deriv_weights(self.t[:m])
            for i in range(m):
                ad += w[i] * self.sol[i]
        return ad


LIM_DENSITY, LIM_PRESSURE = 0, 1


def limiter_zhang_shu(u, rowptr, cols, variable, threshold, gamma=1.4):
    """One variable pass of limiter_zhang_shu! (positivity_zhang_shu_point2d.jl:22-82)
    on the (4, n) Euler state u, in place; stencils (rowptr, cols) in the order given.
    Returns the number of limited nodes."""
    assert u.flags.c_contiguous and u.dtype == np.float64 and u.shape[0] == 4
    rp = np.ascontiguousarray(rowptr, dtype=np.int64)
    ci = np.ascontiguousarray(cols, dtype=np.int32)
    ptrs = (C.c_void_p * 4)(*[u[v].ctypes.data for v in range(4)])
    return int(lib().mfto_limiter_zhang_shu(u.shape[1], 4, gamma, rp, ci, variable, threshold,
                                            C.cast(ptrs, C.c_void_p)))


def stage_limiter(rowptr, cols, variables, thresholds, gamma=1.4):
    """PositivityPreservingLimiterZhangShu(; thresholds, variables) as a callable on u."""
    def lim(u):
        for var, thr in zip(variables, thresholds):
            limiter_zhang_shu(u, rowptr, cols, var, thr, gamma)
    return lim


def ssprk33(semi: Semi, u0, t0, dt, nsteps, history: History | None = None, nthreads=8,
            callback=None, stage_limiter=None):
    """OrdinaryDiffEq SSPRK33 (Shu-Osher form, FSAL) with the HistoryCallback
    applied after every accepted step and once at initialisation; stage_limiter(u)
    (in place) after every stage, as SSPRK33(stage_limiter!) applies it."""
    lim = stage_limiter if stage_limiter is not None else (lambda u: None)
    u = np.array(u0, dtype=np.float64, copy=True)
    t = t0
    k = semi.rhs(u, t, nthreads)
    if history is not None:
        history.push(t, u, 0)
    for step in range(nsteps):
        un = u.copy()
        u1 = un + dt * k
        lim(u1)
        k1 = semi.rhs(u1, t + dt, nthreads)
        u2 = (3.0 * un + u1 + dt * k1) / 4.0
        lim(u2)
        k2 = semi.rhs(u2, t + 0.5 * dt, nthreads)
        u3 = (un + 2.0 * u2 + 2.0 * dt * k2) / 3.0
        lim(u3)
        t = t0 + (step + 1) * dt
        k = semi.rhs(u3, t, nthreads)
        u = u3
        if history is not None:
            history.push(t, u, step + 1)
        if callback is not None:
            callback(step + 1, t, u)
    return u, t


def ssprk33_record(semi: Semi, u0, t0, dt, nsteps, nthreads=8):
    """ssprk33 without callbacks, keeping per step the stage states the adjoint
    sweep linearises about: (u_n, u_1, u_2), each as rhs! left it (strong BCs
    applied).  Returns (u_T, t_T, record); u_T is projected by the BC pass like the
    FSAL evaluation at the end of ssprk33 leaves it."""
    u = np.array(u0, dtype=np.float64, copy=True)
    t = t0
    rec = []
    for step in range(nsteps):
        k = semi.rhs(u, t, nthreads)
        un = u.copy()
        u1 = un + dt * k
        k1 = semi.rhs(u1, t + dt, nthreads)
        u2 = (3.0 * un + u1 + dt * k1) / 4.0
        k2 = semi.rhs(u2, t + 0.5 * dt, nthreads)
        u3 = (un + 2.0 * u2 + 2.0 * dt * k2) / 3.0
        rec.append((un, u1, u2))
        t = t0 + (step + 1) * dt
        u = u3
    semi.rhs(u, t, nthreads)
    return u, t, rec


def ssprk33_adjoint(semi: Semi, rec, dt, lam_T, nthreads=8):
    """Reverse sweep of ssprk33: given lam_T = dJ/du(T), returns dJ/du(t0).
    Per step (Shu-Osher stages with the BC projection Pi):
      a   = Pi(2/3 lam) + 2dt/3 J(u_2)^T lam
      b   = Pi(a/4)     + dt/4  J(u_1)^T a
      lam = Pi(lam/3 + 3a/4 + b) + dt J(u_n)^T b."""
    lam = semi.bc_project(lam_T)
    for un, u1, u2 in reversed(rec):
        a = semi.bc_project((2.0 / 3.0) * lam) + (2.0 * dt / 3.0) * semi.rhs_adjoint(u2, lam, nthreads)
        acc = lam / 3.0
        b = semi.bc_project(0.25 * a) + (0.25 * dt) * semi.rhs_adjoint(u1, a, nthreads)
        acc = acc + 0.75 * a
        lam = semi.bc_project(acc + b) + dt * semi.rhs_adjoint(un, b, nthreads)
    return lam
