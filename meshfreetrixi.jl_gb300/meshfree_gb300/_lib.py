"""ctypes binding of libmeshfree_gb300.so (include/meshfree_gb300.h).

The compute path is the CUDA library only: if the shared library is missing or no
CUDA device is visible, every entry point raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = Path(os.environ.get("MFT_LIBRARY", PKG / "lib" / "libmeshfree_gb300.so"))

MFT_OK, MFT_ERR_ARG, MFT_ERR_CUDA, MFT_ERR_STATE, MFT_ERR_SINGULAR = 0, 1, 2, 3, 4
MFT_ERR_NONFINITE, MFT_ERR_TIMEOUT, MFT_ERR_UNSUPPORTED, MFT_ERR_NOMEM = 5, 6, 7, 8
EQ_EULER2D, EQ_ADVECTION, EQ_EULER3D = 0, 1, 2
BC_DIRICHLET, BC_SLIP_WALL, BC_DO_NOTHING = 0, 1, 2
SRC_RV, SRC_UPWIND, SRC_HV_TOMINEC, SRC_HV_FLYER, SRC_IGR = 0, 1, 2, 3, 4
OP_GRAD, OP_LAP, OP_HV = 0, 1, 2
PREC_FP64, PREC_FP32 = 0, 1
LIM_DENSITY, LIM_PRESSURE = 0, 1
OPT_GATHER, OPT_TUNED_FWD, OPT_TUNED_REV, OPT_FP64_ARITH, OPT_LAYOUT_ORDER = 0, 1, 2, 3, 4
OPT_DW_VARIANT = 5
OPT_HALO_STAGED_FWD, OPT_HALO_STAGED_REV, OPT_HALO_GROUPS, OPT_IGR_ITERS = 6, 7, 8, 9
OPT_ADJ_EVERY, OPT_HALO_ROWS = 10, 11
OPT_ENTRY_ORDER, OPT_BANK_FWD, OPT_BANK_REV = 12, 13, 14
OPT_FUSE_FLUX, OPT_FLUX_FUSED = 15, 16
ARITH_AUTO, ARITH_DFMA, ARITH_DW = 0, 1, 2
GATHER_AUTO, GATHER_THREAD, GATHER_STAGED, GATHER_HALO = 0, 1, 2, 3

# Every entry point of include/meshfree_gb300.h with (restype, argtypes).
VP = C.c_void_p
I32, I64, DBL = C.c_int, C.c_int64, C.c_double
DIRICHLET_FN = C.CFUNCTYPE(None, C.c_double, C.c_int64, C.c_int, C.POINTER(C.c_double), C.c_void_p)
SIGNATURES = {
    "mft_ctx_create": (I32, [C.POINTER(VP), I32, I32]),
    "mft_ctx_destroy": (I32, [VP]),
    "mft_last_error": (C.c_char_p, [VP]),
    "mft_version": (I32, [C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)]),
    "mft_sync": (I32, [VP]),
    "mft_set_points": (I32, [VP, I32, I64, VP, VP]),
    "mft_knn": (I32, [VP, I32, VP, VP, C.POINTER(DBL), C.POINTER(DBL)]),
    "mft_set_stencils": (I32, [VP, VP, VP]),
    "mft_weights": (I32, [VP, I32, I32, I32, I32, VP, C.POINTER(DBL)]),
    "mft_load_csc": (I32, [VP, I32, I32, I64, VP, VP, VP]),
    "mft_weights_noalloc": (I32, [I32, I64, VP, VP, VP, VP, I32, I32, I32, I32, VP, VP,
                                  C.c_char_p, I32]),
    "mft_set_equations": (I32, [VP, I32, VP]),
    "mft_set_bcs": (I32, [VP, I32, VP, VP, VP, VP]),
    "mft_set_dirichlet_values": (I32, [VP, VP]),
    "mft_set_dirichlet_callback": (I32, [VP, DIRICHLET_FN, VP]),
    "mft_set_sources": (I32, [VP, I32, VP, VP]),
    "mft_set_precision": (I32, [VP, I32]),
    "mft_set_option": (I32, [VP, I32, I32]),
    "mft_set_segments": (I32, [VP, I32, VP, VP]),
    "mft_get_option": (I32, [VP, I32, C.POINTER(I32)]),
    "mft_selftest_bounded_wait": (I32, [VP, I32]),
    "mft_measure_fma_rate": (I32, [VP, I32, C.POINTER(DBL)]),
    "mft_rhs": (I32, [VP, VP, VP, I32, DBL]),
    "mft_rhs_device": (I32, [VP, VP, VP, DBL]),
    "mft_set_state": (I32, [VP, VP, I32, DBL]),
    "mft_get_state": (I32, [VP, VP, I32, C.POINTER(DBL)]),
    "mft_history_init": (I32, [VP, I32]),
    "mft_ssprk33": (I32, [VP, DBL, I32, I32]),
    "mft_ssprk33_host": (I32, [VP, VP, I32, C.POINTER(DBL), DBL, I32]),
    "mft_set_rv_state": (I32, [VP, VP, I32, I32]),
    "mft_weights_batch": (I32, [VP, I32, VP, VP]),
    "mft_set_limiter": (I32, [VP, I32, VP, VP]),
    "mft_limit": (I32, [VP, VP, I32]),
    "mft_rhs_adjoint": (I32, [VP, VP, VP, VP, I32, DBL]),
    "mft_rhs_adjoint_device": (I32, [VP, VP, VP, VP, DBL]),
    "mft_ssprk33_record": (I32, [VP, DBL, I32, I32]),
    "mft_ssprk33_adjoint": (I32, [VP, VP, I32]),
    "mft_ssprk33_adjoint_device": (I32, [VP, VP]),
    "mft_get_viscosity": (I32, [VP, VP]),
    "mft_checkpoint_size": (I32, [VP, C.POINTER(C.c_size_t)]),
    "mft_checkpoint_save": (I32, [VP, VP, C.c_size_t]),
    "mft_checkpoint_load": (I32, [VP, VP, C.c_size_t]),
    "mft_profile": (I32, [VP, I32]),
    "mft_profile_get": (I32, [VP, I32, C.POINTER(DBL), C.POINTER(I64), C.POINTER(C.c_char_p)]),
    "mft_region": (I32, [VP, I32, C.POINTER(DBL)]),
}
K_NAMES = ["bc_pass1", "flux", "fwd_gather", "mean", "lexmax", "eps", "rev_gather", "rev_lap",
           "history", "layout", "adjoint", "limiter", "igr"]

_lib = None


class MFTError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("meshfree_gb300 error %d: %s" % (code, msg))
        self.code = code


def load():
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise MFTError(MFT_ERR_STATE, "%s not built (run meshfreetrixi.jl_gb300/build.py)"
                           % LIB_PATH)
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _ptrs(arrs):
    return (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


class WeightGroup(C.Structure):
    """mft_weight_group (include/meshfree_gb300.h)."""
    _fields_ = [("dim", C.c_int), ("n", C.c_int64), ("xyz", C.c_void_p), ("rowptr", C.c_void_p),
                ("cols", C.c_void_p), ("rbf_pow", C.c_int), ("polydeg", C.c_int),
                ("deriv_order", C.c_int), ("w", C.c_void_p)]


class Context:
    """One engine context (one CUDA stream on one device)."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.mft_ctx_create(C.byref(h), device, 0)
        if rc != MFT_OK:
            raise MFTError(rc, "mft_ctx_create failed (no CUDA device %d?)" % device)
        self.h = h
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.mft_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        if rc != MFT_OK:
            raise MFTError(rc, self.lib.mft_last_error(self.h).decode())

    # geometry -----------------------------------------------------------
    def set_points(self, points, period=None):
        x = np.ascontiguousarray(points, dtype=np.float64)
        per = None if period is None else np.ascontiguousarray(period, dtype=np.float64)
        self.check(self.lib.mft_set_points(self.h, x.shape[1], x.shape[0], _p(x), _p(per)))
        self.n, self.dim = x.shape

    def knn(self, k, want_dist=False):
        idx = np.empty((self.n, k), dtype=np.int32)
        dist = np.empty((self.n, k)) if want_dist else None
        dmin, davg = C.c_double(), C.c_double()
        self.check(self.lib.mft_knn(self.h, k, _p(idx), _p(dist), C.byref(dmin), C.byref(davg)))
        self.nnz = self.n * k
        return idx, dist, dmin.value, davg.value

    def set_stencils(self, rowptr, cols):
        rp = np.ascontiguousarray(rowptr, dtype=np.int64)
        ci = np.ascontiguousarray(cols, dtype=np.int32)
        # the C entry point reads n + 1 row offsets and rowptr[n] columns: check the
        # lengths here, where they are known
        if rp.ndim != 1 or rp.size != self.n + 1 or ci.ndim != 1 or rp[-1] != ci.size:
            raise MFTError(MFT_ERR_ARG, "rowptr must hold n + 1 offsets and cols rowptr[n] "
                                        "indices")
        self.check(self.lib.mft_set_stencils(self.h, _p(rp), _p(ci)))
        self.nnz = int(rp[-1])

    def weights(self, op, rbf_pow, polydeg, deriv_order, want_w=False, want_resid=False):
        w = None
        if want_w:
            w = np.empty((self.nnz, self.dim))
        res = C.c_double(np.nan)
        self.check(self.lib.mft_weights(self.h, op, rbf_pow, polydeg, deriv_order, _p(w),
                                        C.byref(res) if want_resid else None))
        return w, (res.value if want_resid else None)

    def load_csc(self, op, comp, colptr, rowval, nzval):
        cp = np.ascontiguousarray(colptr, dtype=np.int64)
        rv = np.ascontiguousarray(rowval, dtype=np.int64)
        nz = np.ascontiguousarray(nzval, dtype=np.float64)
        if cp.ndim != 1 or cp.size < 2 or rv.size < cp[-1] - cp[0] or nz.size < cp[-1] - cp[0]:
            raise MFTError(MFT_ERR_ARG, "colptr must hold n + 1 offsets and rowval / nzval "
                                        "colptr[n] - colptr[0] entries")
        self.check(self.lib.mft_load_csc(self.h, op, comp, cp.size - 1, _p(cp), _p(rv), _p(nz)))

    # physics ------------------------------------------------------------
    def set_equations(self, kind, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        self.check(self.lib.mft_set_equations(self.h, kind, _p(p)))
        self.nvars = {EQ_EULER2D: 4, EQ_EULER3D: 5}.get(kind, 1)

    def set_bcs(self, kinds, ptr, idx, normals):
        k = np.ascontiguousarray(kinds, dtype=np.int32)
        pt = np.ascontiguousarray(ptr, dtype=np.int64)
        ii = np.ascontiguousarray(idx if len(idx) else np.zeros(1), dtype=np.int32)
        nm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float64)
        total = int(pt[-1]) if pt.size else 0
        if pt.size != k.size + 1 or (total and ii.size < total) or (
                nm is not None and total and nm.size < total * max(1, getattr(self, "dim", 2))):
            raise MFTError(MFT_ERR_ARG, "ptr must hold len(kinds) + 1 offsets, idx ptr[-1] "
                                        "nodes and normals dim values per node")
        self.check(self.lib.mft_set_bcs(self.h, k.size, _p(k), _p(pt), _p(ii), _p(nm)))

    def set_dirichlet_values(self, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._keep.append(v)
        self.check(self.lib.mft_set_dirichlet_values(self.h, _p(v)))

    def set_dirichlet_callback(self, fn):
        """fn(t) -> (n_bnodes, nvars) array for all listed boundary nodes."""
        def trampoline(t, nnodes, nvars, out, user):
            vals = np.asarray(fn(t), dtype=np.float64).reshape(nnodes, nvars)
            C.memmove(out, vals.ctypes.data, vals.nbytes)
        cb = DIRICHLET_FN(trampoline) if fn is not None else DIRICHLET_FN()
        self._cb = cb
        self.check(self.lib.mft_set_dirichlet_callback(self.h, cb, None))

    def set_sources(self, kinds, params):
        k = np.ascontiguousarray(kinds, dtype=np.int32)
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        self.check(self.lib.mft_set_sources(self.h, k.size, _p(k) if k.size else None,
                                            _p(p) if p.size else None))

    def set_precision(self, prec):
        self.check(self.lib.mft_set_precision(self.h, prec))

    def set_segments(self, offsets, h):
        """Ensemble members: offsets (nseg+1) and per-member dx_avg (nseg)."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        hh = np.ascontiguousarray(h, dtype=np.float64)
        nseg = off.size - 1
        self.check(self.lib.mft_set_segments(self.h, nseg, _p(off) if nseg else None,
                                             _p(hh) if nseg else None))

    def set_option(self, option, value):
        self.check(self.lib.mft_set_option(self.h, option, value))

    def get_option(self, option):
        v = C.c_int()
        self.check(self.lib.mft_get_option(self.h, option, C.byref(v)))
        return v.value

    def selftest_bounded_wait(self, polls=1000):
        """Runs the bounded-wait self-test; returns its status code (MFT_ERR_TIMEOUT is
        the expected outcome) without raising."""
        return int(self.lib.mft_selftest_bounded_wait(self.h, polls))

    def fma_rate(self, kind):
        """FMAs per second of this GPU: kind 0 FP64, 1 FP32 (mft_measure_fma_rate)."""
        r = C.c_double()
        self.check(self.lib.mft_measure_fma_rate(self.h, kind, C.byref(r)))
        return r.value

    # rhs! / stepping ----------------------------------------------------
    def rhs(self, du, u, t):
        """du, u: (nvars, n) C-contiguous float64 host arrays; u is mutated at BCs."""
        self.check(self.lib.mft_rhs(self.h, _ptrs(list(du)), _ptrs(list(u)), u.shape[0], t))

    def rhs_device(self, du_ptr, u_ptr, t):
        self.check(self.lib.mft_rhs_device(self.h, C.c_void_p(du_ptr), C.c_void_p(u_ptr), t))

    def set_state(self, u, t):
        u = np.ascontiguousarray(u, dtype=np.float64)
        self.check(self.lib.mft_set_state(self.h, _ptrs(list(u)), u.shape[0], t))

    def get_state(self):
        u = np.empty((self.nvars, self.n))
        t = C.c_double()
        self.check(self.lib.mft_get_state(self.h, _ptrs(list(u)), self.nvars, C.byref(t)))
        return u, t.value

    def history_init(self, order):
        self.check(self.lib.mft_history_init(self.h, order))

    def ssprk33(self, dt, nsteps, use_graph=True):
        self.check(self.lib.mft_ssprk33(self.h, dt, nsteps, 1 if use_graph else 0))

    def ssprk33_host(self, u, t, dt, nsteps=1):
        tt = C.c_double(t)
        self.check(self.lib.mft_ssprk33_host(self.h, _ptrs(list(u)), u.shape[0], C.byref(tt),
                                             dt, nsteps))
        return tt.value

    def weights_batch(self, groups, want_resid=False):
        """groups: [(xyz (n, dim), rowptr (n+1), cols, rbf_pow, polydeg, deriv_order)], at most
        two, solved in one batch.  Returns ([w (nnz, dim) per group], max_resid or None)."""
        keep, outs = [], []
        arr = (WeightGroup * len(groups))()
        for g, (xyz, rp, ci, p, deg, order) in enumerate(groups):
            xyz = np.ascontiguousarray(xyz, dtype=np.float64)
            rp = np.ascontiguousarray(rp, dtype=np.int64)
            ci = np.ascontiguousarray(ci, dtype=np.int32)
            w = np.empty((int(rp[-1]), xyz.shape[1]))
            keep += [xyz, rp, ci]
            outs.append(w)
            arr[g] = WeightGroup(xyz.shape[1], xyz.shape[0], xyz.ctypes.data, rp.ctypes.data,
                                 ci.ctypes.data, p, deg, order, w.ctypes.data)
        res = C.c_double()
        self.check(self.lib.mft_weights_batch(self.h, len(groups), arr,
                                              C.byref(res) if want_resid else None))
        return outs, (res.value if want_resid else None)

    # positivity limiter ------------------------------------------------------
    def set_limiter(self, kinds, thresholds):
        k = np.ascontiguousarray(kinds, dtype=np.int32)
        th = np.ascontiguousarray(thresholds, dtype=np.float64)
        self.check(self.lib.mft_set_limiter(self.h, k.size, _p(k) if k.size else None,
                                            _p(th) if k.size else None))

    def limit(self, u):
        """Applies the configured limiter to the (nvars, n) host array u in place."""
        assert u.flags.c_contiguous and u.dtype == np.float64
        self.check(self.lib.mft_limit(self.h, _ptrs(list(u)), u.shape[0]))

    # adjoint --------------------------------------------------------------
    def rhs_adjoint(self, lam, u, t=0.0):
        """(d rhs!(u)/du)^T lam for (nvars, n) host arrays; u is not mutated."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        out = np.empty_like(u)
        self.check(self.lib.mft_rhs_adjoint(self.h, _ptrs(list(out)), _ptrs(list(lam)),
                                            _ptrs(list(u)), u.shape[0], t))
        return out

    def rhs_adjoint_device(self, out_ptr, lam_ptr, u_ptr, t=0.0):
        self.check(self.lib.mft_rhs_adjoint_device(self.h, C.c_void_p(out_ptr), C.c_void_p(lam_ptr),
                                                   C.c_void_p(u_ptr), t))

    def ssprk33_record(self, dt, nsteps, every=0):
        self.check(self.lib.mft_ssprk33_record(self.h, dt, nsteps, every))

    def ssprk33_adjoint(self, lam_T):
        """dJ/du(t0) from dJ/du(T) over the recorded trajectory (host arrays)."""
        lam = np.array(lam_T, dtype=np.float64, order="C", copy=True)
        self.check(self.lib.mft_ssprk33_adjoint(self.h, _ptrs(list(lam)), lam.shape[0]))
        return lam

    def ssprk33_adjoint_device(self, lam_ptr):
        self.check(self.lib.mft_ssprk33_adjoint_device(self.h, C.c_void_p(lam_ptr)))

    def set_rv_state(self, approx_du, success_iter):
        ptrs = None
        if approx_du is not None:
            ad = np.ascontiguousarray(approx_du, dtype=np.float64)
            self._keep.append(ad)
            ptrs = _ptrs(list(ad))
        self.check(self.lib.mft_set_rv_state(self.h, ptrs, self.nvars, success_iter))

    def viscosity(self):
        eps = np.empty(self.n)
        self.check(self.lib.mft_get_viscosity(self.h, _p(eps)))
        return eps

    def checkpoint(self):
        """The time-integration state (t, u, pending first stage, history ring) as bytes
        (mft_checkpoint_save)."""
        size = C.c_size_t(0)
        self.check(self.lib.mft_checkpoint_size(self.h, C.byref(size)))
        buf = (C.c_ubyte * size.value)()
        self.check(self.lib.mft_checkpoint_save(self.h, buf, size.value))
        return bytes(buf)

    def restore(self, image):
        """Loads an image from checkpoint() into this context (mft_checkpoint_load)."""
        image = bytes(image)
        buf = (C.c_ubyte * len(image)).from_buffer_copy(image)
        self.check(self.lib.mft_checkpoint_load(self.h, buf, len(image)))

    def sync(self):
        self.check(self.lib.mft_sync(self.h))

    # timing ---------------------------------------------------------------
    def profile(self, enable=True):
        self.check(self.lib.mft_profile(self.h, 1 if enable else 0))

    def profile_report(self):
        """{kernel name: (total device ms, launches)} since profile(True)."""
        out = {}
        for k in range(len(K_NAMES)):
            ms, n, name = C.c_double(), C.c_int64(), C.c_char_p()
            self.check(self.lib.mft_profile_get(self.h, k, C.byref(ms), C.byref(n), C.byref(name)))
            if n.value:
                out[name.value.decode()] = (ms.value, n.value)
        return out

    def region_begin(self):
        self.check(self.lib.mft_region(self.h, 1, None))

    def region_end(self):
        ms = C.c_double()
        self.check(self.lib.mft_region(self.h, 0, C.byref(ms)))
        return ms.value
