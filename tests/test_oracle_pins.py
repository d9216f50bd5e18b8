"""Pins the CPU oracle against the reference's own tests and LAPACK (CPU only)."""
import numpy as np
import pytest
import scipy.linalg.lapack as lapack
import scipy.sparse as sp
from scipy.spatial import cKDTree

from helpers import GAMMA, cyl_bcs, ic_bumpy, ic_gradient, isapprox, stencil_ops


def test_history_known_answer(oracle):
    """test/history_test.jl:4-32: linear-in-time history gives approx_du == 1."""
    p = 5
    t_hist = np.zeros(p + 1)
    sol = np.zeros((p + 1, p + 1))
    t = 0.0
    u = np.zeros(p + 1)
    for _ in range(p + 1):
        t += 1.0
        u += 1.0
        t_hist[1:] = t_hist[:-1].copy()
        t_hist[0] = t
        sol[:, 1:] = sol[:, :-1].copy()
        sol[:, 0] = u
    success_iter = p + 1
    m = min(success_iter + 1, p + 1)
    w = oracle.time_deriv_weights(t_hist[:m])
    approx_du = sum(w[i] * sol[:, i] for i in range(m))
    assert isapprox(approx_du, np.ones(p + 1))


def test_history_exact_for_polynomials(oracle):
    rng = np.random.default_rng(1)
    for m in range(2, 7):
        t = np.sort(rng.uniform(0.5, 2.0, m))[::-1].copy()
        w = oracle.time_deriv_weights(t)
        c = rng.normal(size=m)
        f = sum(c[k] * t ** k for k in range(m))
        df = sum(k * c[k] * t[0] ** (k - 1) for k in range(1, m))
        assert abs(np.dot(w, f) - df) <= 1e-9 * max(1.0, abs(df))


def _cyl_semi(oracle, cyl, sources=(), rbf_pow=3):
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=rbf_pow)
    bcs = cyl_bcs(cyl, lambda x, t: ic_gradient(x, t).T)
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, bcs=bcs, sources=sources,
                       c_uw=1.0, c_rv=1.0, h=float(cyl["dx"][1]))
    return semi, ops


def test_divergence_identity(oracle, cyl):
    """test/divergence_test.jl:63-82: calc_fluxes! == -Dx fx - Dy fy."""
    semi, ops = _cyl_semi(oracle, cyl)
    u0 = ic_gradient(cyl["positions"])
    du0 = np.zeros_like(u0)
    import ctypes as C
    dptr = (C.c_void_p * 4)(*[du0[v].ctypes.data for v in range(4)])
    uptr = (C.c_void_p * 4)(*[u0[v].ctypes.data for v in range(4)])
    assert oracle.lib().mfto_calc_fluxes(C.byref(semi.s), C.cast(dptr, C.c_void_p),
                                         C.cast(uptr, C.c_void_p), 4) == 0
    from helpers import flux_np
    Dx, Dy = ops[0].to_scipy(), ops[1].to_scipy()
    fx, fy = flux_np(u0, 0), flux_np(u0, 1)
    du1 = np.stack([-(Dx @ fx[v]) - Dy @ fy[v] for v in range(4)])
    assert isapprox(du0, du1)


def test_upwind_viscosity_identity(oracle, cyl):
    """test/upwind_viscosity_test.jl:66-78: source == -Dx'(eps Dx u) - Dy'(eps Dy u)."""
    from oracle.oracle import SRC_UPWIND
    semi_s, ops = _cyl_semi(oracle, cyl, sources=(SRC_UPWIND,))
    semi_0, _ = _cyl_semi(oracle, cyl)
    semi_s.bcs = []
    u0 = ic_gradient(cyl["positions"])
    pts = cyl["positions"]
    # no boundary conditions: the difference of the two rhs! evaluations is the source
    s_nobc = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, sources=(SRC_UPWIND,), c_uw=1.0,
                         h=float(cyl["dx"][1]))
    s_plain = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, h=float(cyl["dx"][1]))
    du_src = s_nobc.rhs(u0.copy(), 0.0) - s_plain.rhs(u0.copy(), 0.0)
    rho, m1, m2, e = u0
    v1, v2 = m1 / rho, m2 / rho
    p = (GAMMA - 1) * (e - 0.5 * (m1 * v1 + m2 * v2))
    eps = 1.0 * 0.5 * cyl["dx"][1] * (np.sqrt(v1 ** 2 + v2 ** 2) + np.sqrt(GAMMA * p / rho))
    Dx, Dy = ops[0].to_scipy(), ops[1].to_scipy()
    du1 = np.stack([-(Dx.T @ (eps * (Dx @ u0[v]))) - Dy.T @ (eps * (Dy @ u0[v])) for v in range(4)])
    assert isapprox(du_src, du1)


def test_bunch_kaufman_matches_lapack(oracle, cyl):
    """The oracle's Bunch-Kaufman solve against LAPACK dsysv (upper), the routine behind
    `Symmetric \\` at compute_operators.jl:435, on the reference fixture's systems."""
    pts = cyl["positions"]
    idx = cyl["knn"]
    n, k = idx.shape
    rowptr = np.arange(n + 1, dtype=np.int64) * k
    st = idx.ravel()
    rng = np.random.default_rng(0)
    worst_rel, worst_res = 0.0, 0.0
    for e in rng.choice(n, 300, replace=False):
        M, b, _s = oracle.saddle_system(pts, rowptr, st, int(e))
        x_o = oracle.bk_solve(M, b)
        _lu, _piv, x_l, info = lapack.dsysv(M, b, lower=0)
        assert info == 0
        worst_rel = max(worst_rel, np.abs(x_o[:k] - x_l[:k]).max() / np.abs(x_l[:k]).max())
        worst_res = max(worst_res, np.abs(M @ x_o - b).max() / np.abs(b).max())
    assert worst_res < 1e-11
    assert worst_rel < 1e-8, worst_rel


def test_weights_reproduce_polynomials(oracle, cyl):
    """RBF-FD weights with degree-3 polynomials differentiate x^a y^b (a+b <= 3)."""
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"])
    Dx, Dy = ops[0].to_scipy(), ops[1].to_scipy()
    x, y = pts[:, 0], pts[:, 1]
    for a in range(4):
        for b in range(4 - a):
            f = x ** a * y ** b
            fx = a * x ** max(a - 1, 0) * y ** b if a else 0 * x
            fy = b * x ** a * y ** max(b - 1, 0) if b else 0 * x
            scale = np.abs(Dx) @ np.abs(f) + 1.0
            assert np.max(np.abs(Dx @ f - fx) / scale) < 1e-9
            assert np.max(np.abs(Dy @ f - fy) / scale) < 1e-9


def test_knn_matches_kdtree(oracle, cyl):
    pts = cyl["positions"]
    idx, dist, dmin, davg = oracle.knn(pts, 20)
    d_ref, i_ref = cKDTree(pts).query(pts, 20)
    assert np.allclose(dist, d_ref, rtol=0, atol=1e-14)
    for i in range(pts.shape[0]):
        assert set(idx[i]) == set(i_ref[i]) or np.isclose(dist[i, -1], d_ref[i, -1])
    assert np.all(idx[:, 0] == np.arange(pts.shape[0]))
    assert dmin == pytest.approx(d_ref[:, 1].min(), rel=0, abs=0)
    assert davg == pytest.approx(d_ref[:, 1].mean(), rel=1e-14)


def _knn_bruteforce(pts, k, period=None):
    n = pts.shape[0]
    out = np.empty((n, k), dtype=np.int64)
    for i in range(n):
        d = pts - pts[i]
        if period is not None:
            for a in range(pts.shape[1]):
                L = period[a]
                d[:, a] = np.where(d[:, a] > 0.5 * L, d[:, a] - L,
                                   np.where(d[:, a] < -0.5 * L, d[:, a] + L, d[:, a]))
        d2 = np.zeros(n)
        for a in range(pts.shape[1]):
            d2 = d2 + d[:, a] * d[:, a]
        out[i] = np.lexsort((np.arange(n), d2))[:k]
    return out


@pytest.mark.parametrize("case", ["grid_ties", "periodic", "3d"])
def test_knn_tie_rule(oracle, case):
    """(squared distance, index) order on inputs with many exact ties."""
    if case == "grid_ties":
        g = np.arange(12) / 12.0
        pts = np.stack(np.meshgrid(g, g, indexing="xy"), -1).reshape(-1, 2)
        period, k = None, 13
    elif case == "periodic":
        g = (np.arange(10) + 0.5) / 10.0
        pts = np.stack(np.meshgrid(g, g, indexing="xy"), -1).reshape(-1, 2)
        period, k = (1.0, 1.0), 21
    else:
        rng = np.random.default_rng(4)
        pts = rng.uniform(0, 1, (400, 3))
        period, k = None, 30
    pts = np.ascontiguousarray(pts)
    idx, _, _, _ = oracle.knn(pts, k, period=period)
    assert np.array_equal(idx, _knn_bruteforce(pts, k, period))


def test_golden_fixture_reproduced(oracle, cyl):
    """The committed fixture outputs are reproduced bit for bit by this build."""
    pts = cyl["positions"]
    idx, _, dmin, davg = oracle.knn(pts, 20)
    assert np.array_equal(idx, cyl["knn"])
    assert dmin == cyl["dx"][0] and davg == cyl["dx"][1]
    _, w = stencil_ops(oracle, pts, idx)
    assert np.array_equal(w, cyl["w_r3"])


def test_rhs_constant_state_is_steady(oracle, cyl):
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"])
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA)
    u = np.ascontiguousarray(np.tile(np.array([[1.0], [0.3], [-0.2], [2.5]]), (1, pts.shape[0])))
    du = semi.rhs(u, 0.0)
    assert np.abs(du).max() < 1e-9


def test_tominec_operator_is_lapT_lap(oracle, cyl):
    pts = cyl["positions"]
    lap_parts, _ = stencil_ops(oracle, pts, cyl["knn"], order=2)
    lap = oracle.csr_add(lap_parts)
    H = oracle.ata(lap)
    Hs = H.to_scipy()
    ls = lap.to_scipy()
    ref = (ls.T @ ls).tocsr()
    ref.sort_indices()
    assert np.array_equal(Hs.indptr, ref.indptr) and np.array_equal(Hs.indices, ref.indices)
    assert np.allclose(Hs.data, ref.data, rtol=1e-12, atol=1e-9 * np.abs(ref.data).max())


def test_rv_norms_reference_quirks(oracle, cyl):
    """ode_mean divides by n*nvars and ode_maximum is lexicographic (mpi.jl:40-81)."""
    from oracle.oracle import SRC_RV
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"])
    u = ic_bumpy(pts)
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, sources=(SRC_RV,), h=0.05)
    _du, (mean, norms) = semi.rhs(u.copy(), 0.0, diag=True)
    n = pts.shape[0]
    assert np.allclose(mean, u.sum(axis=1) / (4 * n), rtol=1e-14)
    loc = np.abs(u - mean[:, None])
    order = np.lexsort(loc[::-1])
    assert np.array_equal(norms, loc[:, order[-1]])
