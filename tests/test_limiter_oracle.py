"""The oracle's Zhang-Shu positivity limiter (positivity_zhang_shu_point2d.jl:22-82):
limited nodes reach the threshold, untouched nodes keep their values, and a state that
needs no limiting is left bit-for-bit alone (CPU only)."""
import numpy as np

GAMMA = 1.4


def dip_state(pts, depth=0.999, width=0.08):
    """Euler state with a narrow density and pressure dip at the square's centre."""
    r2 = (pts[:, 0] - 0.5) ** 2 + (pts[:, 1] - 0.5) ** 2
    rho = 1.0 - depth * np.exp(-r2 / width ** 2)
    p = 1.0 - depth * np.exp(-r2 / width ** 2)
    v1, v2 = 0.3 + 0 * rho, -0.2 + 0 * rho
    e = p / (GAMMA - 1.0) + 0.5 * rho * (v1 * v1 + v2 * v2)
    return np.ascontiguousarray(np.stack([rho, rho * v1, rho * v2, e]))


def pressure(u):
    return (GAMMA - 1.0) * (u[3] - 0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0])


def cloud(oracle, n=32):
    from meshfree_gb300 import workloads as W
    pts, _ = W.jittered_grid(n, n, jitter=0.25)
    idx, _, _, _ = oracle.knn(pts, 35)
    rp = np.arange(pts.shape[0] + 1, dtype=np.int64) * 35
    return pts, rp, idx.ravel()


def test_limiter_reaches_thresholds(oracle):
    pts, rp, ci = cloud(oracle)
    u = dip_state(pts)
    u0 = u.copy()
    thr_rho, thr_p = 0.05, 0.05
    n_rho = oracle.limiter_zhang_shu(u, rp, ci, oracle.LIM_DENSITY, thr_rho)
    n_p = oracle.limiter_zhang_shu(u, rp, ci, oracle.LIM_PRESSURE, thr_p)
    assert n_rho > 0 and n_p > 0
    changed = np.any(u != u0, axis=0)
    assert u[0][changed].min() >= thr_rho * (1 - 1e-12)
    assert pressure(u)[changed].min() >= thr_p * (1 - 1e-9)
    # nodes whose stencil stays above both thresholds are untouched
    far = ((pts[:, 0] - 0.5) ** 2 + (pts[:, 1] - 0.5) ** 2) > 0.3 ** 2
    assert np.array_equal(u[:, far], u0[:, far])


def test_limiter_leaves_admissible_state_alone(oracle):
    pts, rp, ci = cloud(oracle)
    u = dip_state(pts, depth=0.5)
    u0 = u.copy()
    assert oracle.limiter_zhang_shu(u, rp, ci, oracle.LIM_DENSITY, 0.1) == 0
    assert oracle.limiter_zhang_shu(u, rp, ci, oracle.LIM_PRESSURE, 0.1) == 0
    assert np.array_equal(u, u0)
