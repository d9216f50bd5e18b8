"""Seeded synthetic point clouds and initial states for the benchmark workloads.

All random numbers come from numpy's PCG64 with an explicit seed.
"""
from __future__ import annotations

import math

import numpy as np

SEED = 20261203


def rng(seed=SEED):
    return np.random.Generator(np.random.PCG64(seed))


def jittered_grid(nx, ny, lo=(0.0, 0.0), hi=(1.0, 1.0), jitter=0.25, seed=SEED):
    """Cell-centred nx x ny grid on [lo, hi] with uniform jitter of +-jitter*h per axis.
    Row-major node order (x fastest)."""
    g = rng(seed)
    hx = (hi[0] - lo[0]) / nx
    hy = (hi[1] - lo[1]) / ny
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    x = lo[0] + (i.ravel() + 0.5) * hx + g.uniform(-jitter * hx, jitter * hx, nx * ny)
    y = lo[1] + (j.ravel() + 0.5) * hy + g.uniform(-jitter * hy, jitter * hy, nx * ny)
    return np.ascontiguousarray(np.stack([x, y], axis=1)), (hx, hy)


def jittered_grid3(n, lo=0.0, hi=1.0, jitter=0.25, seed=SEED):
    """Cell-centred n x n x n grid on the cube [lo, hi]^3 with uniform jitter of
    +-jitter*h per axis (x fastest)."""
    g = rng(seed)
    h = (hi - lo) / n
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([k.ravel(), j.ravel(), i.ravel()], axis=1)
    pts = lo + (base + 0.5) * h + g.uniform(-jitter * h, jitter * h, base.shape)
    return np.ascontiguousarray(pts), h


def euler3d_wave(x, gamma=1.4):
    """A smooth 3D Euler state on the periodic unit cube: density and pressure waves with
    a swirling velocity (every component varies in every direction)."""
    tp = 2.0 * np.pi
    s = [np.sin(tp * x[:, d]) for d in range(3)]
    c = [np.cos(tp * x[:, d]) for d in range(3)]
    rho = 1.0 + 0.2 * s[0] * c[1] + 0.1 * s[2]
    v1 = 0.3 + 0.1 * s[1] * c[2]
    v2 = -0.2 + 0.1 * s[2] * c[0]
    v3 = 0.1 + 0.1 * s[0] * c[1]
    p = 1.0 + 0.1 * c[0] * s[1] * c[2]
    e = p / (gamma - 1.0) + 0.5 * rho * (v1 * v1 + v2 * v2 + v3 * v3)
    return np.ascontiguousarray(np.stack([rho, rho * v1, rho * v2, rho * v3, e]))


# ------------------------------------------------------------------ scalar advection


def advection_cloud(n=64, seed=SEED):
    """n x n jittered nodes on the unit square plus boundary nodes exactly on the
    edges at spacing h.  Returns points, boundary tags {name: (idx, normals)}, h."""
    pts, (h, _) = jittered_grid(n, n, jitter=0.25, seed=seed)
    s = (np.arange(n) + 0.5) * h
    left = np.stack([np.zeros(n), s], 1)
    bottom = np.stack([s, np.zeros(n)], 1)
    right = np.stack([np.ones(n), s], 1)
    top = np.stack([s, np.ones(n)], 1)
    n0 = pts.shape[0]
    allp = np.ascontiguousarray(np.concatenate([pts, left, bottom, right, top]))
    inflow = np.arange(n0, n0 + 2 * n)
    outflow = np.arange(n0 + 2 * n, n0 + 4 * n)
    nin = np.concatenate([np.tile([-1.0, 0.0], (n, 1)), np.tile([0.0, -1.0], (n, 1))])
    nout = np.concatenate([np.tile([1.0, 0.0], (n, 1)), np.tile([0.0, 1.0], (n, 1))])
    return allp, {"inflow": (inflow, nin), "outflow": (outflow, nout)}, h


def gaussian_bump(x, t, a=(1.0, 0.5), centre=(0.3, 0.3), width=0.05):
    """exp(-|x - centre - a t|^2 / width^2): the exact translated solution."""
    dx = x[:, 0] - centre[0] - a[0] * t
    dy = x[:, 1] - centre[1] - a[1] * t
    return np.exp(-(dx * dx + dy * dy) / (width * width))[None, :]


# ------------------------------------------------------------------ isentropic vortex


def vortex_cloud(n=512, seed=SEED):
    """n x n jittered nodes on the periodic square [-5, 5]^2."""
    pts, (h, _) = jittered_grid(n, n, lo=(-5.0, -5.0), hi=(5.0, 5.0), jitter=0.25, seed=seed)
    return pts, (10.0, 10.0), h


def isentropic_vortex(x, t, gamma=1.4, beta=5.0, vinf=(1.0, 1.0), period=(10.0, 10.0),
                      lo=(-5.0, -5.0)):
    """Isentropic vortex (Shu 1998) advected with vinf on a periodic box: conserved
    variables (4, n).  Background rho = p = 1."""
    xc = np.array([0.0 + vinf[0] * t, 0.0 + vinf[1] * t])
    dx = x[:, 0] - xc[0]
    dy = x[:, 1] - xc[1]
    dx = dx - period[0] * np.round(dx / period[0])
    dy = dy - period[1] * np.round(dy / period[1])
    r2 = dx * dx + dy * dy
    f = np.exp(0.5 * (1.0 - r2))
    u = vinf[0] - beta / (2 * math.pi) * f * dy
    v = vinf[1] + beta / (2 * math.pi) * f * dx
    T = 1.0 - (gamma - 1.0) * beta * beta / (8.0 * gamma * math.pi * math.pi) * f * f
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho ** gamma
    e = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return np.ascontiguousarray(np.stack([rho, rho * u, rho * v, e]))


# ------------------------------------------------------------------ Riemann problem


def riemann_cloud(n=1024, seed=SEED):
    pts, (h, _) = jittered_grid(n, n, jitter=0.25, seed=seed)
    return pts, h


def riemann_states(seed=SEED):
    """Four quadrant states (rho, p) drawn from the seed; zero velocity."""
    g = rng(seed + 1)
    rho = g.uniform(0.125, 1.0, 4)
    p = g.uniform(0.1, 1.0, 4)
    return rho, p


def riemann_ic(x, gamma=1.4, seed=SEED):
    rho4, p4 = riemann_states(seed)
    q = (x[:, 0] >= 0.5).astype(int) + 2 * (x[:, 1] >= 0.5).astype(int)
    rho = rho4[q]
    p = p4[q]
    z = np.zeros_like(rho)
    return np.ascontiguousarray(np.stack([rho, z, z, p / (gamma - 1.0)]))


# ------------------------------------------------------------------ Halton stencils


def halton(n, base, skip=0):
    """Radical-inverse sequence in the given base for indices skip+1 .. skip+n."""
    idx = np.arange(skip + 1, skip + n + 1, dtype=np.int64)
    out = np.zeros(n)
    f = 1.0 / base
    while np.any(idx > 0):
        out += f * (idx % base)
        idx //= base
        f /= base
    return out


def halton_points(n, dim, seed=SEED):
    """Halton points (bases 2, 3, 5) with a seeded random shift modulo 1."""
    g = rng(seed)
    bases = (2, 3, 5)[:dim]
    shift = g.uniform(0.0, 1.0, dim)
    pts = np.stack([(halton(n, b) + shift[d]) % 1.0 for d, b in enumerate(bases)], axis=1)
    return np.ascontiguousarray(pts)


def halton_stencil_sizes(points, seed=SEED, interior_k=35, boundary_k=(40, 60), band=0.02):
    """2D: interior nodes get interior_k; nodes within `band` of the square's edge draw
    k uniformly from boundary_k (inclusive)."""
    g = rng(seed + 7)
    d = np.minimum.reduce([points[:, 0], 1 - points[:, 0], points[:, 1], 1 - points[:, 1]])
    k = np.full(points.shape[0], interior_k, dtype=np.int64)
    b = d < band
    k[b] = g.integers(boundary_k[0], boundary_k[1] + 1, int(b.sum()))
    return k
