#!/usr/bin/env python
"""Benchmark of the RBF-FD rhs! hot path on one GB300 (replicas for --gpus N > 1).

Headline workload (--workload riemann, the default): 2D compressible Euler four-quadrant
Riemann problem on the periodic unit square, N = 1,048,576 seeded jittered nodes, PHS r^3 +
degree-3 polynomials, 35-node stencils, FP64 weights and states, residual viscosity with
the HistoryCallback (approx_order 3) plus Tominec hyperviscosity (c = 1), SSP-RK3 with
dt = 0.1 h.  One step = one SSP-RK3 step = 3 rhs! evaluations.  Metric: node-RHS
updates/s = nodes * rhs! evaluations / device seconds.  The FP64 form's gathers run in
double-word FP32 arithmetic (the engine default); the same workload with FP64 fused
multiply-adds and with the FP32-apply form are reported beside it, and the isentropic
vortex at N = 262,144 (with its L2 error against the exact solution at t = 1) as a
second workload.

--impl reference runs the CPU restatement of the reference's rhs! (the oracle, -O3 build:
the reference is Julia and no Julia toolchain exists on the box) on all host cores,
same workload and metric.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (str(ROOT), str(ROOT / "meshfreetrixi.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "node-RHS updates/s"
UNIT = "node-rhs/s"
K_STENCIL = 35
RHS_PER_STEP = 3
SIDES = {"riemann": 1024, "vortex": 512}
DT_FACTOR = {"riemann": 0.1, "vortex": 0.2}     # dt = factor * h
HV = {"riemann": True, "vortex": False}          # Tominec hyperviscosity on


def _kernel_bytes(prec, hv):
    """Algorithmic bytes per node and launch (V = 4, D = 2, k = 35, int32 indices; a
    neighbour's record counted once, as the scope formula does).
    fwd_gather: idx 4k + weights (2 [+1 lap]) * s k + u V s + du_p V s + t 2V s [+ q V s]
    rev_gather: idx 4k + weights (2 [+1 lap]) * s k + s 2V s [+ q V s] + du_p V s
                + u_s 32 + u_n 32 + out 32 (FP64 state) [+ FP32 shadow 16]"""
    s = 8 if prec == "fp64" else 4
    k = K_STENCIL
    nw = 3 if hv else 2
    fwd = 4 * k + nw * s * k + 4 * s + 4 * s + 8 * s + (4 * s if hv else 0)
    rev = 4 * k + nw * s * k + 8 * s + (4 * s if hv else 0) + 4 * s + 96 + (16 if prec == "fp32" else 0)
    return {"fwd_gather": fwd, "rev_gather": rev}


# Products (one multiply-add each) per node and launch: fwd 14 per stencil entry (t: 8,
# du rows 2-4: 6) [+ 4 for q = lap u]; rev 8 per reverse-adjacency entry [+ 4 lap'].
def _kernel_fmas(hv):
    return {"fwd_gather": (18 if hv else 14) * K_STENCIL, "rev_gather": (12 if hv else 8) * K_STENCIL}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="riemann", choices=["riemann", "vortex"])
    ap.add_argument("--side", type=int, default=0, help="nodes per side (0: the workload's)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ens-members", type=int, default=64,
                    help="members of the ensemble measurement (0 skips it)")
    ap.add_argument("--only", default="all",
                    choices=["all", "adjoint", "riemann", "weights", "igr", "fp32", "setup",
                             "rates", "dw", "dfma", "vortex", "euler3d"],
                    help="run one auxiliary measurement alone")
    ap.add_argument("--gather", default="auto", choices=["auto", "thread", "staged", "halo"],
                    help="FP32 gather mapping of the fp32 measurement (auto: autotuned)")
    ap.add_argument("--halo-rows", type=int, default=0, choices=[0, 128, 256],
                    help="rows per staged group of the dw/dfma/fp32 measurements (0: automatic)")
    ap.add_argument("--entry-order", type=int, default=1, choices=[0, 1],
                    help="entry order inside the staged rows: 1 bank-spreading (default), "
                         "0 ascending columns")
    ap.add_argument("--fuse-flux", type=int, default=1, choices=[0, 1],
                    help="1: the staged double-word forward gather forms the flux records "
                         "while staging (no flux kernel) when it can; 0: never")
    ap.add_argument("--dw-variant", type=int, default=-1,
                    help="double-word gather kernel variant of the dw/dfma measurements "
                         "(-1: autotuned; 0..5 fixed, e.g. for profiling one kernel)")
    ap.add_argument("--igr", type=int, default=1, help="1 runs the IGR-source measurement")
    ap.add_argument("--euler3d-side", type=int, default=64,
                    help="cube side of the 3D Euler measurement (0 skips it)")
    ap.add_argument("--setup", type=int, default=1,
                    help="1 runs the set-up measurement (KNN and weights of the vortex cloud)")
    ap.add_argument("--weights-n", type=int, default=1048576,
                    help="stencils of the batched-weights measurement (0 skips it)")
    ap.add_argument("--riemann-side", type=int, default=1024,
                    help="nodes per side of the Riemann FP32/FP64 run to t = 0.2 (0 skips it)")
    ap.add_argument("--igr-arith", default="dw", choices=["both", "dw", "dfma"],
                    help="engine form(s) of the IGR measurement (the CG itself runs in FP64 "
                         "fused multiply-adds in both)")
    ap.add_argument("--vortex-side", type=int, default=512,
                    help="nodes per side of the vortex measurement (0 skips it)")
    ap.add_argument("--adj-steps", type=int, default=500,
                    help="SSP-RK3 steps of the adjoint measurement")
    ap.add_argument("--adj-tend", type=float, default=0.5,
                    help="end time of the adjoint measurement")
    ap.add_argument("--adj-side", type=int, default=256,
                    help="nodes per side of the adjoint measurement (0 skips it)")
    a = ap.parse_args()
    if a.side <= 0:
        a.side = SIDES[a.workload]
    return a


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def build_problem(workload, side, prec, device, arith="auto"):
    """The workload through the package's Julia-mirroring API (GPU KNN, weights, layout).
    Returns (semi, domain, u0, dt, n)."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    eq = M.CompressibleEulerEquations2D(1.4)
    basis = M.PointCloudBasis(M.Point2D(), 3, approximation_type=M.RBF(M.PolyharmonicSpline(3)),
                              nv=K_STENCIL)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(device=device, precision=prec,
                                                           fp64_arith=arith))
    if workload == "vortex":
        pts, per, h = W.vortex_cloud(side)
        ic = lambda x, t, e: W.isentropic_vortex(x, t)
    else:
        pts, h = W.riemann_cloud(side)
        per = (1.0, 1.0)
        ic = lambda x, t, e: W.riemann_ic(x)
    domain = M.PointCloudDomain(solver, pts, period=per)
    terms = {"rv": M.SourceResidualViscosityTominec(solver, eq, domain, c_rv=1.0, c_uw=1.0)}
    if HV[workload]:
        terms["hv"] = M.SourceHyperviscosityTominec(solver, eq, domain, c=1.0)
    semi = M.SemidiscretizationHyperbolic(domain, eq, ic, solver,
                                          source_terms=M.SourceTerms(**terms))
    return semi, domain, semi.compute_coefficients(0.0), DT_FACTOR[workload] * h, pts.shape[0]


def timed_steps(ctx, u0, dt, warmup, steps, pg, clocks=None):
    """Timed region: `steps` SSP-RK3 steps replayed as per-step CUDA graphs.  A second
    region of the same steps, launched kernel by kernel with an event pair around every
    kernel, gives the per-kernel times for the roofline."""
    ctx.history_init(3)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, warmup, use_graph=True)
    ctx.sync()
    barrier(pg)
    if clocks:
        clocks.start()
    ctx.region_begin()
    ctx.ssprk33(dt, steps, use_graph=True)
    ms = ctx.region_end()
    clk = clocks.stop() if clocks else None
    u_end, _ = ctx.get_state()
    ctx.history_init(3)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, warmup, use_graph=False)
    ctx.profile(True)
    ctx.region_begin()
    ctx.ssprk33(dt, steps, use_graph=False)
    ms_prof = ctx.region_end()
    prof = ctx.profile_report()
    ctx.profile(False)
    return ms, prof, clk, u_end, ms_prof


def ensemble_sizes(members, lo, hi, seed=5):
    """Member node counts drawn uniformly from [lo, hi], rounded to square grids."""
    rng = np.random.default_rng(seed)
    return [int(round(math.sqrt(v))) for v in rng.uniform(lo, hi, members)]


def run_ensemble(args, local, pg):
    """64 independent vortex problems (N uniform in 4,096-131,072) advanced together:
    one context, one CUDA graph per SSP-RK3 step for all members.  The same members
    stepped one context after another (each its own per-step graph) are timed beside it."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    sides = ensemble_sizes(args.ens_members, 4096, 131072)
    clouds = [W.vortex_cloud(s, seed=1000 + i) for i, s in enumerate(sides)]
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=K_STENCIL)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(device=local, precision="fp64"))
    eq = M.CompressibleEulerEquations2D(1.4)

    def semi_of(dom):
        src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
        return M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                              solver, source_terms=src)

    dt = DT_FACTOR["vortex"] * min(c[2] for c in clouds)
    ens = M.PointCloudEnsemble(solver, [c[0] for c in clouds], period=(10.0, 10.0))
    semi = semi_of(ens)
    u0 = semi.compute_coefficients(0.0)
    ntot = int(ens.offsets[-1])
    ms, prof, _, _, _ = timed_steps(ens.ctx, u0, dt, args.warmup, args.steps, pg)
    ms = max_over_ranks(pg, ms)
    ens.ctx.close()
    # the same members, one context each, stepped one after another
    ms_seq = 0.0
    for pts, per, _h in clouds:
        dom = M.PointCloudDomain(solver, pts, period=per)
        s1 = semi_of(dom)
        ctx = dom.ctx
        ctx.history_init(3)
        ctx.set_state(s1.compute_coefficients(0.0), 0.0)
        ctx.ssprk33(dt, args.warmup, use_graph=True)
        ctx.sync()
        ctx.region_begin()
        ctx.ssprk33(dt, args.steps, use_graph=True)
        ms_seq += ctx.region_end()
        ctx.close()
    ms_seq = max_over_ranks(pg, ms_seq)
    launches = sum(v[1] for v in prof.values())
    return {"members": len(sides), "total_nodes": ntot,
            "member_nodes": {"min": min(s * s for s in sides), "max": max(s * s for s in sides)},
            "value": ntot * RHS_PER_STEP * args.steps / (ms * 1e-3), "unit": UNIT,
            "ms_per_step": ms / args.steps, "steps": args.steps,
            "kernel_launches_per_step": launches / args.steps,
            "members_one_at_a_time": {"value": ntot * RHS_PER_STEP * args.steps / (ms_seq * 1e-3),
                                      "ms_per_step": ms_seq / args.steps},
            "workload": "isentropic vortex members on [-5,5]^2, k=%d, RV + history (order 3), "
                        "FP64, dt=0.2 min(h), one CUDA graph per SSP-RK3 step" % K_STENCIL}


def _ragged_stencils(ctx, pts, ks):
    """GPU KNN with the largest k, each node truncated to its own k (nearest first)."""
    ctx.set_points(pts)
    idx, _, _, _ = ctx.knn(int(ks.max()))
    rp = np.zeros(pts.shape[0] + 1, dtype=np.int64)
    rp[1:] = np.cumsum(ks)
    cols = idx[np.arange(idx.shape[1])[None, :] < ks[:, None]].astype(np.int32)
    return rp, cols


def run_setup(args, local):
    """Set-up of the headline workload: KNN stencils (k = 35, periodic minimum image) and
    the gradient operator's weights for every node, each timed as the call a user makes
    (host binning and the engine's host copies included), beside the oracle's KNN and
    per-node Bunch-Kaufman solves on the host cores (the reference's dominant set-up
    cost: one LAPACK factorisation per node)."""
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    from oracle import oracle as O
    pts, per, h = W.vortex_cloud(args.vortex_side or SIDES["vortex"])
    n = pts.shape[0]
    ctx = L.Context(local)
    ctx.set_points(pts, per)
    ctx.knn(K_STENCIL)
    ctx.weights(L.OP_GRAD, 3, 3, 1)            # warm-up (module load, allocations)
    ctx.set_points(pts, per)
    t0 = time.perf_counter()
    ctx.knn(K_STENCIL)
    knn_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.weights(L.OP_GRAD, 3, 3, 1)
    w_s = time.perf_counter() - t0
    # the first rhs! call lays the operators out on the device (sliced ELL, both
    # directions, FP64 and FP32 values); a second call is the plain evaluation
    ctx.set_equations(L.EQ_EULER2D, [1.4])
    ctx.set_bcs([], [0], np.zeros(0, np.int32), None)
    ctx.set_sources([], [])
    u = W.isentropic_vortex(pts, 0.0)
    du = np.empty_like(u)
    t0 = time.perf_counter()
    ctx.rhs(du, u.copy(), 0.0)
    first_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.rhs(du, u.copy(), 0.0)
    rhs_s = time.perf_counter() - t0
    ctx.close()
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    idx, _, _, _ = O.knn(pts, K_STENCIL, period=per, nthreads=nthreads)
    oknn_s = time.perf_counter() - t0
    rowptr = np.arange(n + 1, dtype=np.int64) * K_STENCIL
    t0 = time.perf_counter()
    O.weights(pts, rowptr, idx.ravel(), period=per, nthreads=nthreads)
    ow_s = time.perf_counter() - t0
    return {"workload": "isentropic vortex cloud N=%d, k=%d, periodic; PHS r^3 + degree 3, "
                        "first derivatives" % (n, K_STENCIL),
            "knn_ms": knn_s * 1e3, "weights_ms": w_s * 1e3,
            "layout_ms": (first_s - rhs_s) * 1e3,
            "timing": "wall time of mft_knn and mft_weights (host binning, device search "
                      "and solves, stencil and weight copies the engine keeps); layout: "
                      "first host rhs! call minus a second one",
            "oracle": {"knn_ms": oknn_s * 1e3, "weights_ms": ow_s * 1e3, "cores": nthreads,
                       "kind": "port"}}


def run_weights(args, local):
    """Batched weight generation: 1,048,576 stencils, 90 % 2D seeded-Halton centres
    (interior k = 35, boundary band k uniform in 40..60, degree 3) and 10 % 3D Halton
    (k uniform in 60..90, degree 2), PHS r^3, first derivatives, in one batch
    (size-bucketed persistent launches).  A seeded sample of nodes is checked against
    the oracle's per-node solves; the oracle's time on that sample is the CPU figure."""
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    from oracle import oracle as O
    total = args.weights_n
    n3 = total // 10
    n2 = total - n3
    p2 = W.halton_points(n2, 2, seed=31)
    k2 = W.halton_stencil_sizes(p2, seed=31)
    p3 = W.halton_points(n3, 3, seed=32)
    k3 = np.random.default_rng(32).integers(60, 91, n3)
    ctx2, ctx3 = L.Context(local), L.Context(local)
    rp2, c2 = _ragged_stencils(ctx2, p2, k2)
    rp3, c3 = _ragged_stencils(ctx3, p3, k3)
    pw = W.halton_points(4096, 2, seed=34)                  # warm-up batch
    rpw, cw = _ragged_stencils(ctx3, pw, np.full(4096, K_STENCIL))
    ctx3.close()
    groups = [(p2, rp2, c2, 3, 3, 1), (p3, rp3, c3, 3, 2, 1)]
    ctx2.weights_batch([(pw, rpw, cw, 3, 3, 1)])
    ctx2.region_begin()
    t0 = time.perf_counter()
    (w2, w3), _ = ctx2.weights_batch(groups)
    wall = time.perf_counter() - t0
    dev_ms = ctx2.region_end()
    ctx2.close()
    rng = np.random.default_rng(33)
    # a sample large enough to keep the host cores busy (the CPU figure) and to check
    # bit-identity on tens of thousands of systems
    s2 = np.sort(rng.choice(n2, min(n2, 40000), replace=False))
    s3 = np.sort(rng.choice(n3, min(n3, 4000), replace=False))
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r2 = O.weights_rows(p2, rp2, c2, s2, rbf_pow=3, polydeg=3, nthreads=nthreads)
    r3 = O.weights_rows(p3, rp3, c3, s3, rbf_pow=3, polydeg=2, nthreads=nthreads)
    cpu_s = time.perf_counter() - t0
    m2 = np.zeros(n2, bool)
    m2[s2] = True
    m3 = np.zeros(n3, bool)
    m3[s3] = True
    e2 = np.repeat(m2, k2)
    e3 = np.repeat(m3, k3)
    same = bool(np.array_equal(w2[e2], r2[e2]) and np.array_equal(w3[e3], r3[e3]))
    rel = max(float(np.abs(w2[e2] - r2[e2]).max() / np.abs(r2[e2]).max()),
              float(np.abs(w3[e3] - r3[e3]).max() / np.abs(r3[e3]).max()))
    return {"workload": "%d stencils: %d 2D Halton (k 35 interior, 40-60 boundary band, degree 3) "
                        "+ %d 3D Halton (k 60-90, degree 2), PHS r^3, first derivatives"
                        % (total, n2, n3),
            "systems": total, "max_system": int(max(k2.max() + 10, k3.max() + 10)),
            "value": total / (dev_ms * 1e-3), "unit": "systems/s",
            "device_ms": dev_ms, "wall_s": wall,
            "timing": "device time of the whole batch call on the stream (stencil upload, "
                      "size-bucketed solves, weight download)",
            "parity_sample": {"nodes_2d": int(s2.size), "nodes_3d": int(s3.size),
                              "bit_identical": same, "max_rel_diff": rel},
            "cpu_sample": {"value": (s2.size + s3.size) / cpu_s, "unit": "systems/s",
                           "cores": nthreads, "kind": "port",
                           "sample": "the same %d sampled systems, oracle per-node solves"
                                     % (s2.size + s3.size)}}


CURVE_POINTS = 16


def run_riemann(args, local):
    """Four-quadrant Riemann problem on the unit square, periodic (N = side^2 jittered
    nodes), residual viscosity + Tominec hyperviscosity (c = 1), SSP-RK3 with dt = 0.1 h
    to t = 0.2, in the FP64 form and the FP32-apply form: throughput of both, the FP32
    density error at t = 0.2, and the relative L2 density difference from the FP64 run at
    16 times along the way for the FP32 form and for the FP64 form started from a
    rounding-size perturbation of u0.  (With open edges, one-sided stencils grow unstable boundary
    modes at this resolution; the periodic square keeps the run bounded.)"""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    side = args.riemann_side
    pts, h = W.riemann_cloud(side)
    n = pts.shape[0]
    dt = 0.1 * h
    nsteps = int(round(0.2 / dt))
    eq = M.CompressibleEulerEquations2D(1.4)
    out = {}
    curves = {}
    snaps = []
    # fp64p: the FP64 form from u0 perturbed by seeded relative noise of FP32 rounding size,
    # which measures how strongly this discontinuous flow amplifies such differences
    for prec in ("fp64", "fp32", "fp64p"):
        basis = M.PointCloudBasis(M.Point2D(), 3, nv=K_STENCIL)
        solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(device=local,
                                                               precision=prec[:4]))
        dom = M.PointCloudDomain(solver, pts, period=(1.0, 1.0))
        src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom),
                            hv=M.SourceHyperviscosityTominec(solver, eq, dom))
        semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.riemann_ic(x), solver,
                                              source_terms=src)
        ctx = dom.ctx
        u0 = semi.compute_coefficients(0.0)
        if prec == "fp64p":
            noise = np.random.default_rng(41).uniform(-1.0, 1.0, u0.shape)
            u0 = np.ascontiguousarray(u0 * (1.0 + 6e-8 * noise))
        ctx.history_init(3)
        ctx.set_state(u0, 0.0)
        ctx.ssprk33(dt, 3, use_graph=True)          # warm-up (autotune, graph capture)
        ctx.history_init(3)
        ctx.set_state(u0, 0.0)
        # the run in chunks (the same steps and times as one call), the density read back
        # between chunks outside the timed regions: difference-versus-time curves
        ms = 0.0
        done = 0
        curve = []
        for ch in range(CURVE_POINTS):
            k = (nsteps * (ch + 1)) // CURVE_POINTS - done
            ctx.region_begin()
            ctx.ssprk33(dt, k, use_graph=True)
            ms += ctx.region_end()
            done += k
            uc, tc = ctx.get_state()
            if prec == "fp64":
                snaps.append(uc[0].copy())
                curve.append(tc)
            else:
                ref = snaps[ch]
                curve.append(float(np.linalg.norm(uc[0] - ref) / np.linalg.norm(ref)))
        u, t = ctx.get_state()
        ctx.close()
        out[prec] = (ms, u, t)
        curves[prec] = curve
    ms64, u64, t64 = out["fp64"]
    ms32, u32, _ = out["fp32"]
    v64 = n * RHS_PER_STEP * nsteps / (ms64 * 1e-3)
    v32 = n * RHS_PER_STEP * nsteps / (ms32 * 1e-3)
    return {"workload": "four-quadrant Riemann problem, unit square, N=%d jittered nodes, k=%d, "
                        "RV + Tominec HV, SSP-RK3 dt=0.1h to t=%.3f (%d steps), periodic"
                        % (n, K_STENCIL, t64, nsteps),
            "nodes": n, "steps": nsteps,
            "fp64": {"value": v64, "unit": UNIT, "ms_per_step": ms64 / nsteps,
                     "finite": bool(np.isfinite(u64).all())},
            "fp32_apply": {"value": v32, "unit": UNIT, "ms_per_step": ms32 / nsteps,
                           "speedup_vs_fp64": v32 / v64,
                           "l2_density_err_vs_fp64": float(np.linalg.norm(u32[0] - u64[0])
                                                           / np.linalg.norm(u64[0])),
                           "linf_density_err_vs_fp64": float(np.abs(u32[0] - u64[0]).max()
                                                             / np.abs(u64[0]).max())},
            "fp64_perturbed": {
                "perturbation": "u0 * (1 + 6e-8 U(-1, 1)), seeded (FP32 rounding size)",
                "l2_density_diff_vs_fp64": float(np.linalg.norm(out["fp64p"][1][0] - u64[0])
                                                 / np.linalg.norm(u64[0])),
                "linf_density_diff_vs_fp64": float(np.abs(out["fp64p"][1][0] - u64[0]).max()
                                                   / np.abs(u64[0]).max())},
            "density_range_fp64": [float(u64[0].min()), float(u64[0].max())],
            "l2_density_diff_vs_time": {"t": curves["fp64"], "fp32_apply": curves["fp32"],
                                        "fp64_perturbed": curves["fp64p"]}}


def run_igr(args, local):
    """IGR source on the vortex (N = 262,144, alpha = h^2, at most 20 CG iterations per
    rhs! evaluation): SSP-RK3 steps with graphs, against the same steps without it."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    from meshfree_gb300 import _lib as L
    pts, per, h = W.vortex_cloud(args.vortex_side or SIDES["vortex"])
    n = pts.shape[0]
    eq = M.CompressibleEulerEquations2D(1.4)
    ic = lambda x, t, e: W.isentropic_vortex(x, t)
    res = {}
    for arith in (("dw", "dfma") if args.igr_arith == "both" else (args.igr_arith,)):
        basis = M.PointCloudBasis(M.Point2D(), 3, nv=K_STENCIL)
        solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(device=local, precision="fp64",
                                                               fp64_arith=arith))
        dom = M.PointCloudDomain(solver, pts, period=per)
        out = {}
        for name, src in (("plain", M.SourceTerms()),
                          ("igr", M.SourceTerms(igr=M.SourceIGR(solver, eq, dom, alpha=h * h)))):
            semi = M.SemidiscretizationHyperbolic(dom, eq, ic, solver, source_terms=src)
            u0 = semi.compute_coefficients(0.0)
            ctx = dom.ctx
            ctx.set_state(u0, 0.0)
            ctx.ssprk33(DT_FACTOR["vortex"] * h, 2, use_graph=True)
            ctx.set_state(u0, 0.0)
            ctx.region_begin()
            ctx.ssprk33(DT_FACTOR["vortex"] * h, args.steps, use_graph=True)
            out[name] = ctx.region_end() / args.steps
        iters = ctx.get_option(L.OPT_IGR_ITERS)
        ctx.close()
        res[arith] = {"ms_per_step": out["igr"], "ms_per_step_without_igr": out["plain"],
                      "igr_ms_per_rhs": (out["igr"] - out["plain"]) / RHS_PER_STEP,
                      "cg_iterations_last_solve": iters}
    first = next(iter(res))
    out = {"workload": "isentropic vortex N=%d, k=%d, SourceIGR alpha=h^2, <= 20 CG iterations "
                       "per rhs!, SSP-RK3 graphs" % (n, K_STENCIL),
           "fp64_gather_arithmetic": first}
    out.update(res[first])
    if "dfma" in res and first != "dfma":
        out["fp64_fma_gathers"] = res["dfma"]
    return out


def run_euler3d(args, local, peaks):
    """CompressibleEulerEquations3D on a periodic jittered cube (N = side^3, PHS r^3 +
    degree 2, k = 30): the plain flux divergence in the FP64 form (double-word gathers),
    SSP-RK3 steps with per-step graphs; the gather's HBM roofline by the same convention
    (k indices, 3 k weights, the state and the flux record of the node, the stage's
    u_n / u_s / out)."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    side = args.euler3d_side
    pts, h = W.jittered_grid3(side, seed=11)
    n = pts.shape[0]
    k = 30
    basis = M.PointCloudBasis(M.Point3D(), 2, nv=k)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(device=local, precision="fp64"))
    dom = M.PointCloudDomain(solver, pts, period=(1.0, 1.0, 1.0))
    eq = M.CompressibleEulerEquations3D(1.4)
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.euler3d_wave(x), solver)
    ctx = dom.ctx
    u0 = semi.compute_coefficients(0.0)
    dt = 0.1 * h
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, args.warmup, use_graph=True)
    ctx.region_begin()
    ctx.ssprk33(dt, args.steps, use_graph=True)
    ms = ctx.region_end()
    ctx.profile(True)
    ctx.ssprk33(dt, args.steps, use_graph=False)
    prof = ctx.profile_report()
    ctx.profile(False)
    ctx.close()
    fwd_ms, fwd_n = prof.get("fwd_gather", (0.0, 0))
    per = fwd_ms / max(fwd_n, 1)
    # per node: indices 4k, weights 3*8k, flux record 96 (its 12 distinct values) + state
    # 40 in, stage in/out 80
    bytes_node = 4 * k + 24 * k + 96 + 40 + 80
    return {"workload": "CompressibleEulerEquations3D, periodic unit cube, N=%d jittered nodes, "
                        "PHS r^3 + degree-2 polynomials, k=%d, plain flux divergence (FP64 form, "
                        "double-word gathers), "
                        "SSP-RK3 dt=0.1h, per-step graphs" % (n, k),
            "nodes": n, "value": n * RHS_PER_STEP * args.steps / (ms * 1e-3), "unit": UNIT,
            "ms_per_step": ms / args.steps, "kernels": _kernels(prof),
            "fwd_gather_gbs": bytes_node * n / (per * 1e-3) / 1e9 if fwd_n else None,
            "fwd_gather_hbm_frac": (bytes_node * n / (per * 1e-3) / 1e9) / peaks["hbm_gbs"]
            if fwd_n else None,
            "algorithmic_bytes_per_node": bytes_node}


def run_adjoint(args, local, peaks):
    """Gradient of J = 0.5 |rho(T) - rho*|^2 w.r.t. u0 for the isentropic vortex at
    N = 65,536 (T = 0.5, 500 SSP-RK3 steps; rho* the exact density at T plus seeded
    1e-3 N(0,1) noise), against the forward solve's cost: with the default recording
    policy (every stage state when it fits in memory) and with checkpoints every 20 steps
    and recomputation."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    side, T, nsteps, every = args.adj_side, args.adj_tend, args.adj_steps, 20
    dt = T / nsteps
    pts, per, _h = W.vortex_cloud(side)
    n = pts.shape[0]
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=K_STENCIL)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(device=local, precision="fp64"))
    dom = M.PointCloudDomain(solver, pts, period=per)
    semi = M.SemidiscretizationHyperbolic(dom, M.CompressibleEulerEquations2D(1.4),
                                          lambda x, t, e: W.isentropic_vortex(x, t), solver)
    ctx = dom.ctx
    if args.dw_variant >= 0:
        from meshfree_gb300 import _lib as L
        ctx.set_option(L.OPT_DW_VARIANT, args.dw_variant)
    u0 = semi.compute_coefficients(0.0)
    rng = np.random.default_rng(20)
    target = W.isentropic_vortex(pts, T)[0] + 1e-3 * rng.standard_normal(n)

    def J(u):
        d = u[0] - target
        return 0.5 * float(d @ d)

    def forward(u):
        ctx.set_state(u, 0.0)
        ctx.region_begin()
        ctx.ssprk33(dt, nsteps, use_graph=True)
        ms = ctx.region_end()
        return ctx.get_state()[0], ms

    def gradient(k):
        ctx.set_state(u0, 0.0)
        ctx.region_begin()
        ctx.ssprk33_record(dt, nsteps, k)
        ms_rec = ctx.region_end()
        uT = ctx.get_state()[0]
        lam = np.zeros_like(uT)
        lam[0] = uT[0] - target
        ctx.region_begin()
        g = ctx.ssprk33_adjoint(lam)
        return g, ms_rec, ctx.region_end()

    from meshfree_gb300 import _lib as L
    forward(u0)                     # warm-up (graph capture)
    uT, ms_fwd = forward(u0)
    gradient(every)                 # warm-up
    grad, ms_rec, ms_adj = gradient(every)
    grad0, ms_rec0, ms_adj0 = gradient(-1)   # the default recording policy
    chosen = ctx.get_option(L.OPT_ADJ_EVERY)
    ctx.profile(True)
    gradient(-1)
    prof = ctx.profile_report()
    ctx.profile(False)
    # centred difference of J along a seeded direction, through two forward solves
    v = rng.standard_normal(u0.shape) * np.abs(u0).max(axis=1, keepdims=True)
    e = 1e-6
    fd = (J(forward(np.ascontiguousarray(u0 + e * v))[0])
          - J(forward(np.ascontiguousarray(u0 - e * v))[0])) / (2 * e)
    ad = float(np.sum(grad0 * v))
    ms_k, launches = prof.get("adjoint", (0.0, 0))
    per_launch = ms_k / max(launches, 1)
    # adjoint kernel, per node: idx 4k + D_x, D_y 16k + lam row 32 + u 32 + lam_i 32
    # + acc read/write 64 + out 32 (cached neighbour rows); FP64 FMAs 8 per entry
    bytes_node = 4 * K_STENCIL + 16 * K_STENCIL + 32 * 6
    ctx.close()
    return {"workload": "isentropic vortex N=%d, T=%.1f, %d SSP-RK3 steps, k=%d, no viscosity "
                        "source; J = 0.5|rho(T) - rho*|^2, rho* = exact density + 1e-3 N(0,1) "
                        "(seeded)" % (n, T, nsteps, K_STENCIL),
            "nodes": n, "steps": nsteps,
            "recording_policy": ("every stage state stored (%d bytes: fits in half of the "
                                 "free HBM, so the sweep recomputes nothing)"
                                 % (3 * nsteps * 4 * n * 8)) if chosen == 0 else
                                ("checkpoint every %d steps, stages recomputed" % chosen),
            "forward_ms": ms_fwd, "record_ms": ms_rec0, "adjoint_sweep_ms": ms_adj0,
            "gradient_over_forward": (ms_rec0 + ms_adj0) / ms_fwd,
            "adjoint_sweep_over_forward": ms_adj0 / ms_fwd,
            "checkpointed": {"checkpoint_every": every, "record_ms": ms_rec,
                             "adjoint_sweep_ms": ms_adj,
                             "adjoint_sweep_over_forward": ms_adj / ms_fwd,
                             "gradient_over_forward": (ms_rec + ms_adj) / ms_fwd,
                             "max_abs_diff_vs_default": float(np.abs(grad0 - grad).max())},
            "fd_check": {"directional_fd": fd, "adjoint": ad, "rel_err": abs(fd - ad) / abs(ad),
                         "fd_step": e},
            "kernel": {"name": "adjoint", "avg_launch_ms": per_launch, "launches": launches,
                       "algorithmic_bytes_per_node": bytes_node,
                       "achieved_gbs": bytes_node * n / (per_launch * 1e-3) / 1e9 if launches else None,
                       "hbm_frac": (bytes_node * n / (per_launch * 1e-3) / 1e9) / peaks["hbm_gbs"]
                       if launches else None,
                       "gproducts_s": 8 * K_STENCIL * n / (per_launch * 1e-3) / 1e9 if launches else None}}


# Whole-rhs! algorithmic bytes per node and rhs! (2D Euler, V=4, k=35, int32 indices), the
# formula of the scope table: plain fused rhs! (u read, D_x/D_y weights, indices, du
# write) + the fused SSP-RK stage combination (u_n read) + the residual-viscosity passes
# (D^T weights and indices, t = D u written and read, approx_du, eps) [+ Tominec
# hyperviscosity lap'(lap u): two gathers of lap weights and indices, q written and read].
def path_bytes(prec, hv):
    k = K_STENCIL
    if prec == "fp64":
        parts = [("plain", 764), ("stage", 32), ("RV", 876)]
        if hv:
            parts.append(("Tominec HV", 2 * (8 * k + 4 * k) + 2 * 4 * 8))
    else:
        parts = [("plain", 452), ("stage (FP64 u_n)", 32), ("RV (FP32 weights/t)", 532)]
        if hv:
            parts.append(("Tominec HV", 2 * (4 * k + 4 * k) + 2 * 4 * 4))
    return {"formula": " + ".join("%d %s" % (b, nm) for nm, b in parts),
            "bytes": sum(b for _, b in parts)}


SPEC_HBM_GBS = 8000.0    # the nominal HBM figure the scope table quotes beside the measured one


def path_roofline(node_rhs_per_s, prec, hv, peaks):
    """HBM roofline of the whole rhs! from the end-to-end node-RHS rate."""
    b = path_bytes(prec, hv)
    achieved = b["bytes"] * node_rhs_per_s / 1e9
    return {"bytes_per_node_rhs": b["bytes"], "formula": b["formula"], "achieved_gbs": achieved,
            "frac_of_measured": achieved / peaks["hbm_gbs"],
            "frac_of_8tbs": achieved / SPEC_HBM_GBS}


def roofline(prof, n, prec, hv, peaks, arith=None, tag=None):
    """Roofline of the kernel with the largest share of the profiled steps: algorithmic
    bytes per launch / its average CUDA-event duration, against the measured HBM copy
    bandwidth; for the FP64 form also its multiply-adds per second against the measured
    FP64 (DFMA arithmetic) or FP32 (double-word arithmetic, 12 FP32 operations per
    product) rate."""
    name = max(prof, key=lambda k: prof[k][0])
    ms, launches = prof[name]
    per_launch = ms / launches
    bpn = _kernel_bytes(prec, hv).get(name)
    out = {"kernel": name, "avg_launch_ms": per_launch, "launches": launches,
           "share_of_profiled_step": ms / sum(v[0] for v in prof.values())}
    if bpn is not None:
        achieved = bpn * n / (per_launch * 1e-3) / 1e9
        out.update({"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                    "algorithmic_bytes_per_node": bpn, "peak_source": peaks["source"]})
    traffic = ncu_traffic(name, tag) if tag else None
    out["traffic"] = None if traffic is None else traffic * n
    out["traffic_source"] = (None if traffic is None else
                             "profiles/ncu_%s_%s.md: ncu DRAM bytes per node x N" % (name, tag))
    fmas = _kernel_fmas(hv).get(name)
    if prec == "fp64" and fmas and peaks.get("fma_rates"):
        g = fmas * n / (per_launch * 1e-3)
        if arith == "dfma":
            pk = peaks["fma_rates"]["fp64"]
            out["fp64_issue"] = {"achieved_gfma_s": g / 1e9, "peak_gfma_s": pk / 1e9,
                                 "frac": g / pk, "fma_per_node": fmas,
                                 "peak_source": "mft_measure_fma_rate (this run)"}
        else:
            pk = peaks["fma_rates"]["fp32"] / 12.0
            out["fp32_issue"] = {"achieved_gproducts_s": g / 1e9,
                                 "peak_gproducts_s": pk / 1e9, "frac": g / pk,
                                 "products_per_node": fmas,
                                 "note": "double-word product + compensated sum = 12 FP32 "
                                         "operations; peak = measured FP32 FMA rate / 12"}
    return out


def ncu_traffic(kernel, tag):
    """DRAM bytes per node of one launch from the committed ncu summary, if any."""
    f = ROOT / "profiles" / ("ncu_%s_%s.md" % (kernel, tag))
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_node:"):
            return float(line.split(":")[1])
    return None


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def oracle_problem(workload, side, nthreads):
    """The same workload in the oracle (-O3 timing build): KNN, weights, operators (and
    lap' lap for the hyperviscosity), outside any timed region."""
    from oracle import oracle as O
    from meshfree_gb300 import workloads as W
    O.select_build("speed")
    if workload == "vortex":
        pts, per, h = W.vortex_cloud(side)
        u0 = W.isentropic_vortex(pts, 0.0)
    else:
        pts, h = W.riemann_cloud(side)
        per = (1.0, 1.0)
        u0 = W.riemann_ic(pts)
    n = pts.shape[0]
    idx, _, dmin, davg = O.knn(pts, K_STENCIL, period=per, nthreads=nthreads)
    rowptr = np.arange(n + 1, dtype=np.int64) * K_STENCIL
    w = O.weights(pts, rowptr, idx.ravel(), period=per, nthreads=nthreads)
    ops = O.operators_from_stencils(n, rowptr, idx.ravel(), w)
    kw = {}
    srcs = [O.SRC_RV]
    if HV[workload]:
        w2 = O.weights(pts, rowptr, idx.ravel(), period=per, deriv_order=2, nthreads=nthreads)
        lap = O.csr_add(O.operators_from_stencils(n, rowptr, idx.ravel(), w2))
        kw = {"hv": O.ata(lap, nthreads=nthreads), "hv_gamma": 1.0 * dmin ** 4.5}
        srcs.append(O.SRC_HV_TOMINEC)
    semi = O.Semi(pts, ops, eq="euler", gamma=1.4, sources=tuple(srcs), h=davg, **kw)
    return O, semi, u0, DT_FACTOR[workload] * h, n


def cpu_baseline_oracle(workload, side, max_steps, nthreads, min_seconds=10.0,
                        single_seconds=4.0):
    """The oracle's rhs! + SSP-RK3 (-O3 build) on the host cores over a bounded number of
    steps, with all `nthreads` cores and with one (the reference's own SpMV and flux loops
    are serial).  Returns {threads: (node-rhs/s, seconds, steps)}."""
    O, semi, u0, dt, n = oracle_problem(workload, side, nthreads)
    out = {}
    for nt, budget in ((nthreads, min_seconds), (1, single_seconds)):
        hist = O.History(semi, 3)
        t0 = time.perf_counter()
        O.ssprk33(semi, u0, 0.0, dt, 1, history=hist, nthreads=nt)  # warm-up
        per_step = (time.perf_counter() - t0) / 1.33    # 4 rhs! evaluations in a 1-step call
        done = int(min(max_steps, max(1, budget / per_step)))   # a sample of ~budget s
        hist = O.History(semi, 3)
        t0 = time.perf_counter()
        O.ssprk33(semi, u0, 0.0, dt, done, history=hist, nthreads=nt)
        sec = time.perf_counter() - t0
        out[nt] = (n * RHS_PER_STEP * done / sec, sec, done)
    return out


def run_reference(args):
    ws, rank, local, pg = dist_setup()
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    O, semi, u0, dt, n = oracle_problem(args.workload, args.side, nthreads)
    hist = O.History(semi, 3)
    u, t = O.ssprk33(semi, u0, 0.0, dt, args.warmup, history=hist, nthreads=nthreads)
    t0 = time.perf_counter()
    O.ssprk33(semi, u, t, dt, args.steps, history=hist, nthreads=nthreads)
    sec = time.perf_counter() - t0
    value = n * RHS_PER_STEP * args.steps / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3 / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args.workload, n, "fp64"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "full workload, %d SSP-RK3 steps after %d warm-up"
                                   % (args.steps, args.warmup),
                         "build": _oracle_flags()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C restatement of the reference rhs! (Julia is not installed); OpenMP over rows",
    }
    print(json.dumps(line), flush=True)


def _oracle_flags():
    from oracle import build as B
    return B.flags("speed")


def config_dict(workload, n, prec, arith="dw"):
    if workload == "vortex":
        wl = ("2D Euler isentropic vortex, periodic [-5,5]^2, N=%d jittered nodes, PHS r^3 + "
              "degree-3 polynomials, k=%d, residual viscosity + history (order 3), SSP-RK3 "
              "dt=0.2h; one step = 3 rhs! evaluations" % (n, K_STENCIL))
    else:
        wl = ("2D Euler four-quadrant Riemann problem, periodic unit square, N=%d jittered nodes, "
              "PHS r^3 + degree-3 polynomials, k=%d, residual viscosity + history (order 3) + "
              "Tominec hyperviscosity (c=1), SSP-RK3 dt=0.1h; one step = 3 rhs! evaluations"
              % (n, K_STENCIL))
    return {"workload": wl, "nodes": n, "stencil": K_STENCIL, "precision": prec,
            "fp64_gather_arithmetic": arith if prec == "fp64" else None,
            "l2": "inputs larger than L2 (operator arrays ~%d MB)"
                  % (n * K_STENCIL * (60 if HV[workload] else 40) // 2 ** 20),
            "parallelism": "replicas"}


def timed_workload(args, workload, side, prec, arith, local, pg, clocks=None, dw_variant=-1):
    """Build + the timed region of one workload/form: value, per-kernel profile, end state."""
    semi, dom, u0, dt, n = build_problem(workload, side, prec, local, arith)
    from meshfree_gb300 import _lib as L
    if dw_variant >= 0:
        dom.ctx.set_option(L.OPT_DW_VARIANT, dw_variant)
    if getattr(args, "halo_rows", 0):
        dom.ctx.set_option(L.OPT_HALO_ROWS, args.halo_rows)
    dom.ctx.set_option(L.OPT_ENTRY_ORDER, getattr(args, "entry_order", 1))
    dom.ctx.set_option(L.OPT_FUSE_FLUX, getattr(args, "fuse_flux", 1))
    ms, prof, clk, u_end, ms_prof = timed_steps(dom.ctx, u0, dt, args.warmup, args.steps, pg,
                                                clocks)
    ms = max_over_ranks(pg, ms)
    return dict(semi=semi, dom=dom, u0=u0, dt=dt, n=n, ms=ms, prof=prof, clk=clk, u=u_end,
                ms_prof=ms_prof, value=n * RHS_PER_STEP * args.steps / (ms * 1e-3))


def bank_counts(ctx):
    """Serialised shared-memory accesses per quarter-warp record load of the staged
    gathers' layouts (1.0 = conflict-free), as counted when the layouts were built."""
    from meshfree_gb300 import _lib as L
    return {"fwd_gather": ctx.get_option(L.OPT_BANK_FWD) / 1000.0,
            "rev_gather": ctx.get_option(L.OPT_BANK_REV) / 1000.0}


def _kernels(prof):
    return {k: {"ms": v[0], "launches": v[1], "us_per_launch": v[0] / v[1] * 1e3}
            for k, v in prof.items()}


def run_fp32(args, local, peaks):
    """The FP32-apply form alone on the headline workload, with the gather mapping chosen
    by --gather (profiling runs of the FP32 kernels)."""
    from meshfree_gb300 import _lib as L
    semi, dom, u0, dt, n = build_problem(args.workload, args.side, "fp32", local)
    ctx = dom.ctx
    ctx.set_option(L.OPT_GATHER, {"auto": L.GATHER_AUTO, "thread": L.GATHER_THREAD,
                                  "staged": L.GATHER_STAGED,
                                  "halo": L.GATHER_HALO}[args.gather])
    ctx.set_option(L.OPT_ENTRY_ORDER, args.entry_order)
    ms, prof, _, _, ms_prof = timed_steps(ctx, u0, dt, args.warmup, args.steps, None)
    out = {"value": n * RHS_PER_STEP * args.steps / (ms * 1e-3), "unit": UNIT,
           "ms_per_step": ms / args.steps, "gather": args.gather,
           "mapping": {"fwd_gather": ctx.get_option(L.OPT_TUNED_FWD),
                       "rev_gather": ctx.get_option(L.OPT_TUNED_REV)},
           "entry_order": args.entry_order, "smem_accesses_per_quarter_load": bank_counts(ctx),
           "kernels": _kernels(prof),
           "roofline": roofline(prof, n, "fp32", HV[args.workload], peaks,
                                tag="fp32_" + args.workload)}
    ctx.close()
    return out


def run_one_form(args, local, peaks, prec, arith):
    """One form of the headline workload alone (profiling runs)."""
    r = timed_workload(args, args.workload, args.side, prec, arith, local, None,
                       dw_variant=args.dw_variant)
    from meshfree_gb300 import _lib as L
    out = {"value": r["value"], "unit": UNIT, "ms_per_step": r["ms"] / args.steps,
           "variant": {"fwd_gather": r["dom"].ctx.get_option(L.OPT_TUNED_FWD),
                       "rev_gather": r["dom"].ctx.get_option(L.OPT_TUNED_REV)},
           "halo_rows": r["dom"].ctx.get_option(L.OPT_HALO_ROWS),
           "entry_order": args.entry_order,
           "smem_accesses_per_quarter_load": bank_counts(r["dom"].ctx),
           "flux_records_formed_in_gather": r["dom"].ctx.get_option(L.OPT_FLUX_FUSED),
           "kernels": _kernels(r["prof"]),
           "roofline": roofline(r["prof"], r["n"], prec, HV[args.workload], peaks, arith,
                                tag="%s%s_%s" % (prec, arith if prec == "fp64" else "",
                                                 args.workload))}
    r["dom"].ctx.close()
    return out


def run_vortex(args, local, peaks):
    """The isentropic vortex (N = side^2, RV + history): the FP64 form (double-word
    gathers) and the FP32-apply form, their throughput over the timed steps, and each one's
    L2 density error against the exact vortex at t = 1 (this workload's own accuracy
    check), stepped with per-step graphs."""
    side = args.vortex_side
    out = {}
    ends = {}
    for prec in ("fp64", "fp32"):
        r = timed_workload(args, "vortex", side, prec, "auto", local, None)
        ends[prec] = r["u"]
        ctx, dt, n = r["dom"].ctx, r["dt"], r["n"]
        nsteps = int(round(1.0 / dt))
        ctx.history_init(3)
        ctx.set_state(r["u0"], 0.0)
        ctx.region_begin()
        ctx.ssprk33(dt, nsteps, use_graph=True)
        ms_t1 = ctx.region_end()
        u, t = ctx.get_state()
        from meshfree_gb300 import workloads as W
        ex = W.isentropic_vortex(r["dom"].pd.points, t)
        l2 = float(np.linalg.norm(u[0] - ex[0]) / np.linalg.norm(ex[0]))
        from meshfree_gb300 import _lib as L
        out[prec] = {"value": r["value"], "unit": UNIT, "ms_per_step": r["ms"] / args.steps,
                     "mapping": {"fwd_gather": ctx.get_option(L.OPT_TUNED_FWD),
                                 "rev_gather": ctx.get_option(L.OPT_TUNED_REV)},
                     "kernels": _kernels(r["prof"]),
                     "roofline": roofline(r["prof"], n, prec, False, peaks, "dw",
                                          tag="%s_vortex" % ("fp64dw" if prec == "fp64" else prec)),
                     "path_roofline": path_roofline(r["value"], prec, False, peaks),
                     "to_t1": {"steps": nsteps, "t": t, "ms": ms_t1,
                               "value": n * RHS_PER_STEP * nsteps / (ms_t1 * 1e-3),
                               "l2_density_err_vs_exact": l2}}
        ctx.close()
    out["workload"] = config_dict("vortex", side * side, "fp64")["workload"]
    out["fp32_speedup_vs_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    # the same ratio over the runs to t = 1 (~256 steps each, a longer timed region)
    out["fp32_speedup_vs_fp64_to_t1"] = out["fp32"]["to_t1"]["value"] / out["fp64"]["to_t1"]["value"]
    # the FP32 form's density against the FP64 form after the same timed steps (the
    # FP64 form equals the oracle's trajectory to 1e-10 on this workload: the -m gpu
    # full-size tests)
    d32, d64 = ends["fp32"][0], ends["fp64"][0]
    out["fp32_l2_density_err_vs_fp64"] = float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64))
    out["fp32_steps_compared"] = args.warmup + args.steps
    return out


def fma_rates(local):
    from meshfree_gb300 import _lib as L
    ctx = L.Context(local)
    r = {"fp64": ctx.fma_rate(0), "fp32": ctx.fma_rate(1)}
    ctx.close()
    return r


def run_ours(args):
    ws, rank, local, pg = dist_setup()
    peaks = load_peaks()
    peaks["fma_rates"] = fma_rates(local)
    hv = HV[args.workload]
    if args.only != "all":           # one auxiliary measurement alone (profiling runs)
        if rank == 0:
            legs = {"adjoint": lambda: run_adjoint(args, local, peaks),
                    "riemann": lambda: run_riemann(args, local),
                    "weights": lambda: run_weights(args, local),
                    "igr": lambda: run_igr(args, local),
                    "fp32": lambda: run_fp32(args, local, peaks),
                    "dw": lambda: run_one_form(args, local, peaks, "fp64", "dw"),
                    "dfma": lambda: run_one_form(args, local, peaks, "fp64", "dfma"),
                    "vortex": lambda: run_vortex(args, local, peaks),
                    "euler3d": lambda: run_euler3d(args, local, peaks),
                    "setup": lambda: run_setup(args, local),
                    "rates": lambda: {k: v / 1e9 for k, v in peaks["fma_rates"].items()}}
            leg = legs[args.only]()
            print(json.dumps({args.only: leg}), flush=True)
        return
    # headline: the FP64 form (double-word gathers) of the workload
    clocks = Clocks(local) if rank == 0 else None
    r64 = timed_workload(args, args.workload, args.side, "fp64", "auto", local, pg, clocks)
    n = r64["n"]
    value = r64["value"] * ws
    launches = sum(v[1] for v in r64["prof"].values())
    tag = "fp64dw_" + args.workload
    roof = roofline(r64["prof"], n, "fp64", hv, peaks, "dw", tag=tag)
    from meshfree_gb300 import _lib as L
    dw_variant = {"fwd_gather": r64["dom"].ctx.get_option(L.OPT_TUNED_FWD),
                  "rev_gather": r64["dom"].ctx.get_option(L.OPT_TUNED_REV)}
    dw_layout = {"entry_order": args.entry_order,
                 "smem_accesses_per_quarter_load": bank_counts(r64["dom"].ctx),
                 "flux_records_formed_in_gather": r64["dom"].ctx.get_option(L.OPT_FLUX_FUSED),
                 "halo_rows": r64["dom"].ctx.get_option(L.OPT_HALO_ROWS)}

    # the same workload with FP64 fused multiply-adds in the gathers
    rd = timed_workload(args, args.workload, args.side, "fp64", "dfma", local, pg)
    dfma = {"value": rd["value"] * ws, "unit": UNIT, "ms_per_step": rd["ms"] / args.steps,
            "dw_speedup": r64["value"] / rd["value"],
            "dw_vs_dfma_rel_l2_after_steps": [
                float(np.linalg.norm(r64["u"][v] - rd["u"][v]) / np.linalg.norm(rd["u"][v]))
                for v in range(4)],
            "kernels": _kernels(rd["prof"]),
            "roofline": roofline(rd["prof"], n, "fp64", hv, peaks, "dfma",
                                 tag="fp64dfma_" + args.workload)}
    rd["dom"].ctx.close()

    # FP32-apply form on the same workload and steps
    r32 = timed_workload(args, args.workload, args.side, "fp32", "auto", local, pg)
    from meshfree_gb300 import _lib as L
    mapping = {"fwd_gather": r32["dom"].ctx.get_option(L.OPT_TUNED_FWD),
               "rev_gather": r32["dom"].ctx.get_option(L.OPT_TUNED_REV)}
    u32, u64 = r32["u"], r64["u"]
    l2 = float(np.linalg.norm(u32[0] - u64[0]) / np.linalg.norm(u64[0]))
    linf = float(np.abs(u32[0] - u64[0]).max() / np.abs(u64[0]).max())
    value32 = r32["value"] * ws
    roof32 = roofline(r32["prof"], n, "fp32", hv, peaks, tag="fp32_" + args.workload)
    r32["dom"].ctx.close()

    # end to end through the host entry point: every step uploads u from pinned host
    # memory and downloads the new state
    import torch
    ctx = r64["dom"].ctx
    pinned = torch.empty((4, n), dtype=torch.float64, pin_memory=True)
    uh = pinned.numpy()
    uh[:] = r64["u0"]
    ctx.history_init(3)
    t = ctx.ssprk33_host(uh, 0.0, r64["dt"], 1)
    barrier(pg)
    ctx.region_begin()
    for _ in range(args.steps):
        t = ctx.ssprk33_host(uh, t, r64["dt"], 1)
    ms_e2e = max_over_ranks(pg, ctx.region_end())
    e2e = n * RHS_PER_STEP * args.steps * ws / (ms_e2e * 1e-3)
    ctx.close()

    vortex = run_vortex(args, local, peaks) if args.vortex_side > 0 and rank == 0 else None
    ens = run_ensemble(args, local, pg) if args.ens_members > 0 else None
    adj = run_adjoint(args, local, peaks) if args.adj_side > 0 and rank == 0 else None
    rie = run_riemann(args, local) if args.riemann_side > 0 and rank == 0 else None
    wts = run_weights(args, local) if args.weights_n > 0 and rank == 0 else None
    igr = run_igr(args, local) if args.igr and rank == 0 else None
    e3d = run_euler3d(args, local, peaks) if args.euler3d_side > 0 and rank == 0 else None
    setup = run_setup(args, local) if args.setup and rank == 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        res = cpu_baseline_oracle(args.workload, args.side, 400, nthreads)
        v, sec, cpu_steps = res[nthreads]
        v1, sec1, steps1 = res[1]
        cpu = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": "full N=%d, %d SSP-RK3 steps (%.1f s), oracle rhs! with OpenMP"
                         % (n, cpu_steps, sec),
               "build": _oracle_flags(),
               "single_thread": {"value": v1, "unit": UNIT, "cores": 1,
                                 "sample": "full N=%d, %d SSP-RK3 steps (%.1f s)"
                                           % (n, steps1, sec1)}}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r64["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args.workload, n, "fp64", "dw"),
        "roofline": roof,
        "path_roofline": path_roofline(value / ws, "fp64", hv, peaks),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * n * 8,
                "d2h_bytes_per_step": 4 * n * 8, "entry_point": "mft_ssprk33_host"},
        "gpu_launches": launches,
        "timing": "value: per-step CUDA graphs; kernels/roofline: same steps launched "
                  "directly with CUDA events (%.3f ms/step)" % (r64["ms_prof"] / args.steps),
        "kernels": _kernels(r64["prof"]),
        "clocks": r64["clk"],
        "fma_rates_per_s": peaks["fma_rates"],
        "dw_gather_variant": dw_variant,
        "dw_layout": dw_layout,
        "fp64_dfma": dfma,
        "fp32_apply": {"value": value32, "unit": UNIT, "speedup_vs_fp64": value32 / value,
                       "l2_density_err_vs_fp64": l2, "linf_density_err_vs_fp64": linf,
                       "steps": args.steps, "roofline": roof32,
                       "path_roofline": path_roofline(value32 / ws, "fp32", hv, peaks),
                       "autotuned_mapping": mapping, "kernels": _kernels(r32["prof"])},
        "vortex": vortex,
        "ensemble": ens,
        "adjoint": adj,
        "riemann_to_t02": rie,
        "weights_batch": wts,
        "igr": igr,
        "euler3d": e3d,
        "setup": setup,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
