"""Benchmark: FMM force evaluation at N = 1M Plummer, p = 4, n_max = 32.

Metric (one JSON line on rank 0): bodies/s of one FMM force evaluation of the
mixed-precision form (FP32 P2M/L2P/P2P, FP32 M2L, FP64 state) in ACCURATE mode
(near/far lists by the opening angle theta on the reference's Morton tree,
median relative force error <= 1e-4 against the exact FP64 N^2 sum), with the
FP64 form and the reference-semantics (REF) FP64 form timed beside it, the force
error of each against the FP64 N^2 sum on 1000 seeded sample bodies, whole
leapfrog steps with a static and with a per-step rebuilt tree, and the
adjoint/forward time of reverse-mode rollouts.

  value      whole-job bodies/s with bodies resident in HBM (CUDA events on the
             context stream, L2 flushed by a 256 MB write before every step,
             outside the step's timed interval)
  e2e        the same through the C ABI call gx_compute_forces with pinned host
             buffers: each step moves x, y, m host->device and ax, ay back over
             the host link (read and written by the first and last kernels of
             the evaluation, the arrays being page-locked), timed on the host
  roofline   the dominant kernel (P2P, FP32 pipe): algorithmic FLOPs (14 per
             body-body interaction) per launch / its event-timed duration in the
             timed evaluations (where it shares the SMs with the far-field chain),
             against the FP32 FMA peak measured on this GPU in the same run; the
             *_alone keys time it again started after that chain
  cpu_baseline  the oracle (C restatement of galax-core's CPU FMM, REF semantics,
             OpenMP where the reference uses Rayon) on the host cores
  kdk_steps  leapfrog steps/s, static tree and tree rebuilt every step (the latter
             also with theta_b = 0: no body-level P2L mask plan per tree)
  uniform_10k  the uniform N=10,000 case: 10 leapfrog steps/s of the REF FP64,
             ACCURATE FP64 and mixed forms, force errors against the exact N^2 sum,
             and the oracle's steps/s and end-state difference (CPU leg)
  adjoint    galaxy N=200,001 x 100 steps (FP64 and mixed, finite differences with
             the tree sequence frozen) and Plummer N=1M x 500 steps (mixed,
             checkpoint interval sweep, peak device bytes), both rebuilding the
             tree every step

``--impl reference`` times the reference's CPU algorithm (the oracle port) on the
same workload instead.  ``--sweep disk`` (p x n_max on the 4M disk preset),
``--sweep theta`` (opening angle on the Plummer workload) and ``--build-only``
(device tree builds and plans) print their own JSON lines.  Multi-GPU: the force evaluation does not shard here, so
``--gpus N`` runs N independent replicas (weak scaling); timing is the max over
ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FMM bodies/s (1M, p=4) mixed vs FP64 at equal force error; adjoint/fwd time"
N_DEFAULT = 1_000_000
# DRAM bytes of one k_p2p32_rows launch at the default workload (theta_w = 0.4), the mean
# of two launches of a one-pass ncu capture (dram__bytes_read.sum + dram__bytes_write.sum:
# 34.92 + 1.14 MB and 34.88 + 0.49 MB): the kernel works out of L2
P2P_TRAFFIC_1M = 35.72e6
# the same for k_p2p32_stream (the body-level P2L on, theta_b = 0.3): 50.4 + 4.1 MB and
# 50.5 + 2.7 MB
P2P_STREAM_TRAFFIC_1M = 53.85e6
P, N_MAX, THETA = 4, 32, 0.5
# leaf-level near-list split (M2P / P2L) of the ACCURATE forms: near leaf pairs that are
# far on one side at this opening angle leave P2P
THETA_W = 0.4
# body-level P2L of the P2P pairs the split leaves: source bodies with
# |x_j - com_a| theta_b > R_a join the target leaf's local expansion (0 = off); at 0.3
# the error against the exact sum is that of the split alone (--sweep thetab)
THETA_B = 0.3


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def _barrier(pg):
    if pg is not None:
        pg.barrier()


def _max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms."""

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self._p = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                        "--format=csv,noheader,nounits", "-lms", "20"], stdout=subprocess.PIPE,
                                       stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self._p = None

    def _read(self):
        for line in self._p.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self._p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self._p.terminate()
        try:
            self._p.wait(timeout=5)
        except Exception:
            self._p.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 9 for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def _rel_err(ax, ay, rx, ry):
    den = np.maximum(np.hypot(rx, ry), 1e-30)
    return np.hypot(ax - rx, ay - ry) / den


def _err_stats(ax, ay, rx, ry):
    """Vector metric |a - a*| / |a*| (median, p99) and the reference's magnitude metric
    ||a| - |a*|| / max(|a*|, 1e-20) (validate_fmm, galax-core lib.rs:1553-1557: mean, max)."""
    e = _rel_err(ax, ay, rx, ry)
    am, rm = np.hypot(ax, ay), np.hypot(rx, ry)
    mag = np.abs(am - rm) / np.maximum(rm, 1e-20)
    return {"err_median": float(np.median(e)), "err_p99": float(np.percentile(e, 99)),
            "err_mag_mean": float(np.mean(mag)), "err_mag_max": float(np.max(mag))}


def _cpu_baseline(bodies_sorted, bounds, eps, n_evals: int = 2):
    """The oracle (REF semantics) on the host: full force evaluations of the same workload."""
    from oracle import oracle as O
    O.build()
    ob = O.Bodies.from_arrays(bodies_sorted.x, bodies_sorted.y, bodies_sorted.mass)
    t = O.tree_build(ob, N_MAX, bounds)
    v, u = O.vlist_build(t), O.ulist_build(t)
    times = []
    bb = None
    for _ in range(n_evals):
        bb = ob.copy()
        t0 = time.perf_counter()
        O.compute_fmm_force(bb, t, v, u, P, eps, O.MODE_REF)
        times.append(time.perf_counter() - t0)
    return ob, t, v, u, times, O.get_threads(), bb


def run_reference(args, rank, world, pg):
    """--impl reference: the reference's CPU FMM (oracle port) on the host cores."""
    if rank != 0:
        return 0
    from galax_gb300 import presets
    from oracle import oracle as O
    O.build()
    n = args.n
    b = presets.plummer(n, seed=args.seed)
    bounds = presets.BOUNDS["plummer"]
    ob = O.Bodies.from_arrays(b.x, b.y, b.mass, b.vx, b.vy)
    t = O.tree_build(ob, N_MAX, bounds)
    v, u = O.vlist_build(t), O.ulist_build(t)
    eps = O.cli_softening(ob)
    for _ in range(args.warmup):
        bb = ob.copy()
        O.compute_fmm_force(bb, t, v, u, P, eps, O.MODE_REF)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bb = ob.copy()
        O.compute_fmm_force(bb, t, v, u, P, eps, O.MODE_REF)
    dt = (time.perf_counter() - t0) / args.steps
    value = n / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "bodies/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Plummer preset)",
        "config": {"workload": f"plummer N={n}, p={P}, n_max={N_MAX}, REF semantics (galax-core compute_fmm_force)",
                   "n": n, "p": P, "n_max": N_MAX},
        "cpu_baseline": {"value": value, "unit": "bodies/s", "cores": O.get_threads(), "kind": "port",
                         "sample": f"{args.steps} full force evaluations at N={n} (tree and lists built once, "
                                   f"outside the timed region)"},
        "e2e": {"value": value, "unit": "bodies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _rot(theta):
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c, -s], [s, c]])


def _adjoint_run(G, ctx, b, T, dt, k, R, rebuild=0):
    """One forward rollout and its reverse pass; returns times, gradients and peak bytes."""
    n = len(b)
    ctx.upload_bodies(b)
    t0 = time.perf_counter()
    ctx.rollout_forward(T, dt, k, rebuild)
    t_fwd = time.perf_counter() - t0
    fin = G.Bodies.new(n)
    ctx.download_bodies(fin)
    ids = ctx.body_ids() if rebuild else None
    from galax_gb300.fdcheck import rollout_loss
    L, lxT, lyT, dx0, dy0 = rollout_loss(b.x, b.y, fin.x, fin.y, R, ids)
    z = np.zeros(n)
    t0 = time.perf_counter()
    gx, gy, gvx, gvy, gm, peak = ctx.rollout_backward(lxT, lyT, z, z)
    t_bwd = time.perf_counter() - t0
    return t_fwd, t_bwd, (gx + dx0, gy + dy0, gvx, gvy, gm), peak, L


def run_uniform10k(G, presets, args, with_cpu: bool):
    """Config 1: uniform N=10,000 in [0,100]^2, p=4, n_max=32, CLI softening, 10 leapfrog
    steps with the static tree at dt = 0.5/sqrt(max|a|).  Steps/s of the REF FP64 form
    (reference semantics) and of the ACCURATE FP64 and mixed forms, each form's initial
    force error against the exact FP64 N^2 sum over all bodies; with the CPU leg, the
    oracle's REF simulate of the same steps on the host cores and the largest difference
    of the GPU REF end state from it."""
    n, T = 10_000, 10
    bounds = presets.BOUNDS["uniform"]
    gb = presets.uniform(n, seed=0)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=P, eps64=0.1))
    ctx.set_near_split(args.theta_w)
    ctx.set_body_split(args.theta_b)
    ctx.build_tree(gb, N_MAX, bounds)  # permutes gb into Morton order, as Tree::build does
    eps = presets.cli_softening(gb.x, gb.y)
    ctx.set_params(P, eps)
    idx = np.arange(n)
    ex, ey = ctx.n2_sampled(idx)
    out = {"workload": f"uniform N={n} in [0,100]^2, p={P}, n_max={N_MAX}, {T} KDK steps, static tree", "eps": eps}
    end = {}
    for name, mode, prec in (("ref_fp64", G.MODE_REF, G.PREC_FP64), ("accurate_fp64", G.MODE_ACCURATE, G.PREC_FP64),
                             ("accurate_mixed", G.MODE_ACCURATE, G.PREC_MIXED)):
        ctx.set_mode(mode, prec, THETA)
        ctx.upload_bodies(gb)
        ctx.forces_resident()
        a0 = G.Bodies.new(n)
        ctx.download_bodies(a0)
        if name == "ref_fp64":
            dt = presets.cli_dt(a0.ax, a0.ay)
            out["dt"] = dt
        row = _err_stats(a0.ax, a0.ay, ex, ey)
        ts = []
        for r in range(3):  # the first run is a warm-up
            ctx.upload_bodies(gb)
            ctx.forces_resident()
            t0 = time.perf_counter()
            ctx.kdk_run(T, dt, 0)
            ts.append(time.perf_counter() - t0)
        row.update({"steps_per_s": T / float(np.mean(ts[1:])), "ms_per_step": float(np.mean(ts[1:])) / T * 1e3})
        fin = G.Bodies.new(n)
        ctx.download_bodies(fin)
        end[name] = fin
        out[name] = row
    ctx.close()
    if with_cpu:
        from oracle import oracle as O
        O.build()
        ob = O.Bodies.from_arrays(gb.x, gb.y, gb.mass)
        t = O.tree_build(ob, N_MAX, bounds)
        v, u = O.vlist_build(t), O.ulist_build(t)
        O.compute_fmm_force(ob, t, v, u, P, eps, O.MODE_REF)  # initial forces (galax-cli/src/main.rs:230)
        t0 = time.perf_counter()
        O.simulate(ob, t, v, u, P, eps, out["dt"], T, 0, O.MODE_REF)
        tc = time.perf_counter() - t0
        g = end["ref_fp64"]
        sc, vs = float(np.max(np.abs(ob.x))), float(np.max(np.hypot(ob.vx, ob.vy)))
        out["cpu_baseline"] = {"steps_per_s": T / tc, "cores": O.get_threads(), "kind": "port",
                               "sample": f"{T} REF KDK steps of the same bodies (oracle simulate)"}
        out["ref_fp64"]["end_state_max_rel_diff_vs_oracle"] = max(
            float(np.max(np.abs(g.x - ob.x))) / sc, float(np.max(np.abs(g.y - ob.y))) / sc,
            float(np.max(np.abs(g.vx - ob.vx))) / vs, float(np.max(np.abs(g.vy - ob.vy))) / vs)
    return out


def _grad_rel(g, r):
    return float(max(np.linalg.norm(a - c) / max(np.linalg.norm(c), 1e-300) for a, c in zip(g, r)))


def run_adjoint(G, presets, ctx1m, b1m, args):
    """Reverse-mode rollouts: galaxy N=200,001 x 100 steps (FP64 and mixed; central
    finite differences of the FP64 rollout along seeded directions) and Plummer N=1M x
    500 steps at dt=1e-3 (mixed; checkpoint interval sweep, gradient against the FP64
    GPU adjoint on a 20-step prefix).  The comparison with the exact FP64 N^2 adjoint
    on a 2000-body subset is a test (tests/test_gpu_adjoint.py)."""
    out = {}
    # ---- galaxy, N = 200,001, 100 steps at the CLI time step.  The inner orbits
    # (R = 1, v = 31.6) cross many leaves per step, and with a static tree the
    # expansions diverge within ~30 steps (the oracle does the same), so the tree is
    # rebuilt on the device before every step's force evaluation.
    n, T = 200_001, 100
    bounds = presets.BOUNDS["galaxy"]
    bg = presets.galaxy(n, seed=args.seed + 4)
    cg = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 24, p=P, eps64=0.1))
    cg.build_tree(bg, N_MAX, bounds)
    eps = presets.cli_softening(bg.x, bg.y)
    cg.set_params(P, eps)
    cg.set_mode(G.MODE_ACCURATE, G.PREC_FP64, THETA)
    cg.upload_bodies(bg)
    cg.forces_resident()
    a0 = G.Bodies.new(n)
    cg.download_bodies(a0)
    dt = presets.cli_dt(a0.ax, a0.ay)
    R = _rot(float(np.random.default_rng(args.seed + 5).uniform(0, 2 * np.pi)))
    k = 10
    gal = {"workload": f"galaxy N={n}, p={P}, n_max={N_MAX}, {T} steps, dt={dt:.4g} (CLI rule), tree rebuilt "
                       f"every step, checkpoint every {k} steps", "eps": eps}
    grads = {}
    for name, prec in (("fp64", G.PREC_FP64), ("mixed", G.PREC_MIXED)):
        cg.set_mode(G.MODE_ACCURATE, prec, THETA)
        _adjoint_run(G, cg, bg, 3, dt, k, R, rebuild=1)  # warm-up
        tf, tb, g, peak, L = _adjoint_run(G, cg, bg, T, dt, k, R, rebuild=1)
        grads[name] = g
        gal[name] = {"fwd_s": tf, "bwd_s": tb, "adjoint_over_forward": tb / tf, "peak_bytes": peak,
                     "steps_per_s_forward": T / tf}
    gal["mixed"]["grad_rel_err_vs_fp64"] = _grad_rel(grads["mixed"], grads["fp64"])
    # central finite differences of the FP64 rollout, h = 1e-6, seeded directions, with
    # every step's tree taken from the unperturbed trajectory (the function the adjoint
    # differentiates; a perturbation of 1e-6 reorders bodies across Morton cells)
    from galax_gb300 import fdcheck
    cg.set_mode(G.MODE_ACCURATE, G.PREC_FP64, THETA)
    rng = np.random.default_rng(args.seed + 6)
    h = 1e-6
    dirs = [[rng.standard_normal(n) for _ in range(4)] + [rng.standard_normal(n) * bg.mass]
            for _ in range(args.fd_dirs)]
    num = fdcheck.fd_frozen_trees(G, cg, bg, T, dt, R, dirs, h, N_MAX, bounds, rebuild=True) if dirs else []
    g = grads["fp64"]
    fd = [abs(num[i] - sum(float(np.dot(g[q], dirs[i][q])) for q in range(5))) / abs(num[i]) for i in range(len(dirs))]
    gal["fp64"]["fd_rel_err_max"] = float(max(fd)) if fd else None
    gal["fp64"]["fd_directions"] = args.fd_dirs
    cg.close()
    out["galaxy_200k"] = gal

    # ---- Plummer 1M, 500 steps at dt = 1e-3, mixed, checkpoint sweep.  Core bodies
    # cross ~80 leaf widths in 500 steps; with a static tree the run diverges, so the
    # tree is rebuilt before every step's force evaluation here too.
    T, dt = args.adj_steps, 1e-3
    Rp = _rot(float(np.random.default_rng(args.seed + 8).uniform(0, 2 * np.pi)))
    ctx1m.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, THETA)
    # the stated device-memory budget of the checkpointed rollout: checkpoints, the
    # kept trees of a segment, permutations and adjoint buffers must fit in it
    budget = args.hbm_budget_gb * 1e9
    sweep = {}
    for k in args.adj_k:
        _adjoint_run(G, ctx1m, b1m, 3, dt, k, Rp, rebuild=1)  # warm-up (allocations)
        tf, tb, g, peak, L = _adjoint_run(G, ctx1m, b1m, T, dt, k, Rp, rebuild=1)
        sweep[str(k)] = {"fwd_s": tf, "bwd_s": tb, "adjoint_over_forward": tb / tf, "peak_bytes": peak,
                         "within_hbm_budget": bool(peak <= budget),
                         "finite": bool(all(np.all(np.isfinite(a)) for a in g)) and bool(np.isfinite(L))}
    # gradient of a 20-step prefix: mixed against FP64 (the FP64 form is ~50x slower)
    Tp = 20
    _, _, gm20, _, _ = _adjoint_run(G, ctx1m, b1m, Tp, dt, 5, Rp, rebuild=1)
    ctx1m.set_mode(G.MODE_ACCURATE, G.PREC_FP64, THETA)
    _, _, g64, _, _ = _adjoint_run(G, ctx1m, b1m, Tp, dt, 5, Rp, rebuild=1)
    fit = [int(k) for k, r in sweep.items() if r["within_hbm_budget"]]
    pl = {"workload": f"plummer N={len(b1m)}, p={P}, n_max={N_MAX}, {T} steps, dt={dt}, mixed, tree rebuilt every step",
          "hbm_budget_bytes": budget, "checkpoint_sweep": sweep,
          "fastest_within_budget": (min(fit, key=lambda k: sweep[str(k)]["adjoint_over_forward"]) if fit else None),
          "grad_rel_err_mixed_vs_fp64_20_steps": _grad_rel(gm20, g64)}
    if args.fd_dirs_1m > 0:
        # central differences of the FP64 20-step prefix along seeded directions, trees
        # frozen along the unperturbed trajectory; compared with both adjoints
        from galax_gb300 import fdcheck
        n1 = len(b1m)
        rng = np.random.default_rng(args.seed + 9)
        dirs = [[rng.standard_normal(n1) for _ in range(4)] + [rng.standard_normal(n1) * b1m.mass]
                for _ in range(args.fd_dirs_1m)]
        num = fdcheck.fd_frozen_trees(G, ctx1m, b1m, Tp, dt, Rp, dirs, 1e-6, N_MAX, presets.BOUNDS["plummer"],
                                      rebuild=True)
        for key, g in (("fp64", g64), ("mixed", gm20)):
            err = [abs(num[i] - sum(float(np.dot(g[q], dirs[i][q])) for q in range(5))) / abs(num[i])
                   for i in range(len(dirs))]
            pl[f"fd_rel_err_max_20_steps_{key}"] = float(max(err))
        pl["fd_directions_20_steps"] = args.fd_dirs_1m
    ctx1m.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, THETA)
    out["plummer_1m"] = pl
    return out



def run_disk_compact(G, presets, args):
    """The disk workload (N = 4,000,000, n_max = 32) at p in {2,4,6,8}: ms per force
    evaluation of the mixed and FP64 forms (L2 flushed) and their errors against the
    FP64 N^2 sum on 1000 seeded samples.  ``--sweep disk`` adds n_max 16 and 64."""
    n, n_max = args.sweep_n, 32
    bounds = presets.BOUNDS["disk"]
    b = presets.disk(n, seed=args.seed + 3)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 28, p=8, eps64=0.1))
    ctx.set_near_split(args.theta_w)
    ctx.set_body_split(args.theta_b)
    ctx.build_tree(b, n_max, bounds)
    eps = presets.cli_softening(b.x, b.y)
    ctx.upload_bodies(b)
    idx = np.sort(np.random.default_rng(4321).choice(n, min(1000, n), replace=False))
    rows = []
    for p in (2, 4, 6, 8):
        ctx.set_params(p, eps)
        ex, ey = ctx.n2_sampled(idx)
        for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
            ctx.set_mode(G.MODE_ACCURATE, prec, THETA)
            ctx.forces_resident()
            ms, _ = ctx.bench_forces(3 if name == "mixed" else 1, True, 0)
            r = G.Bodies.new(n)
            ctx.download_bodies(r)
            row = {"p": p, "form": name, "ms": float(np.mean(ms)), "bodies_per_s": n / (float(np.mean(ms)) * 1e-3)}
            row.update(_err_stats(r.ax[idx], r.ay[idx], ex, ey))
            rows.append(row)
    ctx.close()
    return {"workload": f"disk N={n}, n_max={n_max}, theta={THETA}, theta_w={args.theta_w}, ACCURATE", "eps": eps,
            "rows": rows}


def run_build_only(args):
    """Tree construction (device Morton keys, radix sort, permutation, leaves and parent
    rounds) over resident Plummer bodies, then the ACCURATE plan of the new tree, a few
    times: the workload of the tree-build profile.  Prints one JSON line with the
    host-timed rebuilds and plans, and the REF form's lists and plan on the last tree."""
    import galax_gb300 as G
    from galax_gb300 import build as gbuild
    from galax_gb300 import presets
    gbuild.build()
    n = args.n
    b = presets.plummer(n, seed=args.seed)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 28, p=P, eps64=0.1))
    ctx.build_tree(b.copy(), N_MAX, presets.BOUNDS["plummer"])
    ctx.set_params(P, presets.cli_softening(b.x, b.y))
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, THETA)
    ctx.set_near_split(args.theta_w)
    ctx.set_body_split(args.theta_b)
    times, plan = [], []
    for _ in range(max(1, args.steps)):
        ctx.upload_bodies(b)  # unsorted order again: the sort does full work
        t0 = time.perf_counter()
        ctx.rebuild_resident(N_MAX, presets.BOUNDS["plummer"])
        t1 = time.perf_counter()
        ctx.forces_resident()  # the ACCURATE plan of the new tree, then one evaluation
        t2 = time.perf_counter()
        ctx.forces_resident()
        t3 = time.perf_counter()
        times.append(t1 - t0)
        plan.append((t2 - t1) - (t3 - t2))
    # REF form on the last tree: its V/U lists, P2P gather lists and derivative plan
    ctx.set_mode(G.MODE_REF, G.PREC_FP64, THETA)
    t0 = time.perf_counter()
    ctx.forces_resident()
    t1 = time.perf_counter()
    ctx.forces_resident()
    t2 = time.perf_counter()
    ref_plan = (t1 - t0) - (t2 - t1)
    nn, nl, lv, _ = ctx.tree_info()
    ctx.close()
    print(json.dumps({"build_only": True, "n": n, "theta_w": args.theta_w, "nodes": nn, "leaves": nl, "levels": lv,
                      "build_ms": [t * 1e3 for t in times], "plan_ms": [t * 1e3 for t in plan],
                      "ref_plan_ms": ref_plan * 1e3, "ref_eval_ms": (t2 - t1) * 1e3}), flush=True)
    return 0


def run_sweep_disk(args):
    """Accuracy/throughput sweep on the disk preset (N = 4,000,000 by default):
    p in {2,4,6,8} x n_max in {16,32,64}, mixed and FP64 forms, errors against the FP64
    N^2 sum on 1000 seeded samples.  Prints one JSON line."""
    import galax_gb300 as G
    from galax_gb300 import build as gbuild
    from galax_gb300 import presets
    gbuild.build()
    n = args.sweep_n
    bounds = presets.BOUNDS["disk"]
    b0 = presets.disk(n, seed=args.seed + 3)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 28, p=8, eps64=0.1))
    rows = []
    for n_max in (16, 32, 64):
        b = b0.copy()
        ctx.build_tree(b, n_max, bounds)
        eps = presets.cli_softening(b.x, b.y)
        ctx.upload_bodies(b)
        idx = np.sort(np.random.default_rng(4321).choice(n, min(1000, n), replace=False))
        for p in (2, 4, 6, 8):
            ctx.set_params(p, eps)
            ex, ey = ctx.n2_sampled(idx)
            for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
                ctx.set_mode(G.MODE_ACCURATE, prec, THETA)
                ctx.forces_resident()
                reps = 3 if name == "mixed" else 1
                ms, _ = ctx.bench_forces(reps, True, 0)
                r = G.Bodies.new(n)
                ctx.download_bodies(r)
                far, near, inter = ctx.plan_info()
                row = {"n_max": n_max, "p": p, "form": name, "ms": float(np.mean(ms)),
                       "bodies_per_s": n / (float(np.mean(ms)) * 1e-3), "far_pairs": far,
                       "near_leaf_pairs": near, "p2p_interactions": inter,
                       "tiles": {"m2l": f"warp per unit of <= 256 far sources of one target node, lane per source; "
                                        f"C(p)={(p + 1) * (p + 2) // 2} coefficients, "
                                        f"{(2 * p + 1) * (2 * p + 2) // 2} derivatives per pair",
                                 "p2p": f"warp per item (target leaf of <= {n_max} bodies x <= 32 source leaves)"}}
                row.update(_err_stats(r.ax[idx], r.ay[idx], ex, ey))
                rows.append(row)
    ctx.close()
    print(json.dumps({"sweep": "disk", "n": n, "theta": THETA, "seed": args.seed + 3, "rows": rows}), flush=True)
    return 0


def run_sweep_theta(args):
    """Opening-angle sweep on the Plummer workload (N = 1,000,000 by default, p = 4,
    n_max = 32): for each theta the near/far split, the evaluation time of the mixed and
    FP64 forms and their errors against the FP64 N^2 sum on 1000 seeded samples.  The
    headline uses theta = 0.5.  Prints one JSON line."""
    import galax_gb300 as G
    from galax_gb300 import build as gbuild
    from galax_gb300 import presets
    gbuild.build()
    n = args.n
    b = presets.plummer(n, seed=args.seed)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 28, p=P, eps64=0.1))
    ctx.build_tree(b, N_MAX, presets.BOUNDS["plummer"])
    ctx.set_params(P, presets.cli_softening(b.x, b.y))
    ctx.upload_bodies(b)
    idx = np.sort(np.random.default_rng(1234).choice(n, min(1000, n), replace=False))
    ex, ey = ctx.n2_sampled(idx)
    rows = []
    for theta in (0.3, 0.4, 0.5, 0.6, 0.7):
        for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
            ctx.set_mode(G.MODE_ACCURATE, prec, theta)
            ctx.forces_resident()
            ms, _ = ctx.bench_forces(10 if name == "mixed" else 1, True, 0)
            r = G.Bodies.new(n)
            ctx.download_bodies(r)
            far, near, inter = ctx.plan_info()
            row = {"theta": theta, "form": name, "ms": float(np.mean(ms)),
                   "bodies_per_s": n / (float(np.mean(ms)) * 1e-3), "far_pairs": far, "near_leaf_pairs": near,
                   "p2p_interactions": inter}
            row.update(_err_stats(r.ax[idx], r.ay[idx], ex, ey))
            rows.append(row)
    ctx.close()
    print(json.dumps({"sweep": "theta", "n": n, "p": P, "n_max": N_MAX, "seed": args.seed, "rows": rows}), flush=True)
    return 0


def run_sweep_thetaw(args):
    """Near-list split sweep on the Plummer workload (N = 1,000,000, p = 4, n_max = 32):
    at theta = 0.5 for each theta_w (0 = no split), and at the --sweep-thetas opening angles
    for theta_w in {0.3, 0.35, 0.4}, the P2P, M2P and P2L pair counts, the
    evaluation time of the mixed and FP64 forms, the P2P kernel alone, and the errors
    against the FP64 N^2 sum on 1000 seeded samples.  Prints one JSON line."""
    import galax_gb300 as G
    from galax_gb300 import build as gbuild
    from galax_gb300 import presets
    gbuild.build()
    n = args.n
    b = presets.plummer(n, seed=args.seed)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 28, p=P, eps64=0.1))
    ctx.build_tree(b, N_MAX, presets.BOUNDS["plummer"])
    ctx.set_params(P, presets.cli_softening(b.x, b.y))
    ctx.upload_bodies(b)
    idx = np.sort(np.random.default_rng(1234).choice(n, min(1000, n), replace=False))
    ex, ey = ctx.n2_sampled(idx)
    rows = []
    if args.sweep == "thetab":
        grid = [(THETA, tw, tb) for tw in (0.35, 0.4, 0.45) for tb in (0.0, 0.25, 0.3, 0.35)]
    else:
        grid = [(THETA, tw, 0.0) for tw in (0.0, 0.3, 0.35, 0.4, 0.45, 0.5)]
        grid += [(th, tw, 0.0) for th in args.sweep_thetas for tw in (0.3, 0.35, 0.4) if th != THETA]
    for theta, tw, tb in grid:
        ctx.set_near_split(tw)
        ctx.set_body_split(tb)
        # the FP64 form has the mixed form's error (to the third digit); it is timed at the
        # headline opening angle only
        forms = (("mixed", G.PREC_MIXED),)
        if theta == THETA and args.sweep != "thetab":
            forms += (("fp64", G.PREC_FP64),)
        for name, prec in forms:
            ctx.set_mode(G.MODE_ACCURATE, prec, theta)
            ctx.forces_resident()
            ms, kms = ctx.bench_forces(10 if name == "mixed" else 1, True, 0)
            r = G.Bodies.new(n)
            ctx.download_bodies(r)
            far, near, inter = ctx.plan_info()
            m2p, p2l = ctx.plan_split_info()
            moved, body_evals = ctx.plan_body_split_info()
            row = {"theta": theta, "theta_w": tw, "theta_b": tb, "p2p_moved_to_body_p2l": moved,
                   "body_p2l_evaluations": body_evals, "form": name, "ms": float(np.mean(ms)),
                   "p2p_kernel_ms": float(np.mean(kms)),
                   "pass_ms": ctx.last_timings().tolist(), "bodies_per_s": n / (float(np.mean(ms)) * 1e-3),
                   "far_pairs": far, "near_p2p_leaf_pairs": near, "m2p_leaf_pairs": m2p, "p2l_leaf_pairs": p2l,
                   "p2p_interactions": inter - moved}
            if name == "mixed":
                _, kal = ctx.bench_forces(5, True, 2)
                row["p2p_kernel_ms_alone"] = float(np.mean(kal))
            row.update(_err_stats(r.ax[idx], r.ay[idx], ex, ey))
            rows.append(row)
    ctx.close()
    print(json.dumps({"sweep": "theta_w" if args.sweep != "thetab" else "theta_b", "n": n, "p": P, "n_max": N_MAX, "theta": THETA, "seed": args.seed,
                      "rows": rows}), flush=True)
    return 0


def run_ours(args, rank, world, local, pg):
    import galax_gb300 as G
    from galax_gb300 import build as gbuild
    from galax_gb300 import presets
    gbuild.build()
    n = args.n
    bounds = presets.BOUNDS["plummer"]
    b = presets.plummer(n, seed=args.seed)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 28, p=P, eps64=0.1, device=local))
    gb = b.copy()
    t0 = time.perf_counter()
    ctx.build_tree(gb, N_MAX, bounds)
    setup_tree_s = time.perf_counter() - t0
    eps = presets.cli_softening(gb.x, gb.y)
    ctx.set_params(P, eps)
    ctx.upload_bodies(gb)
    nn, nl, nlev, _ = ctx.tree_info()

    ctx.set_near_split(args.theta_w)  # ACCURATE forms only; REF keeps the reference's lists
    ctx.set_body_split(args.theta_b)
    forms = [("mixed", G.MODE_ACCURATE, G.PREC_MIXED), ("fp64", G.MODE_ACCURATE, G.PREC_FP64),
             ("ref_fp64", G.MODE_REF, G.PREC_FP64)]
    res = {}
    clocks = None
    for name, mode, prec in forms:
        ctx.set_mode(mode, prec, THETA)
        t0 = time.perf_counter()
        ctx.forces_resident()  # builds the static plan (lists) for this mode once
        plan_s = time.perf_counter() - t0
        steps = args.steps if name == "mixed" else max(3, min(args.steps, 5))
        warm = args.warmup if name == "mixed" else 1
        ctx.bench_forces(warm, True, 0)
        sampler = None
        if name == "mixed" and rank == 0:
            sampler = ClockSampler(local)
            sampler.start()
        _barrier(pg)
        ms, kms = ctx.bench_forces(steps, True, 0)
        _barrier(pg)
        if sampler is not None:
            clocks = sampler.stop()
        far, near, inter = ctx.plan_info()
        moved, body_evals = ctx.plan_body_split_info() if mode == G.MODE_ACCURATE else (0, 0)
        bb = G.Bodies.new(n)
        ctx.download_bodies(bb)
        # P2P interactions left after the body-level P2L moved `moved` of them
        res[name] = dict(ms=ms, kms=kms, plan_s=plan_s, far=far, near=near, inter=inter - moved, moved=moved,
                         body_evals=body_evals,
                         launches=ctx.last_launch_count(), passes=ctx.last_timings().tolist(),
                         ax=bb.ax.copy(), ay=bb.ay.copy(), steps=steps)
        if name == "ref_fp64":
            # the device tree and the reference's V/U lists of this workload, for the
            # bit-for-bit comparison with the oracle in the CPU leg
            dev_tree = ctx.export_tree()
            dev_lists = (ctx.export_lists(G.LIST_V), ctx.export_lists(G.LIST_U))

    # force error of each form against the exact FP64 N^2 sum (GPU n2 kernel), 1000 seeded samples
    idx = np.sort(np.random.default_rng(1234).choice(n, min(1000, n), replace=False))
    ex, ey = ctx.n2_sampled(idx)
    for name in res:
        res[name].update(_err_stats(res[name]["ax"][idx], res[name]["ay"][idx], ex, ey))
    d = _rel_err(res["mixed"]["ax"], res["mixed"]["ay"], res["fp64"]["ax"], res["fp64"]["ay"])

    # end to end through the C ABI with pinned host buffers (mixed form)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, THETA)
    hx, hy, hm, hax, hay = (G.HostArray(n) for _ in range(5))
    hx.array[:] = gb.x
    hy.array[:] = gb.y
    hm.array[:] = gb.mass
    for _ in range(max(1, args.warmup)):
        ctx.compute_forces(hx.array, hy.array, hm.array, hax.array, hay.array)
    _barrier(pg)
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.compute_forces(hx.array, hy.array, hm.array, hax.array, hay.array)
        e2e_t.append(time.perf_counter() - t0)
    _barrier(pg)
    e2e_ms = _max_over_ranks(pg, float(np.mean(e2e_t)) * 1e3)
    # the P2P kernel once more, started after the far-field chain so that it runs alone
    _, k_alone = ctx.bench_forces(max(3, args.steps // 2), True, 2)
    peak32 = ctx.probe_fp32_tflops()

    # whole steps (kick, drift, forces, kick) with the static tree and with the tree
    # rebuilt on the device before every force evaluation (mixed form, dt = 1e-3); the
    # rebuild also without the body-level P2L, whose mask plan is redone for every tree
    steps_cmp = {}
    runs = [(0, args.theta_b, "static_tree"), (1, args.theta_b, "rebuild_every_step")]
    if args.theta_b > 0:
        runs.append((1, 0.0, "rebuild_every_step_theta_b_0"))
    for rb, tb, key in runs:
        ctx.set_body_split(tb)
        ctx.upload_bodies(gb)
        if rb:
            ctx.rebuild_resident(N_MAX, bounds)
        ctx.forces_resident()
        ctx.kdk_run(2, 1e-3, 0, rebuild_every=rb)  # warm-up
        _barrier(pg)
        t0 = time.perf_counter()
        ctx.kdk_run(args.steps, 1e-3, 0, rebuild_every=rb)
        t_s = (time.perf_counter() - t0) / args.steps
        steps_cmp[key] = {"ms_per_step": t_s * 1e3, "bodies_per_s": n / t_s, "steps_per_s": 1.0 / t_s,
                          "theta_b": tb}
    ctx.set_body_split(args.theta_b)
    ctx.upload_bodies(gb)
    ctx.rebuild_resident(N_MAX, bounds)  # back to the tree of the starting positions (gb is in its order)

    adjoint = None
    if not args.no_adjoint and world == 1:
        ctx.set_near_split(0.0)  # the adjoint transposes P2P, M2L, L2L and L2P, not M2P / P2L
        adjoint = run_adjoint(G, presets, ctx, gb, args)
    mix = res["mixed"]
    ms_step = _max_over_ranks(pg, float(np.mean(mix["ms"])))
    kms = float(np.mean(mix["kms"]))
    flops = 14.0 * mix["inter"]
    achieved = flops / (kms * 1e-3) / 1e12
    # the whole evaluation's FP32 work (P2P and the M2L contraction, 2 C(p)^2 = 450 FLOP
    # per far pair) over its event time: P2P shares the SMs with M2L while it runs
    eval_flops = flops + 2.0 * ((P + 1) * (P + 2) // 2) ** 2 * mix["far"]
    eval_tflops = eval_flops / (float(np.mean(mix["ms"])) * 1e-3) / 1e12
    if rank != 0:
        ctx.close()
        return 0
    uniform10k = run_uniform10k(G, presets, args, not args.no_cpu_baseline)
    cpu = None
    ref_parity = None
    ref_vs_cpu = None
    if not args.no_cpu_baseline:
        ob, t_o, v_o, u_o, times, cores, f_o = _cpu_baseline(gb, bounds, eps, n_evals=2)
        cpu = {"value": n / float(np.median(times)), "unit": "bodies/s", "cores": cores, "kind": "port",
               "sample": f"2 full REF-mode force evaluations of the same N={n} Plummer workload (C restatement "
                         f"of galax-core compute_fmm_force, OpenMP in m2l/l2p like the reference's Rayon)"}
        # parity at the benchmark size: the device tree, the reference's V/U lists and the
        # REF-mode FP64 forces of this run against the oracle's (vector metric)
        tree_eq = (dev_tree.n_nodes == t_o.n_nodes and np.array_equal(dev_tree.level_start, t_o.level_start)
                   and all(np.array_equal(getattr(dev_tree, f), getattr(t_o, f))
                           for f in ("cx", "cy", "hw", "mass", "comx", "comy", "body_start", "body_end",
                                     "parent", "is_leaf", "child")))
        (vd, vl), (ud, ul) = dev_lists
        lists_eq = (np.array_equal(vl, v_o.lengths) and np.array_equal(vd, v_o.data)
                    and np.array_equal(ul, u_o.lengths) and np.array_equal(ud, u_o.data))
        dref = _rel_err(res["ref_fp64"]["ax"], res["ref_fp64"]["ay"], f_o.ax, f_o.ay)
        ref_parity = {"workload": f"plummer N={n}, p={P}, n_max={N_MAX}, REF mode, FP64",
                      "body_order_bit_exact": bool(np.array_equal(ob.x, gb.x) and np.array_equal(ob.y, gb.y)),
                      "tree_bit_exact": bool(tree_eq), "lists_bit_exact": bool(lists_eq),
                      "max_rel_force_diff": float(dref.max()), "median_rel_force_diff": float(np.median(dref)),
                      "tolerance": 1e-10}
        ref_gpu = n / (float(np.mean(res["ref_fp64"]["ms"])) * 1e-3)
        ref_vs_cpu = {"what": "the reference's own algorithm (REF semantics, FP64) on the GPU against the same "
                              "algorithm on the host cores (oracle port), same workload and run: like for like",
                      "gpu_bodies_per_s": ref_gpu, "cpu_bodies_per_s": cpu["value"], "ratio": ref_gpu / cpu["value"]}
    disk = None
    if not args.no_disk:
        disk = run_disk_compact(G, presets, args)
    line = {
        "metric": METRIC, "value": world * n / (ms_step * 1e-3), "unit": "bodies/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (mixed: FP32 P2M/M2L/L2L/L2P/P2P, FP64 state)",
        "data": "synthetic (seeded Plummer preset: a=1, r<=10a, equal masses 1/N)",
        "config": {"workload": f"plummer N={n}, p={P}, n_max={N_MAX}, one force evaluation per step, static tree",
                   "n": n, "p": P, "n_max": N_MAX, "theta": THETA, "theta_w": args.theta_w,
                   "theta_b": args.theta_b, "mode": "ACCURATE",
                   "eps": eps,
                   "l2": "flushed (256 MB write) before every step, outside its timed interval",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * n / (e2e_ms * 1e-3), "unit": "bodies/s", "h2d_bytes_per_step": 3 * 8 * n,
                "d2h_bytes_per_step": 2 * 8 * n},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                     "frac": achieved / peak32 if peak32 else None,
                     "traffic": (P2P_STREAM_TRAFFIC_1M if args.theta_b > 0 else P2P_TRAFFIC_1M)
                     if n == N_DEFAULT and args.theta_w == THETA_W and args.theta_b in (0.0, THETA_B) else None,
                     "kernel": ("k_p2p32_stream" if args.theta_b > 0 else "k_p2p32_rows") +
                               " (P2P, packed FP32; timed on its own stream, where for most of its run it shares the "
                               "SMs with the far-field chain M2M, M2L, L2L, P2L; *_alone: started after that chain)",
                     "peak_source": "FP32 FMA peak measured in this run (gx_probe_fp32_tflops)",
                     "kernel_ms": kms, "kernel_ms_alone": float(np.mean(k_alone)),
                     "achieved_alone": flops / (float(np.mean(k_alone)) * 1e-3) / 1e12,
                     "frac_alone": flops / (float(np.mean(k_alone)) * 1e-3) / 1e12 / peak32 if peak32 else None,
                     "evaluation_tflops": eval_tflops, "evaluation_frac": eval_tflops / peak32 if peak32 else None},
        "gpu_launches": int(sum(r["launches"] * (r["steps"] + 1) for r in res.values())),
        "clocks": clocks,
        "forms": {k: {"bodies_per_s": n / (float(np.mean(r["ms"])) * 1e-3), "ms_per_step": float(np.mean(r["ms"])),
                      "err_median": r["err_median"], "err_p99": r["err_p99"], "err_mag_mean": r["err_mag_mean"],
                      "err_mag_max": r["err_mag_max"], "plan_s": r["plan_s"],
                      "far_pairs": r["far"], "near_leaf_pairs": r["near"], "p2p_interactions": r["inter"],
                      "p2p_moved_to_body_p2l": r["moved"], "body_p2l_evaluations": r["body_evals"],
                      "pass_ms": dict(zip(["total", "prepare", "p2m", "m2m", "m2l", "l2l", "l2p_p2p"], r["passes"]))}
                  for k, r in res.items()},
        "mixed_vs_fp64": {"speedup": float(np.mean(res["fp64"]["ms"])) / float(np.mean(mix["ms"])),
                          "median_rel_diff": float(np.median(d))},
        "tree": {"nodes": nn, "leaves": nl, "levels": nlev, "build_s_incl_host_copies": setup_tree_s},
        "cpu_baseline": cpu,
        "ref_parity": ref_parity,
        "ref_fp64_vs_cpu_reference": ref_vs_cpu,
        "kdk_steps": steps_cmp,
        "disk_4m": disk,
        "uniform_10k": uniform10k,
        "adjoint": adjoint if adjoint is not None else "not run (--no-adjoint, or N>1 replicas: see the N=1 line)",
    }
    if adjoint is not None:
        sw = adjoint["plummer_1m"]["checkpoint_sweep"]
        kk = "22" if "22" in sw else next(iter(sw))
        line["adjoint_over_forward"] = {"value": sw[kk]["adjoint_over_forward"], "checkpoint_every": int(kk),
                                        "workload": adjoint["plummer_1m"]["workload"]}
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adj-steps", type=int, default=500)
    ap.add_argument("--adj-k", type=lambda s: [int(v) for v in s.split(",")], default=[10, 22, 50, 1])
    ap.add_argument("--fd-dirs", type=int, default=16)
    ap.add_argument("--fd-dirs-1m", type=int, default=8)
    ap.add_argument("--sweep", choices=["disk", "theta", "thetaw", "thetab"], default=None)
    ap.add_argument("--build-only", action="store_true")
    ap.add_argument("--sweep-n", type=int, default=4_000_000)
    ap.add_argument("--no-disk", action="store_true")
    ap.add_argument("--theta-w", type=float, default=THETA_W)
    ap.add_argument("--theta-b", type=float, default=THETA_B)
    ap.add_argument("--sweep-thetas", type=lambda v: [float(x) for x in v.split(",")], default=[0.55, 0.6])
    ap.add_argument("--hbm-budget-gb", type=float, default=32.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local, pg = _dist()
    try:
        if args.impl == "reference":
            return run_reference(args, rank, world, pg)
        if args.sweep == "disk":
            return run_sweep_disk(args) if rank == 0 else 0
        if args.sweep == "theta":
            return run_sweep_theta(args) if rank == 0 else 0
        if args.sweep in ("thetaw", "thetab"):
            return run_sweep_thetaw(args) if rank == 0 else 0
        if args.build_only:
            return run_build_only(args) if rank == 0 else 0
        return run_ours(args, rank, world, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
