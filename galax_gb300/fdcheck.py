"""Central finite differences of a leapfrog rollout loss, for checking the adjoint.

With a static tree the rollout is a smooth function of the starting state and plain
central differences apply.  With the tree rebuilt every step it is only piecewise
smooth: a perturbation of 1e-6 moves bodies across Morton cells, which reorders the
bodies and changes leaves, lists and expansion centres.  The adjoint differentiates
the rollout with every step's tree held at its value on the unperturbed trajectory,
so the matching finite difference replays that tree sequence: the unperturbed state
and every perturbed copy advance in lockstep, each step's tree is built from the
unperturbed positions only, and the perturbed copies are evaluated on it
(``GpuContext.compute_forces`` on the resident tree and plan).

The kick and drift are done on the host in FP64 with separately rounded operations,
as the device kernels do, so the unperturbed trajectory is the device one bit for bit.
"""
from __future__ import annotations

import numpy as np

_FIELDS = ("x", "y", "vx", "vy", "m")


def rollout_loss(x0, y0, xT, yT, R, ids=None):
    """L = sum_i |x_T[i] - R x_0[ids[i]]|^2 (ids: starting index of each final body),
    its cotangent dL/dx_T and the direct term dL/dx_0."""
    ids = np.arange(x0.size) if ids is None else ids
    tx = R[0, 0] * x0[ids] + R[0, 1] * y0[ids]
    ty = R[1, 0] * x0[ids] + R[1, 1] * y0[ids]
    rx, ry = xT - tx, yT - ty
    d0x, d0y = np.zeros(x0.size), np.zeros(x0.size)
    d0x[ids] = -2 * (R[0, 0] * rx + R[1, 0] * ry)
    d0y[ids] = -2 * (R[0, 1] * rx + R[1, 1] * ry)
    return float(np.sum(rx * rx + ry * ry)), 2 * rx, 2 * ry, d0x, d0y


def fd_frozen_trees(G, ctx, bodies, n_steps: int, dt: float, R, directions, h: float, n_max: int, bounds,
                    rebuild: bool = True):
    """Central differences (L(s + h d) - L(s - h d)) / 2h of the rollout loss along each
    direction d = (dx, dy, dvx, dvy, dm), trees (and plans) taken from the unperturbed
    trajectory.  ``ctx`` must be in the mode and precision of the rollout under test;
    its resident bodies are overwritten."""
    n = len(bodies)
    base = {"x": bodies.x, "y": bodies.y, "vx": bodies.vx, "vy": bodies.vy, "m": bodies.mass}
    U = {k: np.array(v, dtype=np.float64) for k, v in base.items()}
    V = []
    for d in directions:
        for sg in (1.0, -1.0):
            V.append({k: np.array(base[k] + sg * h * d[q], dtype=np.float64) for q, k in enumerate(_FIELDS)})
    starts = [(s["x"].copy(), s["y"].copy()) for s in V]
    ids = np.arange(n)
    ax = np.zeros(n)
    ay = np.zeros(n)
    acc = [None] * (1 + len(V))

    def forces():
        nonlocal ids
        b = G.Bodies.from_arrays(U["x"], U["y"], U["m"], U["vx"], U["vy"])
        ctx.upload_bodies(b)
        if rebuild:
            perm = ctx.rebuild_resident(n_max, bounds, want_perm=True)
            for s in [U] + V:
                for k in _FIELDS:
                    s[k] = s[k][perm]
            ids = ids[perm]
        ctx.forces_resident()  # builds this tree's plan from the unperturbed positions
        out = G.Bodies.new(n)
        ctx.download_bodies(out)
        acc[0] = (out.ax.copy(), out.ay.copy())
        for j, s in enumerate(V):
            ctx.compute_forces(s["x"], s["y"], s["m"], ax, ay)
            acc[j + 1] = (ax.copy(), ay.copy())

    hh = 0.5 * dt
    forces()
    for _ in range(n_steps):
        for j, s in enumerate([U] + V):
            a = acc[j]
            s["vx"] = s["vx"] + a[0] * hh
            s["vy"] = s["vy"] + a[1] * hh
            s["x"] = s["x"] + s["vx"] * dt
            s["y"] = s["y"] + s["vy"] * dt
        forces()
        for j, s in enumerate([U] + V):
            a = acc[j]
            s["vx"] = s["vx"] + a[0] * hh
            s["vy"] = s["vy"] + a[1] * hh
    out = []
    for i in range(len(directions)):
        lp = rollout_loss(starts[2 * i][0], starts[2 * i][1], V[2 * i]["x"], V[2 * i]["y"], R, ids)[0]
        lm = rollout_loss(starts[2 * i + 1][0], starts[2 * i + 1][1], V[2 * i + 1]["x"], V[2 * i + 1]["y"], R, ids)[0]
        out.append((lp - lm) / (2 * h))
    return np.array(out)
