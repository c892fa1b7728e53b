"""Helpers shared by the parity tests: oracle runs on the same seeded inputs."""
import numpy as np


def oracle_case(O, bodies, n_max, bounds, p, eps=None, mode=0, lists_accel=True):
    ob = O.Bodies.from_arrays(bodies.x, bodies.y, bodies.mass, bodies.vx, bodies.vy)
    t = O.tree_build(ob, n_max, bounds)
    v = O.vlist_build(t, lists_accel)
    u = O.ulist_build(t, lists_accel)
    if eps is None:
        eps = O.cli_softening(ob)
    return ob, t, v, u, eps


def rel_vec_err(ax, ay, rx, ry):
    den = np.maximum(np.hypot(rx, ry), 1e-30)
    return np.hypot(np.asarray(ax) - rx, np.asarray(ay) - ry) / den
