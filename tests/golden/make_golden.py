"""Generates the golden fixtures in this directory from the oracle.

Each case stores the seeded input bodies, the Morton-sorted bodies, the tree
(Tree::build, galax-core/src/lib.rs:163-361), the V- and U-lists
(lib.rs:947-1025, 1358-1392), the softening (galax-cli/src/main.rs:182-190)
and the accelerations of the REF, EXACT and ACCURATE modes.  The reference
itself (Rust) cannot be run here, so these fixtures pin the oracle's
restatement against regressions and give the GPU tests fixed targets.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from galax_gb300 import presets  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = {
    "uniform_600": ("uniform", 600, 21, 32, 4),
    "plummer_800": ("plummer", 800, 22, 16, 4),
    "galaxy_301": ("galaxy", 301, 23, 32, 4),
    "uniform_clamped_500": ("uniform", 500, 24, 32, 2),  # [0,100]^2 bodies in the [-50,50]^2 CLI box
}


def make_case(name):
    preset, n, seed, n_max, p = CASES[name]
    b = presets.make(preset, n, seed)
    bounds = (-50.0, 50.0, -50.0, 50.0) if name == "uniform_clamped_500" else presets.BOUNDS[preset]
    ob = O.Bodies.from_arrays(b.x, b.y, b.mass, b.vx, b.vy)
    t = O.tree_build(ob, n_max, bounds)
    v, u = O.vlist_build(t, False), O.ulist_build(t, False)  # literal builders
    eps = O.cli_softening(ob)
    out = dict(x_in=b.x, y_in=b.y, m_in=b.mass, vx_in=b.vx, vy_in=b.vy, x=ob.x, y=ob.y, m=ob.mass, vx=ob.vx,
               vy=ob.vy, bounds=np.array(bounds), n_max=np.array(n_max), p=np.array(p), eps=np.array(eps),
               cx=t.cx, cy=t.cy, hw=t.hw, mass=t.mass, comx=t.comx, comy=t.comy, body_start=t.body_start,
               body_end=t.body_end, child=t.child, parent=t.parent, is_leaf=t.is_leaf, level_start=t.level_start,
               vdata=v.data, vlen=v.lengths, udata=u.data, ulen=u.lengths)
    for mode, key in ((O.MODE_REF, "ref"), (O.MODE_EXACT, "exact")):
        f = ob.copy()
        O.compute_fmm_force(f, t, v, u, p, eps, mode)
        out[f"ax_{key}"], out[f"ay_{key}"] = f.ax, f.ay
    R = O.node_radii(ob, t)
    far, near = O.mac_lists_build(t, R, 0.5)
    f = ob.copy()
    O.compute_fmm_force_mac(f, t, far, near, p, eps)
    out["ax_acc"], out["ay_acc"] = f.ax, f.ay
    d = ob.copy()
    O.n2_force(d, eps)
    out["ax_n2"], out["ay_n2"] = d.ax, d.ay
    return out


if __name__ == "__main__":
    O.set_threads(1)
    for name in CASES:
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **make_case(name))
        print("wrote", name)
