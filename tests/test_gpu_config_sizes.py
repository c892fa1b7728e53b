"""Parity at the workload sizes, not only at small N.

The galaxy workload at its full size (N = 200,001: a central mass of 1000 and
200,000 test particles) and the disk workload at its full size (N = 4,000,000)
with n_max in {16, 32, 64}: the device tree build (Tree::build,
galax-core/src/lib.rs:163-361), the V-list (InteractionLists::build,
lib.rs:947-1025) and the U-list (build_p2p_lists, lib.rs:1358-1392) are compared
with the oracle bit for bit, and the REF-mode FP64 forces (compute_fmm_force,
lib.rs:1466-1499) within 1e-10 relative per body.  The galaxy case also checks
the ACCURATE FP64 form against the oracle's restatement of it.  The 1M Plummer
workload is compared the same way by the benchmark (its `ref_parity` key).
"""
import numpy as np
import pytest

from helpers import rel_vec_err

pytestmark = pytest.mark.gpu

FIELDS = ["cx", "cy", "hw", "mass", "comx", "comy", "body_start", "body_end", "parent", "is_leaf"]
TOL_FP64 = 1e-10


def _parity(G, O, preset, n, n_max, seed, accurate=False):
    from galax_gb300 import presets
    bounds = presets.BOUNDS[preset]
    b = presets.make(preset, n, seed=seed)
    ob = O.Bodies.from_arrays(b.x, b.y, b.mass, b.vx, b.vy)
    t = O.tree_build(ob, n_max, bounds)
    eps = O.cli_softening(ob)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 26, p=4, eps64=eps))
    gb = b.copy()
    ctx.build_tree(gb, n_max, bounds)
    # the body order (Tree::build permutes in place) and every node field, bit for bit
    for name in ("x", "y", "vx", "vy", "mass"):
        assert np.array_equal(getattr(gb, name), getattr(ob, name)), name
    dt = ctx.export_tree()
    assert dt.n_nodes == t.n_nodes and dt.n_levels == t.n_levels
    assert np.array_equal(dt.level_start, t.level_start)
    for f in FIELDS:
        assert np.array_equal(getattr(dt, f), getattr(t, f)), f
    assert np.array_equal(dt.child, t.child)
    v, u = O.vlist_build(t), O.ulist_build(t)
    vd, vl = ctx.export_lists(G.LIST_V)
    ud, ul = ctx.export_lists(G.LIST_U)
    assert np.array_equal(vl, v.lengths) and np.array_equal(vd, v.data), "V-list"
    assert np.array_equal(ul, u.lengths) and np.array_equal(ud, u.data), "U-list"
    # REF-mode FP64 forces against the oracle's compute_fmm_force
    ref = ob.copy()
    O.compute_fmm_force(ref, t, v, u, 4, eps, O.MODE_REF)
    ctx.set_mode(G.MODE_REF, G.PREC_FP64, 0.5)
    ax, ay = np.zeros(n), np.zeros(n)
    ctx.compute_forces(gb.x, gb.y, gb.mass, ax, ay)
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64, f"REF: max {err.max():.3e} at body {err.argmax()}"
    if accurate:
        R = O.node_radii(ob, t)
        far, near = O.mac_lists_build(t, R, 0.5)
        ref2 = ob.copy()
        O.compute_fmm_force_mac(ref2, t, far, near, 4, eps)
        ctx.set_mode(G.MODE_ACCURATE, G.PREC_FP64, 0.5)
        ctx.upload_bodies(gb)
        ctx.compute_forces(gb.x, gb.y, gb.mass, ax, ay)
        err2 = rel_vec_err(ax, ay, ref2.ax, ref2.ay)
        assert err2.max() < TOL_FP64, f"ACCURATE: max {err2.max():.3e} at body {err2.argmax()}"
    ctx.close()


def test_galaxy_200001_tree_lists_forces(G, oracle):
    _parity(G, oracle, "galaxy", 200_001, 32, seed=4, accurate=True)


@pytest.mark.parametrize("n_max", [16, 32, 64])
def test_disk_4m_tree_lists_forces(G, oracle, n_max):
    _parity(G, oracle, "disk", 4_000_000, n_max, seed=3)
