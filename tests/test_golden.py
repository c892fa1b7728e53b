"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle reproduces every fixture bit for bit (a regression pin on the
restatement), and the accelerated list builders equal the literal ones.
GPU: the device tree, lists and forces match the fixtures.
"""
import glob
import os

import numpy as np
import pytest

from helpers import rel_vec_err

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
TREE_FIELDS = ["cx", "cy", "hw", "mass", "comx", "comy", "body_start", "body_end", "child", "parent", "is_leaf",
               "level_start"]


def _load(path):
    return dict(np.load(path))


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_fixture(oracle, path):
    g = _load(path)
    b = oracle.Bodies.from_arrays(g["x_in"], g["y_in"], g["m_in"], g["vx_in"], g["vy_in"])
    t = oracle.tree_build(b, int(g["n_max"]), tuple(g["bounds"]))
    for k in ("x", "y", "vx", "vy"):
        assert np.array_equal(getattr(b, k), g[k]), k
    assert np.array_equal(b.mass, g["m"])
    for f in TREE_FIELDS:
        assert np.array_equal(getattr(t, f), g[f]), f
    v, u = oracle.vlist_build(t, True), oracle.ulist_build(t, True)
    assert np.array_equal(v.data, g["vdata"]) and np.array_equal(v.lengths, g["vlen"])
    assert np.array_equal(u.data, g["udata"]) and np.array_equal(u.lengths, g["ulen"])
    eps = oracle.cli_softening(b)
    assert eps == float(g["eps"])
    p = int(g["p"])
    for mode, key in ((oracle.MODE_REF, "ref"), (oracle.MODE_EXACT, "exact")):
        f = b.copy()
        oracle.compute_fmm_force(f, t, v, u, p, eps, mode)
        # OpenMP scheduling does not change any sum: each target is summed by one thread
        assert np.array_equal(f.ax, g[f"ax_{key}"]) and np.array_equal(f.ay, g[f"ay_{key}"]), key


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_matches_fixture(G, path):
    g = _load(path)
    n = g["x_in"].size
    p = int(g["p"])
    eps = float(g["eps"])
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 24, p=p, eps64=eps))
    b = G.Bodies.from_arrays(g["x_in"], g["y_in"], g["m_in"], g["vx_in"], g["vy_in"])
    ctx.build_tree(b, int(g["n_max"]), tuple(g["bounds"]))
    assert np.array_equal(b.x, g["x"]) and np.array_equal(b.y, g["y"])
    t = ctx.export_tree()
    for f in TREE_FIELDS:
        assert np.array_equal(getattr(t, f), g[f]), f
    vd, vl = ctx.export_lists(G.LIST_V)
    ud, ul = ctx.export_lists(G.LIST_U)
    assert np.array_equal(vd, g["vdata"]) and np.array_equal(vl, g["vlen"])
    assert np.array_equal(ud, g["udata"]) and np.array_equal(ul, g["ulen"])
    for mode, key in ((G.MODE_REF, "ref"), (G.MODE_EXACT, "exact"), (G.MODE_ACCURATE, "acc")):
        ctx.set_mode(mode, G.PREC_FP64, 0.5)
        ax, ay = np.zeros(n), np.zeros(n)
        ctx.compute_forces(b.x, b.y, b.mass, ax, ay)
        err = rel_vec_err(ax, ay, g[f"ax_{key}"], g[f"ay_{key}"])
        assert err.max() < 1e-10, (key, err.max())
    ctx.close()
