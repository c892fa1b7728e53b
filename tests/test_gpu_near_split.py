"""The leaf-level split of the ACCURATE near lists (M2P and P2L) against the oracle.

A near leaf pair whose target bodies are all far from the source leaf takes the
source's multipole at each target body (M2P); one whose source bodies are all far
from the target leaf adds them to the target's local expansion (P2L); the rest stay
P2P.  The reference has only P2P for its U-list pairs (galax-core/src/lib.rs:1395-1462);
these lists are the W/X-list counterpart of its V-list M2L (lib.rs:1199-1259).  The
device's split must equal the oracle's pair for pair (gxo_near_split), the FP64 form
must match the oracle's evaluation (gxo_compute_fmm_force_wx) within 1e-10, and the
mixed form must keep the error against the exact sum.
"""
import numpy as np
import pytest

from helpers import oracle_case, rel_vec_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10


def _oracle_wx(O, ob, t, theta, theta_w, p, eps):
    R = O.node_radii(ob, t)
    far, near = O.mac_lists_build(t, R, theta)
    p2p, m2p, p2l = O.near_split(t, R, theta_w, near)
    ref = ob.copy()
    O.compute_fmm_force_wx(ref, t, far, p2p, m2p, p2l, p, eps)
    return ref, far, p2p, m2p, p2l


def _leaf_interactions(t, c):
    """Body-body interactions of the P2P lists, a body with itself not counted."""
    cnt = t.body_end - t.body_start
    tot = sum(int(cnt[a]) * int(cnt[c.idx[c.off[a]:c.off[a + 1]]].sum()) for a in range(t.n_leaves))
    return int(tot - cnt[: t.n_leaves].sum())


def _gpu(G, ob, t, v, u, p, eps, prec, theta, theta_w):
    n = len(ob.x)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 24, p=p, eps64=eps))
    ctx.set_mode(G.MODE_ACCURATE, prec, theta)
    ctx.set_near_split(theta_w)
    ctx.upload_tree_data(t, v, u)
    ctx.upload_bodies(G.Bodies.from_arrays(ob.x.copy(), ob.y.copy(), ob.mass.copy()))
    ax, ay = np.zeros(n), np.zeros(n)
    ctx.compute_forces(ob.x.copy(), ob.y.copy(), ob.mass.copy(), ax, ay)
    info = ctx.plan_info(), ctx.plan_split_info()
    ctx.close()
    return ax, ay, info


@pytest.mark.parametrize("preset,n,n_max,p,theta_w", [
    ("uniform", 10_000, 32, 4, 0.4),
    ("plummer", 30_000, 32, 4, 0.4),
    ("plummer", 30_000, 32, 4, 0.5),
    ("galaxy", 5_001, 32, 4, 0.3),
    ("disk", 20_000, 16, 4, 0.4),
    ("uniform", 8_000, 64, 4, 0.4),
    ("plummer", 10_000, 32, 2, 0.4),
    ("plummer", 10_000, 32, 6, 0.4),
    ("plummer", 10_000, 32, 8, 0.4),
    ("uniform", 3_000, 32, 0, 0.4),
])
def test_split_fp64_matches_oracle(G, oracle, preset, n, n_max, p, theta_w):
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=17)
    ob, t, v, u, eps = oracle_case(oracle, b, n_max, presets.BOUNDS[preset], p)
    ref, far, p2p, m2p, p2l = _oracle_wx(oracle, ob, t, 0.5, theta_w, p, eps)
    ax, ay, ((n_far, n_near, inter), (n_m2p, n_p2l)) = _gpu(G, ob, t, v, u, p, eps, G.PREC_FP64, 0.5, theta_w)
    # the same split, pair for pair in count
    assert n_far == far.off[-1]
    assert n_near == int(np.diff(p2p.off)[: t.n_leaves].sum())
    assert n_m2p == int(m2p.off[-1]) and n_p2l == int(p2l.off[-1])
    assert inter == _leaf_interactions(t, p2p)
    if preset != "galaxy":
        assert n_m2p > 0 and n_p2l > 0
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64, f"max {err.max():.3e} at body {err.argmax()}"


@pytest.mark.parametrize("preset,n,p", [("plummer", 30_000, 4), ("uniform", 10_000, 4), ("plummer", 20_000, 6),
                                        ("plummer", 20_000, 8)])
def test_split_mixed_error_budget(G, oracle, preset, n, p):
    """The mixed form with the split: against the oracle's FP64 evaluation of the same
    lists (the FP32 floor), and against the exact sum no worse than 1.3x the unsplit FP64
    form at theta_w = 0.4."""
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=19)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS[preset], p)
    ref, *_ = _oracle_wx(oracle, ob, t, 0.5, 0.4, p, eps)
    mx, my, _ = _gpu(G, ob, t, v, u, p, eps, G.PREC_MIXED, 0.5, 0.4)
    d = rel_vec_err(mx, my, ref.ax, ref.ay)
    assert np.all(np.isfinite(mx)) and np.all(np.isfinite(my))
    assert np.median(d) < 2e-6 and d.max() < 1e-3, (np.median(d), d.max())
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.5)
    base = ob.copy()
    oracle.compute_fmm_force_mac(base, t, far, near, p, eps)
    idx = np.random.default_rng(0).choice(n, 1000, replace=False)
    ex, ey = oracle.n2_sampled(ob.x, ob.y, ob.mass, eps, idx)
    e_split = np.median(rel_vec_err(mx[idx], my[idx], ex, ey))
    e_base = np.median(rel_vec_err(base.ax[idx], base.ay[idx], ex, ey))
    assert e_split <= 1.3 * e_base + 2e-7, (e_split, e_base)


def test_split_off_is_the_accurate_form_and_the_adjoint_needs_it_off(G, oracle):
    """theta_w = 0 gives the unsplit ACCURATE evaluation bit for bit; switching the split on
    re-plans; the adjoint refuses to run with the split on (it transposes P2P only)."""
    from galax_gb300 import presets
    n = 8_000
    b = presets.plummer(n, seed=23)
    gb = b.copy()
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.01))
    ctx.build_tree(gb, 32, presets.BOUNDS["plummer"])
    ctx.upload_bodies(gb)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.forces_resident()
    r0 = G.Bodies.new(n)
    ctx.download_bodies(r0)
    _, _, i0 = ctx.plan_info()
    ctx.set_near_split(0.4)
    ctx.forces_resident()
    r1 = G.Bodies.new(n)
    ctx.download_bodies(r1)
    _, _, i1 = ctx.plan_info()
    assert i1 < i0 and ctx.plan_split_info()[0] > 0
    assert not np.array_equal(r0.ax, r1.ax)
    with pytest.raises(G.GpuError) as e:
        ctx.force_vjp(np.ones(n), np.ones(n))
    assert e.value.code == 8
    ctx.set_near_split(0.0)
    ctx.forces_resident()
    r2 = G.Bodies.new(n)
    ctx.download_bodies(r2)
    assert np.array_equal(r0.ax, r2.ax) and np.array_equal(r0.ay, r2.ay)
    assert ctx.plan_split_info() == (0, 0)
    with pytest.raises(G.GpuError):
        ctx.set_near_split(-1.0)
    ctx.close()


def test_split_with_rebuild_every_step(G):
    """A leapfrog run that rebuilds the tree every step re-plans the split every step; the
    same run twice gives the same bits (the split's partition and sums are ordered)."""
    from galax_gb300 import presets
    n = 20_000
    b = presets.plummer(n, seed=29)
    outs = []
    for _ in range(2):
        gb = b.copy()
        ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.005))
        ctx.build_tree(gb, 32, presets.BOUNDS["plummer"])
        ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
        ctx.set_near_split(0.4)
        ctx.upload_bodies(gb)
        ctx.forces_resident()
        ctx.kdk_run(5, 1e-3, 0, rebuild_every=1)
        r = G.Bodies.new(n)
        ctx.download_bodies(r)
        outs.append(r)
        ctx.close()
    assert np.array_equal(outs[0].x, outs[1].x) and np.array_equal(outs[0].ax, outs[1].ax)
    assert np.all(np.isfinite(outs[0].ax))
