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


# ---------------------------------------------------------------- body-level P2L
THETA_B = 0.3


def _body_split_counts(ob, t, R, p2p, theta_b):
    """(P2P interactions moved, body-level P2L evaluations) by the oracle's per-body test
    (gxo_body_p2l): float32, separately rounded operations, as numpy evaluates them."""
    nl = t.n_leaves
    off, idx = p2p.off, p2p.idx
    A = np.repeat(np.arange(nl), np.diff(off[: nl + 1]))
    S = idx[: off[nl]].astype(np.int64)
    keep = S != A
    A, S = A[keep], S[keep]
    bs, be = t.body_start, t.body_end
    tb = np.float32(theta_b)
    tb2 = tb * tb
    ra = R[A].astype(np.float32)
    ra2 = ra * ra
    hx = (t.comx[S] - t.comx[A]).astype(np.float32)
    hy = (t.comy[S] - t.comy[A]).astype(np.float32)
    moved = evals = 0
    for k in range(32):
        j = bs[S] + k
        ok = j < be[S]
        jj = np.where(ok, j, 0)
        ex = (ob.x[jj] - t.comx[S]).astype(np.float32) + hx
        ey = (ob.y[jj] - t.comy[S]).astype(np.float32) + hy
        far = ok & ((ex * ex + ey * ey) * tb2 > ra2)
        evals += int(far.sum())
        moved += int((far * (be[A] - bs[A])).sum())
    return moved, evals


def _oracle_wxb(O, ob, t, theta, theta_w, theta_b, p, eps):
    R = O.node_radii(ob, t)
    far, near = O.mac_lists_build(t, R, theta)
    p2p, m2p, p2l = O.near_split(t, R, theta_w, near)
    ref = ob.copy()
    O.compute_fmm_force_wxb(ref, t, far, p2p, m2p, p2l, p, eps, R, theta_b)
    return ref, R, p2p


def _gpu_b(G, ob, t, v, u, p, eps, prec, theta_w, theta_b):
    n = len(ob.x)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 24, p=p, eps64=eps))
    ctx.set_mode(G.MODE_ACCURATE, prec, 0.5)
    ctx.set_near_split(theta_w)
    ctx.set_body_split(theta_b)
    ctx.upload_tree_data(t, v, u)
    ctx.upload_bodies(G.Bodies.from_arrays(ob.x.copy(), ob.y.copy(), ob.mass.copy()))
    ax, ay = np.zeros(n), np.zeros(n)
    ctx.compute_forces(ob.x.copy(), ob.y.copy(), ob.mass.copy(), ax, ay)
    info = ctx.plan_body_split_info()
    ctx.close()
    return ax, ay, info


@pytest.mark.parametrize("preset,n,n_max,p", [
    ("plummer", 30_000, 32, 4),
    ("uniform", 10_007, 32, 4),
    ("galaxy", 5_001, 32, 4),
    ("disk", 20_000, 16, 4),
    ("plummer", 10_000, 32, 6),
    ("plummer", 10_000, 32, 2),
])
def test_body_split_fp64_matches_oracle(G, oracle, preset, n, n_max, p):
    """Body-level P2L of the P2P rows (source bodies far from the target leaf's COM join
    its local expansion): the FP64 form against the oracle's evaluation of the same split
    (gxo_compute_fmm_force_wxb) within 1e-10, and the same bodies moved."""
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=47)
    ob, t, v, u, eps = oracle_case(oracle, b, n_max, presets.BOUNDS[preset], p)
    ref, R, p2p = _oracle_wxb(oracle, ob, t, 0.5, 0.4, THETA_B, p, eps)
    ax, ay, (moved, evals) = _gpu_b(G, ob, t, v, u, p, eps, G.PREC_FP64, 0.4, THETA_B)
    assert (moved, evals) == _body_split_counts(ob, t, R, p2p, THETA_B)
    if preset != "galaxy":
        assert moved > 0
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64, f"max {err.max():.3e} at body {err.argmax()}"


@pytest.mark.parametrize("preset,n,n_max,p", [("plummer", 30_017, 32, 4), ("uniform", 10_000, 32, 4),
                                              ("disk", 20_000, 16, 4), ("plummer", 20_000, 32, 6)])
def test_body_split_mixed_error_budget(G, oracle, preset, n, n_max, p):
    """The mixed form with the body-level P2L: against the oracle's FP64 evaluation of the
    same split (the FP32 floor), and against the exact sum no worse than 1.15x the oracle's
    split without it."""
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=53)
    ob, t, v, u, eps = oracle_case(oracle, b, n_max, presets.BOUNDS[preset], p)
    ref, R, p2p = _oracle_wxb(oracle, ob, t, 0.5, 0.4, THETA_B, p, eps)
    mx, my, _ = _gpu_b(G, ob, t, v, u, p, eps, G.PREC_MIXED, 0.4, THETA_B)
    assert np.all(np.isfinite(mx)) and np.all(np.isfinite(my))
    d = rel_vec_err(mx, my, ref.ax, ref.ay)
    assert np.median(d) < 2e-6 and d.max() < 1e-3, (np.median(d), d.max())
    base, *_ = _oracle_wxb(oracle, ob, t, 0.5, 0.4, 0.0, p, eps)
    idx = np.random.default_rng(0).choice(n, 1000, replace=False)
    ex, ey = oracle.n2_sampled(ob.x, ob.y, ob.mass, eps, idx)
    e_body = np.median(rel_vec_err(mx[idx], my[idx], ex, ey))
    e_base = np.median(rel_vec_err(base.ax[idx], base.ay[idx], ex, ey))
    assert e_body <= 1.15 * e_base + 2e-7, (e_body, e_base)


def test_body_split_off_is_the_split_and_repeats(G):
    """theta_b = 0 gives the near-list split's evaluation bit for bit; with it on, the
    same evaluation twice gives the same bits, and the plan reports the moved work."""
    from galax_gb300 import presets
    n = 8_000
    b = presets.plummer(n, seed=59)
    gb = b.copy()
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.01))
    ctx.build_tree(gb, 32, presets.BOUNDS["plummer"])
    ctx.upload_bodies(gb)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.set_near_split(0.4)
    out = []
    for tb in (0.0, THETA_B, THETA_B, 0.0):
        ctx.set_body_split(tb)
        ctx.forces_resident()
        r = G.Bodies.new(n)
        ctx.download_bodies(r)
        out.append((r.ax.copy(), r.ay.copy(), ctx.plan_body_split_info()))
    assert np.array_equal(out[0][0], out[3][0]) and np.array_equal(out[0][1], out[3][1])
    assert np.array_equal(out[1][0], out[2][0]) and np.array_equal(out[1][1], out[2][1])
    assert not np.array_equal(out[0][0], out[1][0])
    assert out[0][2] == (0, 0) and out[1][2][0] > 0 and out[1][2][1] > 0
    # the REF form's plan in between leaves the ACCURATE plan's split as it was
    ctx.set_body_split(THETA_B)
    ctx.forces_resident()
    ctx.set_mode(G.MODE_REF, G.PREC_FP64, 0.5)
    ctx.forces_resident()
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.forces_resident()
    r = G.Bodies.new(n)
    ctx.download_bodies(r)
    assert np.array_equal(r.ax, out[1][0]) and np.array_equal(r.ay, out[1][1])
    assert ctx.plan_body_split_info() == out[1][2]
    with pytest.raises(G.GpuError):
        ctx.set_body_split(-0.1)
    ctx.close()
