"""The oracle's accelerated list and constrained-tree builders equal the literal
O(n^2) restatements of the reference (InteractionLists::build lib.rs:947-1025,
build_p2p_lists lib.rs:1358-1392, neighbors_geometric lib.rs:382-423)."""
import numpy as np
import pytest

from galax_gb300 import presets


@pytest.mark.parametrize("preset,n,n_max", [("uniform", 8000, 32), ("plummer", 20000, 32), ("galaxy", 6001, 16),
                                            ("disk", 15000, 8), ("plummer", 3000, 1)])
def test_accelerated_lists_equal_literal(oracle, preset, n, n_max):
    b = presets.make(preset, n, seed=31)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, n_max, presets.BOUNDS[preset])
    va, vl = oracle.vlist_build(t, True), oracle.vlist_build(t, False)
    ua, ul = oracle.ulist_build(t, True), oracle.ulist_build(t, False)
    assert np.array_equal(va.lengths, vl.lengths) and np.array_equal(va.data, vl.data)
    assert np.array_equal(ua.lengths, ul.lengths) and np.array_equal(ua.data, ul.data)


def test_accelerated_lists_with_nonfinite_nodes(oracle):
    b = presets.uniform(2000, seed=32)
    b.x[10] = np.nan
    b.y[20] = np.inf
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, 16, presets.BOUNDS["uniform"])
    va, vl = oracle.vlist_build(t, True), oracle.vlist_build(t, False)
    ua, ul = oracle.ulist_build(t, True), oracle.ulist_build(t, False)
    assert np.array_equal(va.data, vl.data) and np.array_equal(ua.data, ul.data)


@pytest.mark.parametrize("preset,n,n_max", [("uniform", 1500, 16), ("plummer", 2000, 16)])
def test_constrained_accel_equals_literal(oracle, preset, n, n_max):
    b = presets.make(preset, n, seed=33)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    oracle.tree_build(ob, n_max, presets.BOUNDS[preset])  # Morton-sort first, as the CLI does
    t1 = oracle.tree_build_constrained(ob, n_max, presets.BOUNDS[preset], accel=True)
    t2 = oracle.tree_build_constrained(ob, n_max, presets.BOUNDS[preset], accel=False)
    assert t1.n_nodes == t2.n_nodes
    for f in ("cx", "cy", "hw", "body_start", "body_end", "child", "parent"):
        assert np.array_equal(getattr(t1, f), getattr(t2, f))


def test_ref_cache_first_inserter(oracle):
    """m2l's derivative cache (lib.rs:1209-1247): pairs whose truncated offsets agree
    share the derivatives of the first pair in (target id, slot) order."""
    b = presets.uniform(3000, seed=34)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, 32, presets.BOUNDS["uniform"])
    v = oracle.vlist_build(t)
    pk, kd = oracle.m2l_ref_keys(v, t)
    off, idx = v.csr()
    tgt = np.repeat(np.arange(t.n_nodes), v.lengths.astype(np.int64))
    dx = t.comx[tgt] - t.comx[idx]
    dy = t.comy[tgt] - t.comy[idx]
    keys = np.stack([np.trunc(dx), np.trunc(dy)], 1)
    first = {}
    for q, k in enumerate(map(tuple, keys)):
        first.setdefault(k, q)
    assert len(first) == kd.shape[0]
    for q, k in enumerate(map(tuple, keys)):
        f = first[k]
        assert kd[pk[q], 0] == dx[f] and kd[pk[q], 1] == dy[f]


def test_accurate_lists_cover_every_pair_once(oracle):
    """ACCURATE mode: far pairs plus near leaf pairs count every body pair exactly once."""
    b = presets.plummer(3000, seed=35)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, 16, presets.BOUNDS["plummer"])
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.5)
    cover = np.zeros((3000, 3000), np.int32)
    for a in range(t.n_nodes):
        for s in far.idx[far.off[a]:far.off[a + 1]]:
            cover[t.body_start[a]:t.body_end[a], t.body_start[s]:t.body_end[s]] += 1
        if t.is_leaf[a]:
            for s in near.idx[near.off[a]:near.off[a + 1]]:
                cover[t.body_start[a]:t.body_end[a], t.body_start[s]:t.body_end[s]] += 1
    assert np.all(cover == 1)


def test_near_split_partitions_the_near_lists(oracle):
    """The near-list split (M2P / P2L / P2P) is a partition of every leaf's near list that
    keeps list order within each part; far pairs plus the three parts still count every
    body pair once; and each classified pair satisfies its test, recomputed here in
    float32 from the same operands (the COM (hi, lo) split and the radii rounded once)."""
    b = presets.plummer(3000, seed=36)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, 16, presets.BOUNDS["plummer"])
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.5)
    p2p, m2p, p2l = oracle.near_split(t, R, 0.4, near)
    assert m2p.off[-1] > 0 and p2l.off[-1] > 0
    f32 = np.float32
    hx = t.comx.astype(f32)
    lx = (t.comx - hx.astype(np.float64)).astype(f32)
    hy = t.comy.astype(f32)
    ly = (t.comy - hy.astype(np.float64)).astype(f32)
    R32 = R.astype(f32)
    tw = f32(0.4)
    tw2 = f32(tw * tw)

    def kind(a, s):
        ex = f32(f32(hx[a] - hx[s]) + f32(lx[a] - lx[s]))
        ey = f32(f32(hy[a] - hy[s]) + f32(ly[a] - ly[s]))
        lhs = f32(f32(f32(ex * ex) + f32(ey * ey)) * tw2)
        sm = f32(R32[s] + f32(tw * R32[a]))
        if lhs > f32(sm * sm):
            return 1
        sl = f32(R32[a] + f32(tw * R32[s]))
        return 2 if lhs > f32(sl * sl) else 0

    cover = np.zeros((3000, 3000), np.int32)
    for a in range(t.n_nodes):
        for s in far.idx[far.off[a]:far.off[a + 1]]:
            cover[t.body_start[a]:t.body_end[a], t.body_start[s]:t.body_end[s]] += 1
        if not t.is_leaf[a]:
            continue
        whole = list(near.idx[near.off[a]:near.off[a + 1]])
        parts = [list(c.idx[c.off[a]:c.off[a + 1]]) for c in (p2p, m2p, p2l)]
        expect = [[s for s in whole if (0 if s == a else kind(a, s)) == k] for k in range(3)]
        assert parts == expect, a
        for part in parts:
            for s in part:
                cover[t.body_start[a]:t.body_end[a], t.body_start[s]:t.body_end[s]] += 1
    assert np.all(cover == 1)


def test_body_split_oracle(oracle):
    """The oracle's body-level P2L (gxo_compute_fmm_force_wxb): theta_b = 0 is the
    near-list split bit for bit; at theta_b = 0.3 it moves source bodies out of P2P and
    keeps the error against the exact sum within 1.15x of the split without it; every
    moved body passes the per-body test (|x_j - com_a| theta_b > R_a, truncation bounded
    by theta_b^(p+1))."""
    n, p = 6000, 4
    b = presets.plummer(n, seed=61)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, 32, presets.BOUNDS["plummer"])
    eps = oracle.cli_softening(ob)
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.5)
    p2p, m2p, p2l = oracle.near_split(t, R, 0.4, near)
    a0, a1, a2 = ob.copy(), ob.copy(), ob.copy()
    oracle.compute_fmm_force_wx(a0, t, far, p2p, m2p, p2l, p, eps)
    oracle.compute_fmm_force_wxb(a1, t, far, p2p, m2p, p2l, p, eps, R, 0.0)
    oracle.compute_fmm_force_wxb(a2, t, far, p2p, m2p, p2l, p, eps, R, 0.3)
    assert np.array_equal(a0.ax, a1.ax) and np.array_equal(a0.ay, a1.ay)
    assert not np.array_equal(a0.ax, a2.ax)
    idx = np.arange(0, n, 6)
    ex, ey = oracle.n2_sampled(ob.x, ob.y, ob.mass, eps, idx)
    def med(bb):
        return np.median(np.hypot(bb.ax[idx] - ex, bb.ay[idx] - ey) / np.hypot(ex, ey))
    assert med(a2) <= 1.15 * med(a0) + 1e-8, (med(a2), med(a0))
    # a moved body is at least R_a / theta_b from the target leaf's COM (up to the FP32
    # rounding of the test)
    nl = t.n_leaves
    moved = 0
    for a in range(0, nl, 7):
        for q in range(p2p.off[a], p2p.off[a + 1]):
            s = p2p.idx[q]
            if s == a:
                continue
            for j in range(t.body_start[s], t.body_end[s]):
                if oracle.body_p2l(ob, t, R, a, s, j, 0.3):
                    moved += 1
                    d = np.hypot(ob.x[j] - t.comx[a], ob.y[j] - t.comy[a])
                    assert d * 0.3 > R[a] * (1 - 1e-6)
    assert moved > 0


@pytest.mark.parametrize("p", [4, 8])
def test_near_split_oracle_converges_like_the_unsplit_form(oracle, p):
    """The oracle's M2P and P2L (gxo_compute_fmm_force_wx) against the exact sum: at each
    order the split's error stays within 1.5x of the unsplit ACCURATE form's, and both
    fall with p (a wrong M2P or P2L formula would leave an error of the size of the moved
    interactions, independent of p)."""
    n = 3000
    b = presets.plummer(n, seed=63)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, 16, presets.BOUNDS["plummer"])
    eps = oracle.cli_softening(ob)
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.5)
    p2p, m2p, p2l = oracle.near_split(t, R, 0.4, near)
    assert m2p.off[-1] > 0 and p2l.off[-1] > 0
    idx = np.arange(0, n, 3)
    ex, ey = oracle.n2_sampled(ob.x, ob.y, ob.mass, eps, idx)

    def med(bb):
        return float(np.median(np.hypot(bb.ax[idx] - ex, bb.ay[idx] - ey) / np.hypot(ex, ey)))

    a0, a1 = ob.copy(), ob.copy()
    oracle.compute_fmm_force_mac(a0, t, far, near, p, eps)
    oracle.compute_fmm_force_wx(a1, t, far, p2p, m2p, p2l, p, eps)
    e0, e1 = med(a0), med(a1)
    assert e1 <= 1.5 * e0 + 1e-12, (e1, e0)
    assert e1 < (1e-4 if p == 4 else 1e-6), e1  # 6.4e-5 and 3.1e-7 here


@pytest.mark.parametrize("p", [6, 8])
def test_body_split_oracle_at_high_orders(oracle, p):
    """The oracle's body-level P2L at p = 6 and 8: the error against the exact sum stays
    within 1.1x of the near-list split without it (2.4e-6 and 2.2e-7 here), so the moved
    bodies' expansion is right to high order, not only at p = 4."""
    n = 6000
    b = presets.plummer(n, seed=61)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    t = oracle.tree_build(ob, 32, presets.BOUNDS["plummer"])
    eps = oracle.cli_softening(ob)
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.5)
    p2p, m2p, p2l = oracle.near_split(t, R, 0.4, near)
    idx = np.arange(0, n, 6)
    ex, ey = oracle.n2_sampled(ob.x, ob.y, ob.mass, eps, idx)

    def med(bb):
        return float(np.median(np.hypot(bb.ax[idx] - ex, bb.ay[idx] - ey) / np.hypot(ex, ey)))

    a0, a1 = ob.copy(), ob.copy()
    oracle.compute_fmm_force_wx(a0, t, far, p2p, m2p, p2l, p, eps)
    oracle.compute_fmm_force_wxb(a1, t, far, p2p, m2p, p2l, p, eps, R, 0.3)
    assert not np.array_equal(a0.ax, a1.ax)
    e0, e1 = med(a0), med(a1)
    assert e1 <= 1.1 * e0, (e1, e0)
    assert e1 < (5e-6 if p == 6 else 5e-7), e1
