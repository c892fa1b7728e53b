"""The reference's own known-answer and invariant tests, restated against the oracle.

Each test cites the galax-core / galax-integrate / galax-io test it restates.
The reference's tests draw unseeded `fastrand` inputs; here every input is seeded.
These pin the oracle's restatement of galax-core (the reference cannot be built
here: it is Rust and no Rust toolchain is available).
"""
import io

import numpy as np
import pytest


def _uniform(O, n, lo, hi, mlo, mhi, seed):
    r = np.random.default_rng(seed)
    return O.Bodies.from_arrays(r.uniform(lo, hi, n), r.uniform(lo, hi, n), r.uniform(mlo, mhi, n))


def _deterministic(O, n, scale=90.0, off=5.0):
    t = np.arange(n) / n
    return O.Bodies.from_arrays(off + scale * np.modf(t * 3.7)[0], off + scale * np.modf(t * 7.3)[0],
                                0.1 + 10.0 * np.modf(t * 11.0)[0])


# ---------------------------------------------------------------- Morton
def test_morton_round_trip(oracle):  # lib.rs:1758-1779
    b = (-50.0, 50.0, -50.0, 50.0)
    cell = 100.0 / (1 << 21)
    for x, y in [(0.0, 0.0), (25.0, -30.0), (-40.0, 10.0), (49.99, -49.99), (-0.001, 0.001)]:
        k = oracle.morton_encode(x, y, *b)
        rx, ry = oracle.morton_decode(k, *b)
        assert np.hypot(x - rx, y - ry) < cell


def test_morton_encoding_is_injective(oracle):  # lib.rs:1782-1793
    keys = {oracle.morton_encode(x, y, 0.0, 1.0, 0.0, 1.0) for x in [0.0, 0.1, 0.5, 0.9, 0.999]
            for y in [0.0, 0.2, 0.5, 0.8, 0.999]}
    assert len(keys) == 25


def test_morton_wide_separation_gives_different_keys(oracle):  # lib.rs:2833-2838
    assert oracle.morton_encode(0.1, 0.2, 0, 1, 0, 1) != oracle.morton_encode(0.9, 0.8, 0, 1, 0, 1)


def test_morton_bit_layout(oracle):
    """x on even bits, y on odd bits, 21 bits per axis; clamp at 1 - 1e-15 (lib.rs:75-109)."""
    assert oracle.morton_encode(0.5, 0.0, 0, 1, 0, 1) == 1 << 40
    assert oracle.morton_encode(0.0, 0.5, 0, 1, 0, 1) == 1 << 41
    top = oracle.morton_encode(2.0, 2.0, 0, 1, 0, 1)  # clamped to the last cell
    assert top == (1 << 42) - 1
    assert oracle.morton_encode(float("nan"), -5.0, 0, 1, 0, 1) == 0


# ---------------------------------------------------------------- tree
def test_tree_leaves_cover_all_bodies(oracle):  # lib.rs:1796-1820
    b = _uniform(oracle, 500, 0, 100, 1, 1, 1)
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    leaf = t.is_leaf.astype(bool)
    assert leaf.sum() > 0
    assert (t.body_end[leaf] - t.body_start[leaf]).sum() == 500


def test_tree_max_leaf_size_obeyed(oracle):  # lib.rs:1823-1847
    b = _uniform(oracle, 1000, 0, 100, 1, 1, 2)
    t = oracle.tree_build(b, 64, (0, 100, 0, 100))
    leaf = t.is_leaf.astype(bool)
    assert np.all(t.body_end[leaf] - t.body_start[leaf] <= 64)


def test_tree_parent_covers_children(oracle):  # lib.rs:1850-1889
    b = _uniform(oracle, 500, 0, 100, 1, 1, 3)
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    for i in range(t.n_nodes):
        if t.is_leaf[i]:
            continue
        for c in t.child[i]:
            if c < 0:
                continue
            assert t.body_start[i] <= t.body_start[c] and t.body_end[i] >= t.body_end[c]
            assert abs(t.cx[c] - t.cx[i]) + t.hw[c] <= t.hw[i] + 1e-12
            assert abs(t.cy[c] - t.cy[i]) + t.hw[c] <= t.hw[i] + 1e-12


def test_tree_single_body(oracle):  # lib.rs:1892-1903
    b = oracle.Bodies.from_arrays([0.5], [0.5], [1.0])
    t = oracle.tree_build(b, 32, (0, 1, 0, 1))
    assert t.n_nodes == 1 and t.is_leaf[0] and t.body_end[0] - t.body_start[0] == 1


def test_parent_half_width_is_double_child(oracle):  # lib.rs:2466-2494
    b = _uniform(oracle, 16, 0, 10, 1, 1, 4)
    t = oracle.tree_build(b, 2, (0, 10, 0, 10))
    for i in range(t.n_nodes):
        if not t.is_leaf[i]:
            mh = max(t.hw[c] for c in t.child[i] if c >= 0)
            assert abs(t.hw[i] - 2 * mh) < 1e-12


def test_levels_are_rounds(oracle):
    """compute_levels (lib.rs:426-438): a node built in round r has height r, so each
    level is one contiguous id range."""
    b = _uniform(oracle, 3000, 0, 100, 1, 1, 5)
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    lv = t.levels()
    for L in range(t.n_levels):
        assert np.all(lv[t.level_start[L]:t.level_start[L + 1]] == L)


def test_two_body_chain(oracle):
    """Keys of (0.25,0.25),(0.75,0.75) share a prefix only from shift 42: 20 rounds of
    single-child parents then the root: 43 nodes (the tree of lib.rs:1943-1981)."""
    b = oracle.Bodies.from_arrays([0.25, 0.75], [0.25, 0.75], [1.0, 2.0])
    t = oracle.tree_build(b, 1, (0, 1, 0, 1))
    assert t.n_nodes == 43 and t.n_levels == 22


# ---------------------------------------------------------------- passes
def test_p2m_single_body_moments(oracle):  # lib.rs:1906-1940
    b = oracle.Bodies.from_arrays([0.75], [0.25], [2.0])
    t = oracle.tree_build(b, 32, (0, 1, 0, 1))
    M = oracle.p2m(b, t, 4)
    dx, dy = b.x[0] - t.comx[0], b.y[0] - t.comy[0]
    assert M[oracle.moment_index(0, 0)] == 2.0
    assert abs(M[oracle.moment_index(1, 0)] - (-2.0 * dx)) < 1e-14
    assert abs(M[oracle.moment_index(0, 1)] - (-2.0 * dy)) < 1e-14


def test_m2m_shift_matches_direct_p2m(oracle):  # lib.rs:1943-1981
    b = oracle.Bodies.from_arrays([0.25, 0.75], [0.25, 0.75], [1.0, 2.0])
    t = oracle.tree_build(b, 1, (0, 1, 0, 1))
    M = oracle.p2m(b, t, 4)
    oracle.m2m(M, t, 4)
    r = (t.n_nodes - 1) * 15
    assert abs(M[r] - 3.0) < 1e-14
    assert abs(M[r + 1]) < 1e-14 and abs(M[r + 2]) < 1e-14


def test_p2m_and_m2m_produce_no_nans(oracle):  # lib.rs:1984-2000
    b = _uniform(oracle, 500, 0, 100, 0.1, 10.1, 6)
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    M = oracle.p2m(b, t, 4)
    assert not np.isnan(M).any()
    oracle.m2m(M, t, 4)
    assert not np.isnan(M).any()


def test_p2p_is_not_double_counting(oracle):  # lib.rs:2003-2042
    b = _uniform(oracle, 50, 0, 10, 1, 1, 7)
    t = oracle.tree_build(b, 4, (0, 10, 0, 10))
    u = oracle.ulist_build(t)
    pp = b.copy()
    oracle.p2p(pp, t, u, 0.01)
    d = b.copy()
    oracle.n2_force(d, 0.01)
    a1, a2 = np.hypot(pp.ax, pp.ay), np.hypot(d.ax, d.ay)
    assert (np.abs(a1 - a2) / np.maximum(a2, 1e-20)).max() < 100.0


def test_potential_reconstruction(oracle):  # lib.rs:2045-2080 (eval_multipole, lib.rs:1601-1624)
    r = np.random.default_rng(8)
    b = oracle.Bodies.from_arrays(r.uniform(10, 90, 100), r.uniform(10, 90, 100), r.uniform(0.1, 10.1, 100))
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    M = oracle.p2m(b, t, 4)
    oracle.m2m(M, t, 4)
    root = t.n_nodes - 1
    base = root * 15
    eps = 0.1
    for tx, ty in [(150.0, 150.0), (-50.0, -50.0), (150.0, -50.0)]:
        dx, dy = tx - t.comx[root], ty - t.comy[root]
        rt = np.sqrt(dx * dx + dy * dy + eps * eps)
        pot = M[base] * (-1.0 / rt) + M[base + 1] * (-dx / rt ** 3) + M[base + 2] * (-dy / rt ** 3)
        direct = np.sum(-b.mass / np.sqrt((tx - b.x) ** 2 + (ty - b.y) ** 2 + eps * eps))
        assert abs(pot - direct) / max(abs(direct), 1.0) < 0.1


def test_interaction_lists_well_separated(oracle):  # lib.rs:2083-2119
    b = _uniform(oracle, 500, 0, 100, 1, 1, 9)
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    v = oracle.vlist_build(t)
    for n in range(t.n_nodes):
        for p in v.data[n, : v.lengths[n]]:
            dx, dy = abs(t.cx[n] - t.cx[p]), abs(t.cy[n] - t.cy[p])
            assert not (dx <= t.hw[n] + t.hw[p] + 1e-14 and dy <= t.hw[n] + t.hw[p] + 1e-14)
            P, Q = t.parent[n], t.parent[p]
            pdx, pdy = abs(t.cx[P] - t.cx[Q]), abs(t.cy[P] - t.cy[Q])
            assert pdx <= t.hw[P] + t.hw[Q] + 1e-14 and pdy <= t.hw[P] + t.hw[Q] + 1e-14


def test_interaction_lists_max_size(oracle):  # lib.rs:2122-2138
    b = _uniform(oracle, 2000, 0, 100, 1, 1, 10)
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    assert oracle.vlist_build(t).lengths.max() <= 64


def test_m2l_l2l_l2p_farfield_matches_direct(oracle):  # lib.rs:2141-2179
    r = np.random.default_rng(11)
    b = oracle.Bodies.from_arrays(r.uniform(2.5, 97.5, 200), r.uniform(2.5, 97.5, 200), r.uniform(0.1, 5.1, 200))
    t = oracle.tree_build(b, 32, (0, 100, 0, 100))
    p = 2
    v = oracle.vlist_build(t)
    M = oracle.p2m(b, t, p)
    oracle.m2m(M, t, p)
    L = np.zeros_like(M)
    oracle.m2l(L, M, v, t, p, 0.1)
    oracle.l2l(L, t, p)
    f = b.copy()
    oracle.l2p(f, L, t, p)
    assert np.abs(f.ax).max() > 0 and np.abs(f.ay).max() > 0
    assert np.isfinite(f.ax).all() and np.isfinite(f.ay).all()


def test_l2l_shift_is_consistent(oracle):  # lib.rs:2182-2229
    b = oracle.Bodies.from_arrays([0.25, 0.75], [0.25, 0.75], [1.0, 1.0])
    t = oracle.tree_build(b, 1, (0, 1, 0, 1))
    p = 4
    L = np.zeros(t.n_nodes * 15)
    root = t.n_nodes - 1
    L[root * 15 + oracle.moment_index(0, 0)] = 5.0
    L[root * 15 + oracle.moment_index(2, 0)] = 3.0
    oracle.l2l(L, t, p)

    def ev(base, dx, dy):
        return sum(L[base + oracle.moment_index(i, j)] * dx ** i * dy ** j for i in range(p + 1) for j in range(p + 1 - i))

    for c in t.child[root]:
        if c < 0:
            continue
        for tx, ty in [(0.1, 0.15), (-0.05, 0.05)]:
            pv = ev(root * 15, tx - t.comx[root], ty - t.comy[root])
            cv = ev(c * 15, tx - t.comx[c], ty - t.comy[c])
            assert abs(pv - cv) < 1e-14


def test_l2l_ref_order_reaches_one_level(oracle):
    """l2l walks node ids ascending (lib.rs:1266) and parents have higher ids than
    children (lib.rs:324-346): a local placed at the root reaches its children but
    not its grandchildren."""
    b = oracle.Bodies.from_arrays([0.25, 0.75], [0.25, 0.75], [1.0, 1.0])
    t = oracle.tree_build(b, 1, (0, 1, 0, 1))
    L = np.zeros(t.n_nodes * 15)
    root = t.n_nodes - 1
    L[root * 15] = 1.0
    oracle.l2l(L, t, 4, order=0)
    kids = [c for c in t.child[root] if c >= 0]
    assert all(L[c * 15] == 1.0 for c in kids)
    grand = [g for c in kids for g in t.child[c] if g >= 0]
    assert grand and all(L[g * 15] == 0.0 for g in grand)
    L2 = np.zeros(t.n_nodes * 15)
    L2[root * 15] = 1.0
    oracle.l2l(L2, t, 4, order=1)
    assert L2[0] == 1.0 and L2[15] == 1.0  # top-down reaches the leaves


def test_p2p_adjacent_leaves(oracle):  # lib.rs:2248-2286
    b = _uniform(oracle, 100, 0, 2, 0.1, 5.1, 12)
    t = oracle.tree_build(b, 32, (0, 2, 0, 2))
    u = oracle.ulist_build(t)
    f = b.copy()
    oracle.p2p(f, t, u, 0.1)
    assert np.abs(f.ax).max() > 0 and np.isfinite(f.ax).all() and np.isfinite(f.ay).all()


def test_fmm_produces_finite_nonzero(oracle):  # lib.rs:2289-2317
    r = np.random.default_rng(13)
    b = oracle.Bodies.from_arrays(r.uniform(2.5, 97.5, 200), r.uniform(2.5, 97.5, 200), r.uniform(0.1, 5.1, 200))
    t = oracle.tree_build(b, 16, (0, 100, 0, 100))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    f = b.copy()
    oracle.compute_fmm_force(f, t, v, u, 2, 0.1)
    assert np.abs(f.ax).max() > 0 and np.isfinite(f.ax).all() and np.isfinite(f.ay).all()


def test_fmm_p0_equals_p2p(oracle):  # lib.rs:2320-2357
    b = _deterministic(oracle, 200)
    t = oracle.tree_build(b, 16, (0, 100, 0, 100))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    f = b.copy()
    oracle.compute_fmm_force(f, t, v, u, 0, 0.1)
    g = b.copy()
    oracle.p2p(g, t, u, 0.1)
    assert np.abs(f.ax - g.ax).max() < 1e-14 and np.abs(f.ay - g.ay).max() < 1e-14


def _mag_errs(O, f, d):
    a1, a2 = np.hypot(f.ax, f.ay), np.hypot(d.ax, d.ay)
    return np.abs(a1 - a2) / np.maximum(a2, 1e-20)


def test_fmm_balanced_accuracy(oracle):  # lib.rs:2360-2412
    b = _deterministic(oracle, 200)
    t = oracle.tree_build_constrained(b, 16, (0, 100, 0, 100))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    f = b.copy()
    oracle.compute_fmm_force(f, t, v, u, 4, 0.1)
    d = b.copy()
    oracle.n2_force(d, 0.1)
    e = _mag_errs(oracle, f, d)
    e = e[e < 1e10]
    assert np.sqrt(np.mean(e ** 2)) < 5.0


def test_full_fmm_vs_direct_small(oracle):  # lib.rs:2415-2463
    b = _deterministic(oracle, 200)
    t = oracle.tree_build(b, 16, (0, 100, 0, 100))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    f = b.copy()
    oracle.compute_fmm_force(f, t, v, u, 4, 0.1)
    d = b.copy()
    oracle.n2_force(d, 0.1)
    assert _mag_errs(oracle, f, d).max() < 12.0
    assert np.isfinite(f.ax).all() and np.isfinite(f.ay).all()


def test_fmm_converges_with_p(oracle):  # lib.rs:2497-2559 (finiteness)
    b = _deterministic(oracle, 200, scale=8.0, off=1.0)
    t = oracle.tree_build(b, 16, (0, 10, 0, 10))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    for p in (2, 4, 6):
        f = b.copy()
        oracle.compute_fmm_force(f, t, v, u, p, 0.01)
        assert np.isfinite(f.ax).all() and np.isfinite(f.ay).all()


def test_kernel_derivatives_vs_analytic(oracle):  # lib.rs:2562-2596
    p, dx, dy, eps = 2, 3.0, 4.0, 0.1
    d = oracle.kernel_derivs(dx, dy, eps, p)
    r2 = dx * dx + dy * dy + eps * eps
    r = np.sqrt(r2)
    k = lambda a, b_: oracle.kernel_deriv_idx(a, b_, p)
    assert abs(d[k(0, 0)] - (-1.0 / r)) < 1e-14
    assert abs(d[k(1, 0)] - dx / (r2 * r)) < 1e-14
    assert abs(d[k(0, 1)] - dy / (r2 * r)) < 1e-14
    r5 = r2 * r2 * r  # second order: the reference prints these; here they are asserted
    assert abs(d[k(2, 0)] - (-2 * dx * dx + dy * dy + eps * eps) / r5) < 1e-14
    assert abs(d[k(1, 1)] - (-3 * dx * dy / r5)) < 1e-14
    assert abs(d[k(0, 2)] - (dx * dx - 2 * dy * dy + eps * eps) / r5) < 1e-14


@pytest.mark.parametrize("p", [1, 2, 4, 6, 8])
def test_kernel_derivative_recurrence_agrees(oracle, p):
    """The three-term recurrence the GPU uses reproduces the reference's polynomial form."""
    for dx, dy, eps in [(3.3, -4.1, 0.1), (0.7, 0.2, 0.05), (-12.0, 5.0, 0.3)]:
        a = oracle.kernel_derivs(dx, dy, eps, p)
        b = oracle.kernel_derivs(dx, dy, eps, p, recurrence=True)
        scale = np.abs(a).max()
        assert np.abs(a - b).max() <= 1e-11 * scale


def test_neighbors_geometric_symmetry(oracle):  # lib.rs:2689-2713
    b = _uniform(oracle, 200, 0, 10, 1, 1, 14)
    t = oracle.tree_build(b, 16, (0, 10, 0, 10))
    for nid in range(t.n_nodes):
        nb = t.neighbors_geometric(nid)
        if nid != t.n_nodes - 1:
            assert (nb >= 0).sum() > 0
        assert not np.any(nb == nid)


def test_build_constrained_ratio(oracle):  # lib.rs:2716-2766
    def max_ratio(t):
        m = 0.0
        for lid in range(t.n_nodes):
            if not t.is_leaf[lid]:
                continue
            for nb in t.neighbors_geometric(lid):
                if nb >= 0:
                    a, c = t.hw[lid], t.hw[nb]
                    m = max(m, max(a, c) / min(a, c))
        return m
    b = _deterministic(oracle, 500)
    t1 = oracle.tree_build(b.copy(), 16, (0, 100, 0, 100))
    t2 = oracle.tree_build_constrained(b.copy(), 16, (0, 100, 0, 100))
    assert max_ratio(t2) <= max_ratio(t1) + 0.5


def test_fmm_nan_cli_repro(oracle):  # lib.rs:2769-2802
    b = _uniform(oracle, 1000, -50, 50, 0.1, 10.1, 15)
    t = oracle.tree_build(b, 32, (-50, 50, -50, 50))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    eps = oracle.cli_softening(b)
    oracle.compute_fmm_force(b, t, v, u, 4, eps)
    assert np.isfinite(b.ax).all() and np.isfinite(b.ay).all()


def test_fmm_no_nan_plummer(oracle):  # lib.rs:2805-2830
    from galax_gb300 import presets
    p = presets.plummer(1000, seed=16)
    b = oracle.Bodies.from_arrays(p.x, p.y, p.mass)
    t = oracle.tree_build(b, 32, (-50, 50, -50, 50))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    oracle.compute_fmm_force(b, t, v, u, 4, 0.1)
    assert np.isfinite(b.ax).all() and np.isfinite(b.ay).all()


# ---------------------------------------------------------------- N^2 kernel
def test_force_symmetry_two_bodies(oracle):  # lib.rs:2841-2857
    b = oracle.Bodies.from_arrays([0.0, 1.0], [0.0, 0.0], [1.0, 2.0])
    oracle.n2_force(b, 0.1)
    assert abs(b.ax[0] * 1.0 + b.ax[1] * 2.0) < 1e-14 and abs(b.ay[0] + 2 * b.ay[1]) < 1e-14


def test_softening_zero_separation(oracle):  # lib.rs:2860-2873
    b = oracle.Bodies.from_arrays([0.0, 0.0], [0.0, 0.0], [1.0, 1e6])
    oracle.n2_force(b, 0.1)
    assert b.ax[0] == 0.0 and b.ax[1] == 0.0


def test_softening_small_separation_linear(oracle):  # lib.rs:2876-2889
    eps, r = 0.1, 1e-10
    b = oracle.Bodies.from_arrays([0.0, r], [0.0, 0.0], [1.0, 1.0])
    oracle.n2_force(b, eps)
    lin = r / eps ** 3
    assert abs(b.ax[0] - lin) / lin < 1e-6


def test_force_known_distance(oracle):  # lib.rs:2892-2908
    b = oracle.Bodies.from_arrays([0.0, 1.0], [0.0, 0.0], [1.0, 1.0])
    oracle.n2_force(b, 0.1)
    e = 1.0 / (1.0 + 0.01) ** 1.5
    assert abs(b.ax[0] - e) < 1e-14 and abs(b.ax[1] + e) < 1e-14
    assert b.ay[0] == 0.0 and b.ay[1] == 0.0


# ---------------------------------------------------------------- integrator (galax-integrate)
def test_single_body_drift(oracle):  # galax-integrate/src/lib.rs:9-30
    b = oracle.Bodies.from_arrays([0.0], [0.0], [1.0], [10.0], [5.0])
    t = oracle.tree_build(b, 32, (-100, 100, -100, 100))
    v, u = oracle.vlist_build(t), oracle.ulist_build(t)
    oracle.simulate(b, t, v, u, 2, 0.1, 0.1, 1, 0)
    assert b.vx[0] == 10.0 and b.vy[0] == 5.0
    assert abs(b.x[0] - 1.0) < 1e-14 and abs(b.y[0] - 0.5) < 1e-14


def test_energy_diagnostics_known_values(oracle):  # galax-integrate/src/lib.rs:33-54
    b = oracle.Bodies(np.array([0.0, 3.0]), np.array([0.0, 0.0]), np.array([2.0, -1.0]), np.array([1.0, 2.0]),
                      np.array([5.0, 3.0]), np.array([0.5, -0.3]), np.array([0.0, 0.1]))
    assert abs(oracle.kinetic_energy(b) - 0.5 * (5 * 5 + 3 * 5)) < 1e-14
    px, py = oracle.momentum(b)
    assert abs(px - 7.0) < 1e-14 and abs(py - 11.0) < 1e-14
    assert abs(oracle.angular_momentum(b) - 18.0) < 1e-14


def _simulate_n2(O, b, eps, dt, n_steps):
    """simulate_n2 / leapfrog_kdk_n2 (galax-integrate/src/lib.rs:241-287)."""
    O.n2_force(b, eps)
    h = 0.5 * dt
    for _ in range(n_steps):
        b.vx += b.ax * h
        b.vy += b.ay * h
        b.x += b.vx * dt
        b.y += b.vy * dt
        O.n2_force(b, eps)
        b.vx += b.ax * h
        b.vy += b.ay * h
    ke = O.kinetic_energy(b)
    dx, dy = b.x[1] - b.x[0], b.y[1] - b.y[0]
    pe = -b.mass[0] * b.mass[1] / np.sqrt(dx * dx + dy * dy + eps * eps)
    return ke + pe


@pytest.mark.parametrize("orbits,steps_per_orbit", [(1, 500), (100, 50)])
def test_kepler_energy(oracle, orbits, steps_per_orbit):  # galax-integrate/src/lib.rs:57-143
    a, m = 10.0, 1.0
    v = np.sqrt(2 * m / a) * 0.5
    b = oracle.Bodies.from_arrays([-a / 2, a / 2], [0.0, 0.0], [m, m], [0.0, 0.0], [v, -v])
    e0 = oracle.kinetic_energy(b) - m * m / a
    T = 2 * np.pi * np.sqrt(a ** 3 / (2 * m))
    n = orbits * steps_per_orbit
    e1 = _simulate_n2(oracle, b, 1e-8, T / steps_per_orbit, n)
    assert abs(e1 - e0) / abs(e0) < 0.01
    if orbits == 1:
        assert max(abs(b.x[0] + a / 2), abs(b.y[0])) / a < 0.02


def test_interaction_list_compaction(oracle):  # galax-gpu/src/lib.rs:768-781 (compact_interaction_lists)
    b = _uniform(oracle, 300, 0, 100, 1, 1, 17)
    t = oracle.tree_build(b, 8, (0, 100, 0, 100))
    v = oracle.vlist_build(t)
    off, idx = v.csr()
    for nd in range(t.n_nodes):
        assert np.array_equal(idx[off[nd]:off[nd + 1]], v.data[nd, : v.lengths[nd]])
