"""Device tree build and interaction lists, bit-exact against the oracle.

Tree::build (galax-core/src/lib.rs:163-361): Morton keys, stable sort, permute,
leaves, parent rounds; InteractionLists::build (lib.rs:947-1025) and
build_p2p_lists (lib.rs:1358-1392); build_constrained (lib.rs:541-588).
"""
import numpy as np
import pytest

from helpers import oracle_case

pytestmark = pytest.mark.gpu

FIELDS = ["cx", "cy", "hw", "mass", "comx", "comy", "body_start", "body_end", "parent", "is_leaf"]


def _ctx(G, n):
    return G.GpuContext(G.GpuConfig(max_n=max(n, 1), max_nodes=1 << 26, p=4, eps64=0.1))


def _compare_tree(G, O, b, n_max, bounds, balanced=False):
    ob = O.Bodies.from_arrays(b.x, b.y, b.mass, b.vx, b.vy)
    if balanced:
        t = O.tree_build_constrained(ob, n_max, bounds, accel=True)
    else:
        t = O.tree_build(ob, n_max, bounds)
    ctx = _ctx(G, len(b))
    gb = b.copy()
    ctx.build_tree(gb, n_max, bounds, balanced=balanced)
    # Tree::build permutes every body array in place (lib.rs:204)
    for name in ("x", "y", "vx", "vy", "mass"):
        assert np.array_equal(getattr(gb, name), getattr(ob, name), equal_nan=True), name
    dt = ctx.export_tree()
    assert dt.n_nodes == t.n_nodes
    assert dt.n_levels == t.n_levels
    assert np.array_equal(dt.level_start, t.level_start)
    for f in FIELDS:
        a, r = getattr(dt, f), getattr(t, f)
        assert np.array_equal(a, r, equal_nan=True), f
    assert np.array_equal(dt.child, t.child)
    v = O.vlist_build(t)
    u = O.ulist_build(t)
    vd, vl = ctx.export_lists(G.LIST_V)
    ud, ul = ctx.export_lists(G.LIST_U)
    assert np.array_equal(vl, v.lengths) and np.array_equal(vd, v.data)
    assert np.array_equal(ul, u.lengths) and np.array_equal(ud, u.data)
    ctx.close()
    return t


@pytest.mark.parametrize("preset,n,n_max", [
    ("uniform", 10_000, 32),
    ("plummer", 20_000, 32),
    ("galaxy", 5_001, 32),
    ("disk", 20_000, 16),
    ("uniform", 3_000, 64),
    # more than 2048 leaves: the single-child rounds are built by one fused kernel
    ("plummer", 200_000, 32),
    ("uniform", 100_000, 16),
])
def test_tree_and_lists_bit_exact(G, oracle, preset, n, n_max):
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=3)
    _compare_tree(G, oracle, b, n_max, presets.BOUNDS[preset])


def test_cli_box_clamping_and_duplicate_keys(G, oracle):
    """Bodies outside the [-50,50]^2 CLI box clamp onto edge cells (lib.rs:76);
    duplicates share keys and keep input order (stable sort)."""
    from galax_gb300 import presets
    b = presets.uniform(4_000, seed=5)  # [0,100]^2 in a [-50,50]^2 box: half clamps
    b.x[:50] = b.x[50:100]  # exact duplicates
    b.y[:50] = b.y[50:100]
    _compare_tree(G, oracle, b, 32, (-50.0, 50.0, -50.0, 50.0))


@pytest.mark.parametrize("n,n_max", [(1, 32), (2, 1), (33, 32), (64, 32), (17, 1), (200, 4)])
def test_small_trees(G, oracle, n, n_max):
    from galax_gb300 import presets
    b = presets.uniform(n, seed=11)
    _compare_tree(G, oracle, b, n_max, presets.BOUNDS["uniform"])


def test_two_body_chain_known_answer(G, oracle):
    """(0.25,0.25),(0.75,0.75) with n_max=1 in [0,1]^2: the keys first share a prefix
    at shift 42, so rounds 1..20 are single-child chains: 2*21+1 = 43 nodes."""
    from galax_gb300 import Bodies
    b = Bodies.from_arrays([0.25, 0.75], [0.25, 0.75], [1.0, 2.0])
    t = _compare_tree(G, oracle, b, 1, (0.0, 1.0, 0.0, 1.0))
    assert t.n_nodes == 43


def test_nonfinite_positions(G, oracle):
    """NaN/inf positions before sanitising: NaN keys become 0 (Rust `as u64`)."""
    from galax_gb300 import presets
    b = presets.uniform(500, seed=2)
    b.x[3] = np.nan
    b.y[7] = np.inf
    b.x[11] = -np.inf
    _compare_tree(G, oracle, b, 16, presets.BOUNDS["uniform"])


@pytest.mark.parametrize("preset,n,n_max", [("uniform", 500, 16), ("plummer", 3000, 16), ("uniform", 4000, 32)])
def test_balanced_tree(G, oracle, preset, n, n_max):
    """build_constrained (lib.rs:541-588): no sort, iterative 2:1 split points."""
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=9)
    # build_constrained assumes Morton-sorted bodies: sort with Tree::build first
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass, b.vx, b.vy)
    oracle.tree_build(ob, n_max, presets.BOUNDS[preset])
    from galax_gb300 import Bodies
    sb = Bodies.from_arrays(ob.x, ob.y, ob.mass, ob.vx, ob.vy)
    _compare_tree(G, oracle, sb, n_max, presets.BOUNDS[preset], balanced=True)


def test_empty(G):
    from galax_gb300 import Bodies
    ctx = _ctx(G, 1)
    ctx.build_tree(Bodies.new(0), 32, (0.0, 1.0, 0.0, 1.0))
    assert ctx.tree_info()[0] == 0
    ctx.close()


@pytest.mark.parametrize("preset,n", [("plummer", 30_000), ("uniform", 7_001)])
def test_resident_rebuild_matches_host_build(G, oracle, preset, n):
    """gx_rebuild_resident: the same Morton order, tree and (lazily built) REF lists as
    Tree::build over the same bodies, and a permutation that maps the old order to the new."""
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=21)
    bounds = presets.BOUNDS[preset]
    ctx = _ctx(G, n)
    ctx.upload_bodies(b)
    perm = ctx.rebuild_resident(32, bounds, want_perm=True)
    out = G.Bodies.new(n)
    ctx.download_bodies(out)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass, b.vx, b.vy)
    t = oracle.tree_build(ob, 32, bounds)
    for name in ("x", "y", "vx", "vy", "mass"):
        assert np.array_equal(getattr(out, name), getattr(ob, name)), name
        assert np.array_equal(getattr(out, name), getattr(b, name)[perm]), name
    dt = ctx.export_tree()
    for f in FIELDS:
        assert np.array_equal(getattr(dt, f), getattr(t, f)), f
    v = oracle.vlist_build(t)
    vd, vl = ctx.export_lists(G.LIST_V)
    assert np.array_equal(vl, v.lengths) and np.array_equal(vd, v.data)
    ctx.close()


def test_rebuild_after_steps_sorts_the_moved_bodies(G, oracle):
    """Steps on a static tree, then a resident rebuild: the bodies come out in the
    Morton order of their new positions; the ACCURATE forces of the rebuilt tree match
    those of a fresh host build of the same bodies bit for bit."""
    from galax_gb300 import presets
    n = 20_001
    b = presets.galaxy(n, seed=22)
    bounds = presets.BOUNDS["galaxy"]
    ctx = _ctx(G, n)
    ctx.build_tree(b, 32, bounds)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.upload_bodies(b)
    ctx.forces_resident()
    ctx.kdk_run(5, 1e-2, 0)
    moved = G.Bodies.new(n)
    ctx.download_bodies(moved)
    ctx.rebuild_resident(32, bounds)
    ctx.forces_resident()
    out = G.Bodies.new(n)
    ctx.download_bodies(out)
    ob = oracle.Bodies.from_arrays(moved.x, moved.y, moved.mass, moved.vx, moved.vy)
    oracle.tree_build(ob, 32, bounds)
    assert np.array_equal(out.x, ob.x) and np.array_equal(out.y, ob.y)
    c2 = _ctx(G, n)
    fresh = moved.copy()
    c2.build_tree(fresh, 32, bounds)
    c2.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    c2.upload_bodies(fresh)
    c2.forces_resident()
    ref = G.Bodies.new(n)
    c2.download_bodies(ref)
    c2.close()
    ctx.close()
    assert np.array_equal(out.ax, ref.ax) and np.array_equal(out.ay, ref.ay)


def test_morton_keys_bit_exact_at_cell_boundaries(G, oracle):
    """morton_encode (lib.rs:95-109) on the device without a division per coordinate: keys
    equal the oracle's (IEEE division) for positions on, and one or two ulps either side
    of, cell boundaries, the box edges, out-of-box values, signed zeros, huge and denormal
    values, NaN and infinities, over three boxes, plus a million random bodies."""
    rng = np.random.default_rng(77)
    ctx = G.GpuContext(G.GpuConfig(max_n=1 << 21, max_nodes=1 << 20, p=4, eps64=0.1))
    boxes = [(-50.0, 50.0, -50.0, 50.0), (0.0, 100.0, 0.0, 100.0), (-0.3, 7.1, 1e-3, 1e-3 + 3.7)]
    for lo_x, hi_x, lo_y, hi_y in boxes:
        w = hi_x - lo_x
        k = rng.integers(0, 1 << 21, 20000)
        base = lo_x + (k / 2.0 ** 21) * w  # on (or one rounding from) a cell boundary
        xs = [base, np.nextafter(base, np.inf), np.nextafter(base, -np.inf),
              np.nextafter(np.nextafter(base, np.inf), np.inf), np.nextafter(np.nextafter(base, -np.inf), -np.inf)]
        special = np.array([lo_x, hi_x, np.nextafter(lo_x, -np.inf), np.nextafter(hi_x, np.inf),
                            np.nextafter(hi_x, -np.inf), lo_x - 1e-300, 0.0, -0.0, 1e308, -1e308, np.nan, np.inf,
                            -np.inf, lo_x + w * (1 - 1e-15), lo_x + w * (1 - 2.0 ** -21), lo_x + w * 2.0 ** -21,
                            5e-324, -5e-324])
        x = np.concatenate(xs + [special, rng.uniform(lo_x - 0.1 * w, hi_x + 0.1 * w, 100000)])
        y = np.concatenate([rng.uniform(lo_y, hi_y, x.size - special.size), special])
        y = y[rng.permutation(y.size)]
        got = ctx.morton_encode(x, y, (lo_x, hi_x, lo_y, hi_y))
        want = oracle.morton_encode_many(x, y, (lo_x, hi_x, lo_y, hi_y))
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, (lo_x, hi_x, bad[:5], x[bad[:5]], y[bad[:5]])
    x = rng.uniform(-60, 60, 1_000_000)
    y = rng.standard_normal(1_000_000) * 20
    assert np.array_equal(ctx.morton_encode(x, y, boxes[0]), oracle.morton_encode_many(x, y, boxes[0]))
    ctx.close()
