"""Device-resident leapfrog, diagnostics and the sampled exact sum against the oracle.

simulate / leapfrog_kdk (galax-integrate/src/lib.rs:158-237), diagnostics
(galax-core/src/lib.rs:1638-1683), validate_fmm's exact sum (lib.rs:1537-1553)
and compute_n2_force (lib.rs:1685-1721).
"""
import numpy as np
import pytest

from helpers import oracle_case, rel_vec_err

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1e-300)


def test_config1_uniform_10k_ten_steps(G, oracle):
    """Uniform 10k in [0,100]^2, p=4, n_max=32, CLI softening, dt = 0.5/sqrt(max|a|),
    10 KDK steps with the static tree; diagnostics every step."""
    from galax_gb300 import presets
    n, p = 10_000, 4
    b = presets.uniform(n, seed=0)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS["uniform"], p)
    ref = ob.copy()
    oracle.compute_fmm_force(ref, t, v, u, p, eps, oracle.MODE_REF)  # initial forces (galax-cli/src/main.rs:230)
    dt = oracle.cli_dt(ref.ax, ref.ay)
    diag_ref = oracle.simulate(ref, t, v, u, p, eps, dt, 10, 1, oracle.MODE_REF)

    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=p, eps64=eps))
    gb = b.copy()
    ctx.build_tree(gb, 32, presets.BOUNDS["uniform"])
    assert np.array_equal(gb.x, ob.x)
    ctx.upload_bodies(gb)
    ctx.forces_resident()
    g0 = G.Bodies.new(n)
    ctx.download_bodies(g0)
    assert presets.cli_dt(g0.ax, g0.ay) == pytest.approx(dt, rel=1e-12)
    diag = ctx.kdk_run(10, dt, 1)
    out = G.Bodies.new(n)
    ctx.download_bodies(out)
    ctx.close()
    scale = np.max(np.abs(ref.x))
    assert np.max(np.abs(out.x - ref.x)) / scale < 1e-10 and np.max(np.abs(out.y - ref.y)) / scale < 1e-10
    vs = np.max(np.hypot(ref.vx, ref.vy))
    assert np.max(np.abs(out.vx - ref.vx)) / vs < 1e-10 and np.max(np.abs(out.vy - ref.vy)) / vs < 1e-10
    assert rel_vec_err(out.ax, out.ay, ref.ax, ref.ay).max() < 1e-10
    assert diag.shape == diag_ref.shape == (10, 6)
    assert np.array_equal(diag[:, 0], diag_ref[:, 0])
    for col in (1, 2, 5):  # KE, FMM PE, Lz
        assert _rel(diag[:, col], diag_ref[:, col]).max() < 1e-10
    pscale = np.sum(ref.mass * np.hypot(ref.vx, ref.vy))
    assert np.max(np.abs(diag[:, 3:5] - diag_ref[:, 3:5])) / pscale < 1e-10


def test_diagnostics_known_values(G):
    """galax-integrate/src/lib.rs:33-54."""
    b = G.Bodies(np.array([0.0, 3.0]), np.array([0.0, 0.0]), np.array([2.0, -1.0]), np.array([1.0, 2.0]),
                 np.array([5.0, 3.0]), np.array([0.5, -0.3]), np.array([0.0, 0.1]))
    ctx = G.GpuContext(G.GpuConfig(max_n=2, p=4, eps64=0.1))
    ctx.upload_bodies(b)
    ke, pe, px, py, lz = ctx.diagnostics()
    ctx.close()
    assert abs(ke - 20.0) < 1e-14 and abs(px - 7.0) < 1e-14 and abs(py - 11.0) < 1e-14 and abs(lz - 18.0) < 1e-14
    # FMM PE: -1/2 sum m |a| max(r, 1)
    e = -0.5 * (5.0 * 0.5 * 1.0 + 3.0 * np.hypot(0.3, 0.1) * 3.0)
    assert abs(pe - e) < 1e-14


def test_single_body_drift(G):
    """galax-integrate/src/lib.rs:9-30 on the device."""
    b = G.Bodies.from_arrays([0.0], [0.0], [1.0], [10.0], [5.0])
    ctx = G.GpuContext(G.GpuConfig(max_n=1, p=2, eps64=0.1))
    ctx.build_tree(b, 32, (-100.0, 100.0, -100.0, 100.0))
    ctx.upload_bodies(b)
    ctx.kdk_run(1, 0.1, 0)
    out = G.Bodies.new(1)
    ctx.download_bodies(out)
    ctx.close()
    assert out.vx[0] == 10.0 and out.vy[0] == 5.0
    assert abs(out.x[0] - 1.0) < 1e-14 and abs(out.y[0] - 0.5) < 1e-14


@pytest.mark.parametrize("preset,n", [("plummer", 20_000), ("galaxy", 5_001)])
def test_sampled_n2_matches_oracle(G, oracle, preset, n):
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=12)
    eps = 0.05
    ctx = G.GpuContext(G.GpuConfig(max_n=n, p=4, eps64=eps))
    ctx.upload_bodies(b)
    idx = np.random.default_rng(3).choice(n, 500, replace=False)
    ax, ay = ctx.n2_sampled(idx)
    rx, ry = oracle.n2_sampled(b.x, b.y, b.mass, eps, idx)
    assert rel_vec_err(ax, ay, rx, ry).max() < 1e-12
    full = ctx.n2_debug(G.Bodies.from_arrays(b.x[:3000], b.y[:3000], b.mass[:3000]))
    ob = oracle.Bodies.from_arrays(b.x[:3000], b.y[:3000], b.mass[:3000])
    oracle.n2_force(ob, eps)
    assert rel_vec_err(full[0], full[1], ob.ax, ob.ay).max() < 1e-12
    ctx.close()


def test_validate_fmm_and_n2_regression_match_the_oracle(G, oracle):
    """validate_fmm / n2_regression (galax-core/src/lib.rs:1502-1598) in REF mode: the
    sampled magnitude errors equal the ones formed from the oracle's REF FMM and exact
    sum on the same samples; n2_regression refuses N > 2000."""
    from galax_gb300 import presets
    n, p = 5_000, 4
    b = presets.uniform(n, seed=21)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS["uniform"], p)
    ref = ob.copy()
    oracle.compute_fmm_force(ref, t, v, u, p, eps, oracle.MODE_REF)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 20, p=p, eps64=eps))
    gb = b.copy()
    ctx.build_tree(gb, 32, presets.BOUNDS["uniform"])
    k, mx, mean, zero = ctx.validate_fmm(gb, 400, seed=5)
    idx = np.sort(np.random.default_rng(5).permutation(n)[:400])
    rx, ry = oracle.n2_sampled(ob.x, ob.y, ob.mass, eps, idx)
    rel = G._mag_rel_err(ref.ax[idx], ref.ay[idx], rx, ry)
    assert (k, zero) == (400, 0.0)
    assert mx == pytest.approx(float(rel.max()), rel=1e-8)
    assert mean == pytest.approx(float(rel.mean()), rel=1e-8)
    # N <= 2000: the full regression
    m = 1_500
    b2 = presets.uniform(m, seed=22)
    ob2, t2, v2, u2, eps2 = oracle_case(oracle, b2, 32, presets.BOUNDS["uniform"], p)
    ref2 = ob2.copy()
    oracle.compute_fmm_force(ref2, t2, v2, u2, p, eps2, oracle.MODE_REF)
    d2 = ob2.copy()
    oracle.n2_force(d2, eps2)
    c2 = G.GpuContext(G.GpuConfig(max_n=m, max_nodes=1 << 20, p=p, eps64=eps2))
    g2 = b2.copy()
    c2.build_tree(g2, 32, presets.BOUNDS["uniform"])
    got = c2.n2_regression(g2)
    want = float(G._mag_rel_err(ref2.ax, ref2.ay, d2.ax, d2.ay).max())
    assert got == pytest.approx(want, rel=1e-8)
    with pytest.raises(ValueError):
        ctx.n2_regression(gb)
    ctx.close()
    c2.close()


def test_convergence_table_matches_the_oracle(G, oracle):
    """galax-cli --convergence (galax-cli/src/main.rs:355-377) on a 5k uniform case after
    5 leapfrog steps (the CLI runs it on the final, drifted state): build_constrained on
    the bodies as ordered, the reference's V/U lists, validate_fmm at p in {2,4,6,8}.
    The table equals the one formed from the oracle's constrained tree, REF FMM and
    exact sum on the same samples."""
    from galax_gb300 import presets
    n, n_max, T = 5_000, 32, 5
    bounds = presets.BOUNDS["uniform"]
    b = presets.uniform(n, seed=23)
    ob, t, v, u, eps = oracle_case(oracle, b, n_max, bounds, 4)
    oracle.compute_fmm_force(ob, t, v, u, 4, eps, oracle.MODE_REF)
    dt = oracle.cli_dt(ob.ax, ob.ay)
    oracle.simulate(ob, t, v, u, 4, eps, dt, T, 0, oracle.MODE_REF)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 20, p=4, eps64=eps))
    state = G.Bodies.from_arrays(ob.x, ob.y, ob.mass, ob.vx, ob.vy)
    rows = ctx.convergence(state, n_max, bounds, eps, sample_size=400, seed=7)
    # the oracle's table: ref_bodies = copies of x, y, mass (main.rs:358-361)
    cb = oracle.Bodies.from_arrays(ob.x, ob.y, ob.mass)
    tc = oracle.tree_build_constrained(cb, n_max, bounds, accel=True)
    vc, uc = oracle.vlist_build(tc), oracle.ulist_build(tc)
    idx = np.sort(np.random.default_rng(7).permutation(n)[:400])
    rx, ry = oracle.n2_sampled(cb.x, cb.y, cb.mass, eps, idx)
    assert [r[0] for r in rows] == [2, 4, 6, 8]
    for p, k, mx, mean in rows:
        f = cb.copy()
        oracle.compute_fmm_force(f, tc, vc, uc, p, eps, oracle.MODE_REF)
        rel = G._mag_rel_err(f.ax[idx], f.ay[idx], rx, ry)
        assert k == 400
        assert mx == pytest.approx(float(rel.max()), rel=1e-8), p
        assert mean == pytest.approx(float(rel.mean()), rel=1e-8), p
    ctx.close()


def test_accurate_mixed_kdk_conserves_momentum(G):
    """The mixed ACCURATE form over 20 steps of the galaxy preset: total momentum stays
    at its initial value relative to sum m|v| (the reference has no device check of this)."""
    from galax_gb300 import presets
    n = 20_001
    b = presets.galaxy(n, seed=13)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.05))
    ctx.build_tree(b, 32, presets.BOUNDS["galaxy"])
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.upload_bodies(b)
    ctx.forces_resident()
    diag = ctx.kdk_run(20, 1e-3, 10)
    ctx.close()
    pscale = np.sum(b.mass * np.hypot(b.vx, b.vy))
    p0 = np.array([np.sum(b.mass * b.vx), np.sum(b.mass * b.vy)])
    assert diag.shape == (2, 6)
    assert np.all(np.abs(diag[:, 3:5] - p0) / pscale < 1e-5)


def test_simulate_writes_snapshots_in_upload_order(G, tmp_path):
    """simulate() with --snap-every semantics: GALX snapshots every k steps, bodies in
    the order of the upload although the tree (and the resident order) is rebuilt every
    step; the last snapshot equals the final state."""
    import io
    from galax_gb300 import galx_io, presets
    n = 5_001
    b = presets.galaxy(n, seed=14)
    bounds = presets.BOUNDS["galaxy"]
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.05))
    ctx.build_tree(b, 32, bounds)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.upload_bodies(b)
    ctx.forces_resident()
    snaps = {}

    def snapshot(step, bodies):
        f = io.BytesIO()
        galx_io.write_snapshot(f, bodies, timestamp=float(step))
        snaps[step] = f.getvalue()

    diag = ctx.simulate(12, 2e-3, energy_every=4, snap_every=4, snapshot=snapshot, rebuild_every=1)
    final = G.Bodies.new(n)
    ctx.download_bodies(final)
    ids = ctx.body_ids()
    ctx.close()
    assert sorted(snaps) == [4, 8, 12]
    assert diag.shape == (3, 6) and list(diag[:, 0]) == [4.0, 8.0, 12.0]
    last = galx_io.read_snapshot(io.BytesIO(snaps[12]))
    assert np.array_equal(last.x[ids], final.x) and np.array_equal(last.vy[ids], final.vy)
    assert np.array_equal(last.mass, b.mass)  # upload order
