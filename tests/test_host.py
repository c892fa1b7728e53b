"""Host-side logic: presets, GALX snapshots, the CLI's softening and dt rules."""
import io

import numpy as np
import pytest

from galax_gb300 import Bodies, galx_io, presets


def test_presets_shapes_and_masses():
    u = presets.uniform(1000, seed=1)
    assert u.x.min() >= 0 and u.x.max() <= 100 and 0.5 <= u.mass.min() and u.mass.max() <= 1.5
    assert np.all(u.vx == 0)
    p = presets.plummer(20000, seed=2)
    r = np.hypot(p.x, p.y)
    assert r.max() <= 10.0 and abs(p.mass.sum() - 1.0) < 1e-12
    # the radius is placed in the plane: its median is the half-mass radius
    # a/sqrt(2^(2/3) - 1) = 1.305a (slightly less after the r <= 10a truncation)
    assert 1.25 < np.median(r) < 1.32
    d = presets.disk(20000, seed=3)
    assert np.hypot(d.x, d.y).max() <= 60.0 and abs(d.mass.sum() - 1.0) < 1e-12
    g = presets.galaxy(2001, seed=4)
    assert g.mass[0] == 1000.0 and np.all(g.mass[1:] == 1e-6)
    rg = np.hypot(g.x[1:], g.y[1:])
    assert rg.min() >= 1.0 and rg.max() <= 50.0
    v = np.hypot(g.vx[1:], g.vy[1:])
    assert np.allclose(v, np.sqrt(1000.0 / rg))


def test_presets_are_seeded():
    a, b = presets.plummer(1000, seed=7), presets.plummer(1000, seed=7)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.vy, b.vy)


def test_galx_round_trip_and_errors():
    b = presets.disk(100, seed=5)
    b.ax[:] = np.arange(100)
    f = io.BytesIO()
    galx_io.write_snapshot(f, b, timestamp=1.5)
    raw = f.getvalue()
    assert raw[:4] == b"GALX" and len(raw) == 24 + 7 * 8 * 100
    r = galx_io.read_snapshot(io.BytesIO(raw))
    for k in ("x", "y", "vx", "vy", "mass", "ax", "ay"):
        assert np.array_equal(getattr(r, k), getattr(b, k))
    with pytest.raises(galx_io.SnapshotError):
        galx_io.read_snapshot(io.BytesIO(b"XXXX" + raw[4:]))
    with pytest.raises(galx_io.SnapshotError):
        galx_io.read_snapshot(io.BytesIO(raw[:4] + (2).to_bytes(4, "little") + raw[8:]))
    with pytest.raises(galx_io.SnapshotError):
        galx_io.read_snapshot(io.BytesIO(raw[:-8]))


def test_cli_rules_match_oracle(oracle):
    b = presets.uniform(3000, seed=6)
    ob = oracle.Bodies.from_arrays(b.x, b.y, b.mass)
    oracle.tree_build(ob, 32, presets.BOUNDS["uniform"])
    assert presets.cli_softening(ob.x, ob.y) == oracle.cli_softening(ob)
    ax, ay = np.array([3.0, -4.0]), np.array([4.0, 0.0])
    assert presets.cli_dt(ax, ay) == 0.5 / 5.0 ** 0.5
    assert presets.cli_dt(np.zeros(3), np.zeros(3)) == 0.01


def test_rollout_loss_partials_match_finite_differences():
    """galax_gb300.fdcheck.rollout_loss: L = sum_i |x_T[i] - R x_0[ids[i]]|^2 with the
    final bodies in a rebuilt (permuted) order."""
    import numpy as np
    from galax_gb300 import fdcheck
    rng = np.random.default_rng(0)
    n = 50
    x0, y0, xT, yT = (rng.standard_normal(n) for _ in range(4))
    ids = rng.permutation(n)
    c, s = np.cos(0.7), np.sin(0.7)
    R = np.array([[c, -s], [s, c]])
    L, lx, ly, d0x, d0y = fdcheck.rollout_loss(x0, y0, xT, yT, R, ids)
    h = 1e-6
    for arr, grad in ((xT, lx), (yT, ly), (x0, d0x), (y0, d0y)):
        for i in (0, 17, 49):
            old = arr[i]
            arr[i] = old + h
            lp = fdcheck.rollout_loss(x0, y0, xT, yT, R, ids)[0]
            arr[i] = old - h
            lm = fdcheck.rollout_loss(x0, y0, xT, yT, R, ids)[0]
            arr[i] = old
            assert abs((lp - lm) / (2 * h) - grad[i]) < 1e-6 * max(1.0, abs(grad[i]))
    # identity order by default
    L2 = fdcheck.rollout_loss(x0, y0, xT, yT, R)[0]
    L3 = fdcheck.rollout_loss(x0, y0, xT, yT, R, np.arange(n))[0]
    assert L2 == L3


def test_magnitude_error_metric_known_values():
    """validate_fmm's per-body metric (galax-core/src/lib.rs:1553-1557): the magnitudes
    are compared, not the vectors, and a zero exact force divides by 1e-20."""
    from galax_gb300 import _mag_rel_err
    ax, ay = np.array([3.0, 0.0, 1.0, 0.0]), np.array([4.0, 2.0, 0.0, 1e-30])
    ex, ey = np.array([0.0, 0.0, 2.0, 0.0]), np.array([5.0, 1.0, 0.0, 0.0])
    r = _mag_rel_err(ax, ay, ex, ey)
    assert r[0] == 0.0  # same magnitude, different direction
    assert r[1] == 1.0 and r[2] == 0.5
    assert r[3] == 1e-30 / 1e-20
