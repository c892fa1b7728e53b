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
