"""Reverse mode: the force VJP and the checkpointed reverse leapfrog (ACCURATE, FP64).

Not in the reference (galax has no gradients); checked against central finite
differences of the GPU forward with the tree frozen (h = 1e-6) and against the
oracle's exact FP64 N^2 adjoint (gxo_n2_vjp / gxo_n2_rollout_grad).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(G, b, bounds, eps, p=4, theta=0.5):
    n = len(b)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=p, eps64=eps))
    ctx.build_tree(b, 32, bounds)  # permutes b into tree order
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_FP64, theta)
    ctx.upload_bodies(b)
    ctx.forces_resident()  # builds the plan (lists, radii) once: the tree is frozen from here
    return ctx


def _forces(ctx, x, y, m):
    ax, ay = np.zeros(x.size), np.zeros(x.size)
    ctx.compute_forces(x, y, m, ax, ay)
    return ax, ay


@pytest.mark.parametrize("preset,n,p", [("plummer", 20_000, 4), ("uniform", 8_000, 2), ("galaxy", 6_001, 6),
                                          ("uniform", 4_000, 0), ("plummer", 6_000, 8)])
def test_force_vjp_matches_finite_differences(G, preset, n, p):
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=51)
    ctx = _ctx(G, b, presets.BOUNDS[preset], 0.05, p=p)
    rng = np.random.default_rng(1)
    lx, ly = rng.standard_normal(n), rng.standard_normal(n)
    gx, gy, gm = ctx.force_vjp(lx, ly)
    # h well below the closest pair separations (the FD truncation error goes as (h/r)^2)
    # and well above the rounding noise of the forces
    h = 1e-6
    for kind in ("positions", "masses", "both"):
        dx, dy, dm = rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n) * b.mass
        if kind == "positions":
            dm = np.zeros(n)
        elif kind == "masses":
            dx, dy = np.zeros(n), np.zeros(n)
        ap = _forces(ctx, b.x + h * dx, b.y + h * dy, b.mass + h * dm)
        am = _forces(ctx, b.x - h * dx, b.y - h * dy, b.mass - h * dm)
        fd = (np.dot(lx, ap[0] - am[0]) + np.dot(ly, ap[1] - am[1])) / (2 * h)
        an = np.dot(gx, dx) + np.dot(gy, dy) + np.dot(gm, dm)
        assert abs(fd - an) <= 1e-6 * abs(fd), (kind, fd, an)
    ctx.close()


def test_force_vjp_close_to_exact_n2_adjoint(G, oracle):
    """The VJP of the FMM approximates the VJP of the exact sum to FMM accuracy."""
    from galax_gb300 import presets
    n = 10_000
    b = presets.plummer(n, seed=52)
    ctx = _ctx(G, b, presets.BOUNDS["plummer"], 0.05)
    rng = np.random.default_rng(2)
    lx, ly = rng.standard_normal(n), rng.standard_normal(n)
    gx, gy, gm = ctx.force_vjp(lx, ly)
    rx, ry, rm = oracle.n2_vjp(b.x, b.y, b.mass, 0.05, lx, ly)
    ctx.close()
    ex = np.linalg.norm(np.hypot(gx - rx, gy - ry)) / np.linalg.norm(np.hypot(rx, ry))
    em = np.linalg.norm(gm - rm) / np.linalg.norm(rm)
    assert ex < 2e-3 and em < 2e-3, (ex, em)


def test_force_vjp_with_long_item_ranges_close_to_exact_n2_adjoint(G, oracle):
    """At an opening angle of 0.02 on 2500 leaves of 8 bodies nearly every pair is a
    direct (P2P) interaction and every leaf has more than 32 P2P items, whose partials
    are folded in groups before the ordered sum: the VJP is the exact sum's to rounding,
    in both forms."""
    from galax_gb300 import presets
    n = 20_000
    b = presets.uniform(n, seed=57)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.05))
    ctx.build_tree(b, 8, presets.BOUNDS["uniform"])
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_FP64, 0.02)
    ctx.upload_bodies(b)
    ctx.forces_resident()
    _, n_near, _ = ctx.plan_info()
    assert n_near > 32 * 32 * (n // 8)
    rng = np.random.default_rng(5)
    lx, ly = rng.standard_normal(n), rng.standard_normal(n)
    r64 = ctx.force_vjp(lx, ly)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.02)
    r32 = ctx.force_vjp(lx, ly)
    ctx.close()
    rx, ry, rm = oracle.n2_vjp(b.x, b.y, b.mass, 0.05, lx, ly)
    for gx, gy, gm, tol in ((*r64, 1e-6), (*r32, 1e-4)):
        ex = np.linalg.norm(np.hypot(gx - rx, gy - ry)) / np.linalg.norm(np.hypot(rx, ry))
        em = np.linalg.norm(gm - rm) / np.linalg.norm(rm)
        assert ex < tol and em < tol, (ex, em, tol)


def _rot(theta):
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c, -s], [s, c]])


def _loss_and_grads(x0, y0, xT, yT, R):
    """L = sum |x_T - R x_0|^2 (the rollout loss of the benchmark's adjoint config)."""
    tx = R[0, 0] * x0 + R[0, 1] * y0
    ty = R[1, 0] * x0 + R[1, 1] * y0
    rx, ry = xT - tx, yT - ty
    L = float(np.sum(rx * rx + ry * ry))
    # dL/dx_T and the direct dL/dx_0 = -2 R^T (x_T - R x_0)
    return L, 2 * rx, 2 * ry, -2 * (R[0, 0] * rx + R[1, 0] * ry), -2 * (R[0, 1] * rx + R[1, 1] * ry)


def _rollout(ctx, G, b, n_steps, dt):
    ctx.upload_bodies(b)
    ctx.forces_resident()
    ctx.kdk_run(n_steps, dt, 0)
    out = G.Bodies.new(len(b))
    ctx.download_bodies(out)
    return out


@pytest.mark.parametrize("k", [1, 4, 20])
def test_rollout_gradient_matches_finite_differences(G, k):
    from galax_gb300 import presets
    n, T, dt = 4_001, 20, 2e-3
    b = presets.galaxy(n, seed=53)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    R = _rot(0.3)
    ctx.upload_bodies(b)
    ctx.rollout_forward(T, dt, k)
    fin = G.Bodies.new(n)
    ctx.download_bodies(fin)
    L, lxT, lyT, dx0, dy0 = _loss_and_grads(b.x, b.y, fin.x, fin.y, R)
    gx, gy, gvx, gvy, gm, peak = ctx.rollout_backward(lxT, lyT, np.zeros(n), np.zeros(n))
    gx, gy = gx + dx0, gy + dy0
    assert peak > 0
    rng = np.random.default_rng(3)
    for _ in range(3):
        d = [rng.standard_normal(n) for _ in range(4)] + [rng.standard_normal(n) * b.mass]
        h = 1e-6
        def L_at(sign):
            p = G.Bodies.from_arrays(b.x + sign * h * d[0], b.y + sign * h * d[1], b.mass + sign * h * d[4],
                                     b.vx + sign * h * d[2], b.vy + sign * h * d[3])
            f = _rollout(ctx, G, p, T, dt)
            return _loss_and_grads(p.x, p.y, f.x, f.y, R)[0]
        fd = (L_at(1) - L_at(-1)) / (2 * h)
        an = np.dot(gx, d[0]) + np.dot(gy, d[1]) + np.dot(gvx, d[2]) + np.dot(gvy, d[3]) + np.dot(gm, d[4])
        assert abs(fd - an) <= 1e-5 * abs(fd), (fd, an)
    ctx.close()


def test_checkpoint_interval_does_not_change_the_gradient(G):
    """Recomputed segments are bit-identical to the forward pass."""
    from galax_gb300 import presets
    n, T, dt = 3_001, 12, 2e-3
    b = presets.galaxy(n, seed=54)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    res = []
    for k in (1, 5, 12):
        ctx.upload_bodies(b)
        ctx.rollout_forward(T, dt, k)
        fin = G.Bodies.new(n)
        ctx.download_bodies(fin)
        res.append(ctx.rollout_backward(fin.x, fin.y, fin.vx, np.zeros(n))[:5])
    ctx.close()
    for r in res[1:]:
        for a, c in zip(r, res[0]):
            assert np.array_equal(a, c)


def test_rollout_gradient_close_to_exact_n2_adjoint(G, oracle):
    """The FMM rollout gradient against the exact FP64 N^2 reverse leapfrog: a 2000-body
    galaxy (central mass and 1999 test particles), 100 steps."""
    from galax_gb300 import presets
    n, T, dt = 2_000, 100, 2e-3
    b = presets.galaxy(n, seed=55)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    R = _rot(-0.7)
    ctx.upload_bodies(b)
    ctx.rollout_forward(T, dt, 10)
    fin = G.Bodies.new(n)
    ctx.download_bodies(fin)
    L, lxT, lyT, dx0, dy0 = _loss_and_grads(b.x, b.y, fin.x, fin.y, R)
    g = ctx.rollout_backward(lxT, lyT, np.zeros(n), np.zeros(n))
    ctx.close()
    r = oracle.n2_rollout_grad(b.x, b.y, b.vx, b.vy, b.mass, 0.05, dt, T, lxT, lyT, np.zeros(n), np.zeros(n))
    for k in range(5):
        err = np.linalg.norm(g[k] - r[k]) / np.linalg.norm(r[k])
        assert err < 1e-3, (k, err)


def test_mixed_force_vjp_close_to_fp64(G):
    """The FP32 (mixed) VJP against the FP64 VJP of the same tree and lists."""
    from galax_gb300 import presets
    n = 20_000
    b = presets.plummer(n, seed=56)
    ctx = _ctx(G, b, presets.BOUNDS["plummer"], 0.05)
    rng = np.random.default_rng(4)
    lx, ly = rng.standard_normal(n), rng.standard_normal(n)
    r64 = ctx.force_vjp(lx, ly)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    r32 = ctx.force_vjp(lx, ly)
    ctx.close()
    ex = np.linalg.norm(np.hypot(r32[0] - r64[0], r32[1] - r64[1])) / np.linalg.norm(np.hypot(r64[0], r64[1]))
    em = np.linalg.norm(r32[2] - r64[2]) / np.linalg.norm(r64[2])
    assert ex < 1e-4 and em < 1e-4, (ex, em)


def _rollout_grad(ctx, G, b, T, dt, k, R):
    n = len(b)
    ctx.upload_bodies(b)
    ctx.rollout_forward(T, dt, k)
    fin = G.Bodies.new(n)
    ctx.download_bodies(fin)
    L, lxT, lyT, dx0, dy0 = _loss_and_grads(b.x, b.y, fin.x, fin.y, R)
    gx, gy, gvx, gvy, gm, peak = ctx.rollout_backward(lxT, lyT, np.zeros(n), np.zeros(n))
    return gx + dx0, gy + dy0, gvx, gvy, gm


def test_mixed_rollout_gradient_close_to_fp64(G):
    from galax_gb300 import presets
    n, T, dt = 4_001, 20, 2e-3
    b = presets.galaxy(n, seed=57)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    R = _rot(0.9)
    g64 = _rollout_grad(ctx, G, b, T, dt, 4, R)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    g32 = _rollout_grad(ctx, G, b, T, dt, 4, R)
    ctx.close()
    for k in range(5):
        err = np.linalg.norm(g32[k] - g64[k]) / np.linalg.norm(g64[k])
        assert err < 1e-3, (k, err)


def test_mixed_checkpoint_interval_does_not_change_the_gradient(G):
    from galax_gb300 import presets
    n, T, dt = 3_001, 13, 2e-3
    b = presets.galaxy(n, seed=58)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    R = _rot(0.2)
    res = [_rollout_grad(ctx, G, b, T, dt, k, R) for k in (1, 4, 13, 20)]
    ctx.close()
    for r in res[1:]:
        for a, c in zip(r, res[0]):
            assert np.array_equal(a, c)


def test_rollout_backward_needs_forward_and_same_precision(G):
    from galax_gb300 import presets
    n = 2_001
    b = presets.galaxy(n, seed=59)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    z = np.zeros(n)
    with pytest.raises(G.GpuError):
        ctx.rollout_backward(z, z, z, z)
    ctx.rollout_forward(3, 1e-3, 2)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    with pytest.raises(G.GpuError):
        ctx.rollout_backward(z, z, z, z)
    with pytest.raises(ValueError):
        ctx.force_vjp(z[:10], z[:10])
    ctx.close()


def _loss_ids(x0, y0, xT, yT, ids, R):
    """L = sum_i |x_T[i] - R x_0[ids[i]]|^2 with the final bodies in rebuilt order."""
    tx = R[0, 0] * x0[ids] + R[0, 1] * y0[ids]
    ty = R[1, 0] * x0[ids] + R[1, 1] * y0[ids]
    rx, ry = xT - tx, yT - ty
    d0x, d0y = np.zeros(x0.size), np.zeros(x0.size)
    d0x[ids] = -2 * (R[0, 0] * rx + R[1, 0] * ry)
    d0y[ids] = -2 * (R[0, 1] * rx + R[1, 1] * ry)
    return float(np.sum(rx * rx + ry * ry)), 2 * rx, 2 * ry, d0x, d0y


def _rebuild_grad(ctx, G, b, T, dt, k, R):
    n = len(b)
    ctx.upload_bodies(b)
    ctx.rollout_forward(T, dt, k, rebuild_every=1)
    ids = ctx.body_ids()
    fin = G.Bodies.new(n)
    ctx.download_bodies(fin)
    L, lxT, lyT, d0x, d0y = _loss_ids(b.x, b.y, fin.x, fin.y, ids, R)
    gx, gy, gvx, gvy, gm, _ = ctx.rollout_backward(lxT, lyT, np.zeros(n), np.zeros(n))
    return (gx + d0x, gy + d0y, gvx, gvy, gm), ids, lxT, lyT


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_rebuild_rollout_checkpoint_interval_bit_identical(G, prec):
    from galax_gb300 import presets
    n, T, dt = 3_001, 12, 5e-3
    b = presets.galaxy(n, seed=60)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    if prec == "mixed":
        ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    R = _rot(0.4)
    res = [_rebuild_grad(ctx, G, b, T, dt, k, R)[0] for k in (1, 5, 12)]
    ctx.close()
    for r in res[1:]:
        for a, c in zip(r, res[0]):
            assert np.array_equal(a, c)


def test_rebuild_rollout_gradient_close_to_exact_n2_adjoint(G, oracle):
    """100 steps with a tree rebuilt every step: the gradient in the bodies' starting
    order against the exact FP64 N^2 reverse leapfrog (2000-body galaxy)."""
    from galax_gb300 import presets
    n, T, dt = 2_000, 100, 5e-3
    b = presets.galaxy(n, seed=61)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    R = _rot(1.1)
    g, ids, lxT, lyT = _rebuild_grad(ctx, G, b, T, dt, 10, R)
    assert sorted(ids.tolist()) == list(range(n))
    ctx.close()
    # the oracle keeps the starting order: its terminal cotangents are ours un-permuted
    ox, oy = np.zeros(n), np.zeros(n)
    ox[ids], oy[ids] = lxT, lyT
    r = oracle.n2_rollout_grad(b.x, b.y, b.vx, b.vy, b.mass, 0.05, dt, T, ox, oy, np.zeros(n), np.zeros(n))
    direct = (-(R[0, 0] * ox + R[1, 0] * oy), -(R[0, 1] * ox + R[1, 1] * oy))
    r = (r[0] + direct[0], r[1] + direct[1], r[2], r[3], r[4])
    for k in range(5):
        err = np.linalg.norm(g[k] - r[k]) / np.linalg.norm(r[k])
        assert err < 2e-3, (k, err)


def test_kdk_rebuild_every_step_stays_finite_and_conserves_momentum(G):
    """The galaxy preset at the CLI time step: with a static tree the bodies leave their
    leaves and the expansions diverge within ~30 steps; rebuilding every step keeps the
    run finite and conserves momentum to FMM accuracy."""
    from galax_gb300 import presets
    n = 20_001
    b = presets.galaxy(n, seed=62)
    ctx = _ctx(G, b, presets.BOUNDS["galaxy"], 0.05)
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.upload_bodies(b)
    ctx.forces_resident()
    a0 = G.Bodies.new(n)
    ctx.download_bodies(a0)
    dt = presets.cli_dt(a0.ax, a0.ay)
    diag = ctx.kdk_run(60, dt, 20, rebuild_every=1)
    out = G.Bodies.new(n)
    ctx.download_bodies(out)
    ids = ctx.body_ids()
    ctx.close()
    assert np.all(np.isfinite(out.x)) and np.all(np.isfinite(out.vx))
    assert np.array_equal(out.mass, b.mass[ids])
    pscale = np.sum(b.mass * np.hypot(b.vx, b.vy))
    p0 = np.array([np.sum(b.mass * b.vx), np.sum(b.mass * b.vy)])
    assert np.all(np.abs(diag[:, 3:5] - p0) / pscale < 1e-3)


@pytest.mark.parametrize("rebuild", [0, 1])
def test_rollout_gradient_matches_frozen_tree_finite_differences(G, rebuild):
    """FP64 rollout gradient against central differences with every step's tree taken
    from the unperturbed trajectory (galax_gb300.fdcheck), static and rebuilt trees."""
    from galax_gb300 import fdcheck, presets
    n, T, dt = 3_001, 15, 5e-3
    bounds = presets.BOUNDS["galaxy"]
    b = presets.galaxy(n, seed=63)
    ctx = _ctx(G, b, bounds, 0.05)
    R = _rot(0.8)
    n_ = len(b)
    ctx.upload_bodies(b)
    ctx.rollout_forward(T, dt, 4, rebuild_every=rebuild)
    ids = ctx.body_ids() if rebuild else None
    fin = G.Bodies.new(n_)
    ctx.download_bodies(fin)
    L, lxT, lyT, d0x, d0y = fdcheck.rollout_loss(b.x, b.y, fin.x, fin.y, R, ids)
    gx, gy, gvx, gvy, gm, _ = ctx.rollout_backward(lxT, lyT, np.zeros(n_), np.zeros(n_))
    g = (gx + d0x, gy + d0y, gvx, gvy, gm)
    rng = np.random.default_rng(7)
    dirs = [[rng.standard_normal(n_) for _ in range(4)] + [rng.standard_normal(n_) * b.mass] for _ in range(3)]
    num = fdcheck.fd_frozen_trees(G, ctx, b, T, dt, R, dirs, 1e-6, 32, bounds, rebuild=bool(rebuild))
    ctx.close()
    for i, d in enumerate(dirs):
        an = sum(float(np.dot(g[q], d[q])) for q in range(5))
        assert abs(num[i] - an) <= 1e-5 * abs(num[i]), (i, num[i], an)
