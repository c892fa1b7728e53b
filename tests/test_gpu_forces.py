"""Force evaluation through the C ABI against the oracle.

REF mode must match compute_fmm_force (galax-core/src/lib.rs:1466-1499) within
1e-10 relative per body (vector metric, |a*| floored at 1e-30).  EXACT and
ACCURATE FP64 modes match the oracle's restatement of the same algorithm within
1e-10.  The mixed-precision form is checked against the FP64 form (1e-4 median)
and both against the exact FP64 N^2 sum.
"""
import numpy as np
import pytest

from helpers import oracle_case, rel_vec_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10


def _run_gpu(G, b_sorted, t, v, u, p, eps, mode, prec=0, theta=0.5, via="upload"):
    n = len(b_sorted.x)
    ctx = G.GpuContext(G.GpuConfig(max_n=max(n, 1), max_nodes=1 << 26, p=p, eps64=eps))
    ctx.set_mode(mode, prec, theta)
    if via == "upload":
        ctx.upload_tree_data(t, v, u)
    ax, ay = np.zeros(n), np.zeros(n)
    x, y, m = b_sorted.x.copy(), b_sorted.y.copy(), b_sorted.mass.copy()
    if via == "build":
        gb = G.Bodies.from_arrays(x, y, m)
        ctx.build_tree(gb, t.n_max, t.bounds)
        x, y, m = gb.x, gb.y, gb.mass
    if mode == G.MODE_ACCURATE:
        ctx.upload_bodies(G.Bodies.from_arrays(x, y, m))
    ctx.compute_forces(x, y, m, ax, ay)
    ctx.close()
    return ax, ay


@pytest.mark.parametrize("preset,n,p", [("uniform", 10_000, 4), ("plummer", 20_000, 4), ("galaxy", 5_001, 4),
                                        ("uniform", 3_000, 2), ("uniform", 3_000, 0)])
@pytest.mark.parametrize("via", ["upload", "build"])
def test_ref_mode_matches_oracle(G, oracle, preset, n, p, via):
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=1)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS[preset], p)
    ref = ob.copy()
    oracle.compute_fmm_force(ref, t, v, u, p, eps, oracle.MODE_REF)
    ax, ay = _run_gpu(G, ob, t, v, u, p, eps, G.MODE_REF, via=via)
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64, f"max {err.max():.3e} at body {err.argmax()}"


@pytest.mark.parametrize("p", [1, 3, 6, 8])
def test_ref_mode_orders(G, oracle, p):
    from galax_gb300 import presets
    b = presets.uniform(2_000, seed=4)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS["uniform"], p)
    ref = ob.copy()
    oracle.compute_fmm_force(ref, t, v, u, p, eps, oracle.MODE_REF)
    ax, ay = _run_gpu(G, ob, t, v, u, p, eps, G.MODE_REF)
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64


def test_exact_mode_matches_oracle(G, oracle):
    from galax_gb300 import presets
    b = presets.uniform(10_000, seed=2)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS["uniform"], 4)
    ref = ob.copy()
    oracle.compute_fmm_force(ref, t, v, u, 4, eps, oracle.MODE_EXACT)
    ax, ay = _run_gpu(G, ob, t, v, u, 4, eps, G.MODE_EXACT)
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64


@pytest.mark.parametrize("preset,n", [("uniform", 10_000), ("plummer", 30_000)])
def test_accurate_mode_fp64_matches_oracle(G, oracle, preset, n):
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=6)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS[preset], 4)
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.5)
    ref = ob.copy()
    oracle.compute_fmm_force_mac(ref, t, far, near, 4, eps)
    ax, ay = _run_gpu(G, ob, t, v, u, 4, eps, G.MODE_ACCURATE, theta=0.5)
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64, f"max {err.max():.3e}"


def test_accurate_plan_regrows_its_storage(G, oracle):
    """A tiny opening angle (0.02) on 2500 leaves of 8 bodies: almost every leaf pair is
    near (6.2M leaf near pairs, more list units and entries than the plan's first
    capacities), so the plan overflows, grows its arrays and is redone.  The lists and
    forces must equal the oracle's, in the FP64 and the mixed form."""
    from galax_gb300 import presets
    n = 20_000
    b = presets.uniform(n, seed=11)
    ob, t, v, u, eps = oracle_case(oracle, b, 8, presets.BOUNDS["uniform"], 4)
    R = oracle.node_radii(ob, t)
    far, near = oracle.mac_lists_build(t, R, 0.02)
    ref = ob.copy()
    oracle.compute_fmm_force_mac(ref, t, far, near, 4, eps)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=eps))
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_FP64, 0.02)
    ctx.upload_tree_data(t, v, u)
    ctx.upload_bodies(G.Bodies.from_arrays(ob.x.copy(), ob.y.copy(), ob.mass.copy()))
    ax, ay = np.zeros(n), np.zeros(n)
    ctx.compute_forces(ob.x.copy(), ob.y.copy(), ob.mass.copy(), ax, ay)
    n_far, n_near, _ = ctx.plan_info()
    # the mixed form on the same plan: every leaf has ~80 P2P items (> 32), so its
    # partials are folded in groups before the ordered sum
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.02)
    mx, my = np.zeros(n), np.zeros(n)
    ctx.compute_forces(ob.x.copy(), ob.y.copy(), ob.mass.copy(), mx, my)
    ctx.close()
    assert n_far == far.off[-1]
    assert n_near == int(np.diff(near.off)[: t.n_leaves].sum())
    assert n_near > 32 * 32 * t.n_leaves  # more than 32 items of 32 source leaves per leaf on average
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert err.max() < TOL_FP64, f"max {err.max():.3e}"
    e32 = rel_vec_err(mx, my, ref.ax, ref.ay)
    assert np.median(e32) < 1e-5 and e32.max() < 1e-3, (np.median(e32), e32.max())


@pytest.mark.parametrize("preset,n", [("uniform", 10_000), ("plummer", 30_000)])
def test_mixed_precision_error_budget(G, oracle, preset, n):
    """Mixed form vs FP64 form, and both vs the exact FP64 N^2 sum on 1000 samples:
    median relative force error <= 1e-4."""
    from galax_gb300 import presets
    b = presets.make(preset, n, seed=8)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS[preset], 4)
    a64 = _run_gpu(G, ob, t, v, u, 4, eps, G.MODE_ACCURATE, G.PREC_FP64)
    a32 = _run_gpu(G, ob, t, v, u, 4, eps, G.MODE_ACCURATE, G.PREC_MIXED)
    idx = np.random.default_rng(0).choice(n, 1000, replace=False)
    ex, ey = oracle.n2_sampled(ob.x, ob.y, ob.mass, eps, idx)
    e64 = rel_vec_err(a64[0][idx], a64[1][idx], ex, ey)
    e32 = rel_vec_err(a32[0][idx], a32[1][idx], ex, ey)
    d = rel_vec_err(a32[0], a32[1], a64[0], a64[1])
    assert np.median(e64) <= 1e-4, np.median(e64)
    assert np.median(e32) <= 1e-4, np.median(e32)
    assert np.median(d) < 1e-5, np.median(d)


def test_sanitised_inputs_match_oracle(G, oracle):
    """compute_fmm_force zeroes invalid positions and sets bad masses to 1 (lib.rs:1474-1482)."""
    from galax_gb300 import presets
    b = presets.uniform(3_000, seed=12)
    ob, t, v, u, eps = oracle_case(oracle, b, 32, presets.BOUNDS["uniform"], 4)
    bad = ob.copy()
    bad.mass[5] = -1.0
    bad.mass[9] = np.nan
    bad.x[17] = 1e101
    bad.y[23] = np.inf
    ref = bad.copy()
    oracle.compute_fmm_force(ref, t, v, u, 4, eps, oracle.MODE_REF)
    ax, ay = _run_gpu(G, bad, t, v, u, 4, eps, G.MODE_REF)
    err = rel_vec_err(ax, ay, ref.ax, ref.ay)
    assert np.all(np.isfinite(ax)) and err.max() < TOL_FP64
    # the sanitising is reported by gx_last_status, and a clean call clears it
    ctx = G.GpuContext(G.GpuConfig(max_n=len(bad.x), max_nodes=1 << 20, p=4, eps64=eps))
    ctx.upload_tree_data(t, v, u)
    ax2, ay2 = np.zeros(len(bad.x)), np.zeros(len(bad.x))
    ctx.compute_forces(bad.x.copy(), bad.y.copy(), bad.mass.copy(), ax2, ay2)
    assert ctx.last_status() == G.STATUS_SANITIZED
    ctx.compute_forces(ob.x.copy(), ob.y.copy(), ob.mass.copy(), ax2, ay2)
    assert ctx.last_status() == 0
    ctx.close()


def test_p2p_only_at_p0_equals_p2p(G, oracle):
    """test_fmm_p0_equals_p2p (lib.rs:2320-2357): at p=0 the far field vanishes."""
    n = 200
    t_ = np.arange(n) / n
    from galax_gb300 import Bodies
    b = Bodies.from_arrays(5 + 90 * np.modf(t_ * 3.7)[0], 5 + 90 * np.modf(t_ * 7.3)[0],
                           0.1 + 10 * np.modf(t_ * 11.0)[0])
    ob, t, v, u, _ = oracle_case(oracle, b, 16, (0.0, 100.0, 0.0, 100.0), 0)
    pp = ob.copy()
    oracle.p2p(pp, t, u, 0.1)
    ax, ay = _run_gpu(G, ob, t, v, u, 0, 0.1, G.MODE_REF)
    assert np.max(np.abs(ax - pp.ax)) < 1e-12 and np.max(np.abs(ay - pp.ay)) < 1e-12


@pytest.mark.parametrize("p", [6, 8])
def test_mixed_high_order_dense_cluster_stays_finite(G, p):
    """100k bodies in the unit square: far pairs at R ~ 0.04, where the order-2p
    derivatives (R^-(4p+1) (2p)!) exceed the FP32 range at p = 8.  The FP32 M2L forms
    them at unit distance and rescales the operands; the mixed forces stay finite and
    agree with the FP64 form."""
    n = 100_000
    rng = np.random.default_rng(31)
    b = G.Bodies.from_arrays(rng.uniform(0, 1, n), rng.uniform(0, 1, n), np.full(n, 1.0 / n))
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=p, eps64=1e-3))
    ctx.build_tree(b, 32, (0.0, 1.0, 0.0, 1.0))
    ctx.upload_bodies(b)
    out = {}
    for name, prec in (("fp64", G.PREC_FP64), ("mixed", G.PREC_MIXED)):
        ctx.set_mode(G.MODE_ACCURATE, prec, 0.5)
        ctx.forces_resident()
        r = G.Bodies.new(n)
        ctx.download_bodies(r)
        out[name] = (r.ax.copy(), r.ay.copy())
    ctx.close()
    assert np.all(np.isfinite(out["mixed"][0])) and np.all(np.isfinite(out["mixed"][1]))
    d = rel_vec_err(out["mixed"][0], out["mixed"][1], out["fp64"][0], out["fp64"][1])
    assert np.median(d) < 1e-5, np.median(d)


def test_near_field_alone_gives_the_same_forces(G):
    """gx_bench_forces(which=2) starts the near field after the far-field chain instead of
    beside it: a measurement mode that must not change a single bit of the result."""
    from galax_gb300 import presets
    n = 50_000
    b = presets.plummer(n, seed=31)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.05))
    ctx.build_tree(b, 32, presets.BOUNDS["plummer"])
    ctx.set_mode(G.MODE_ACCURATE, G.PREC_MIXED, 0.5)
    ctx.upload_bodies(b)
    ctx.forces_resident()
    r0 = G.Bodies.new(n)
    ctx.download_bodies(r0)
    ms, kms = ctx.bench_forces(2, False, 2)
    r1 = G.Bodies.new(n)
    ctx.download_bodies(r1)
    ctx.close()
    assert np.all(kms > 0) and np.all(ms >= kms)
    assert np.array_equal(r0.ax, r1.ax) and np.array_equal(r0.ay, r1.ay)


@pytest.mark.parametrize("mode,prec", [(0, 0), (2, 1)])
def test_compute_forces_into_pinned_arrays(G, mode, prec):
    """Page-locked and pageable host arrays give the same bits through
    gx_compute_forces (the page-locked ones are read and written by the kernels
    themselves once the plan exists), on a tree built here and again after a device
    rebuild, and inputs to sanitise are sanitised the same way."""
    from galax_gb300 import presets
    n = 30_001
    b = presets.plummer(n, seed=41)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.05))
    ctx.build_tree(b, 32, presets.BOUNDS["plummer"])
    ctx.set_mode(mode, prec, 0.5)
    ctx.upload_bodies(b)
    hx, hy, hm, pax, pay = (G.HostArray(n) for _ in range(5))
    for rnd in range(2):
        if rnd == 1:
            b.x += 0.01 * np.sin(b.y)
            ctx.upload_bodies(b)
            perm = ctx.rebuild_resident(32, presets.BOUNDS["plummer"], want_perm=True)
            for k in ("x", "y", "mass", "vx", "vy"):
                setattr(b, k, getattr(b, k)[perm])
        ax, ay = np.zeros(n), np.zeros(n)
        ctx.compute_forces(b.x, b.y, b.mass, ax, ay)
        hx.array[:] = b.x
        hy.array[:] = b.y
        hm.array[:] = b.mass
        pax.array[:] = np.nan
        pay.array[:] = np.nan
        ctx.compute_forces(hx.array, hy.array, hm.array, pax.array, pay.array)
        assert np.array_equal(ax, pax.array) and np.array_equal(ay, pay.array)
        assert ctx.last_status() == 0
        # a non-finite position and a negative mass, through both routes
        xin, min_ = b.x.copy(), b.mass.copy()
        xin[5], min_[7] = np.nan, -1.0
        ctx.compute_forces(xin, b.y, min_, ax, ay)
        assert ctx.last_status() == G.STATUS_SANITIZED
        hx.array[:] = xin
        hm.array[:] = min_
        ctx.compute_forces(hx.array, hy.array, hm.array, pax.array, pay.array)
        assert ctx.last_status() == G.STATUS_SANITIZED
        assert np.array_equal(ax, pax.array) and np.array_equal(ay, pay.array)
    ctx.close()


@pytest.mark.parametrize("n_max", [8, 16, 64])
def test_mixed_form_with_other_leaf_sizes(G, n_max):
    """Leaves of at most 16 bodies take the one-target P2P kernel, larger leaves than a
    warp the chunked one: the mixed form stays within FP32 rounding of the FP64 form."""
    from galax_gb300 import presets
    n = 40_000
    b = presets.plummer(n, seed=51)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=4, eps64=0.05))
    ctx.build_tree(b, n_max, presets.BOUNDS["plummer"])
    ctx.upload_bodies(b)
    out = {}
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        ctx.set_mode(G.MODE_ACCURATE, prec, 0.5)
        ctx.forces_resident()
        r = G.Bodies.new(n)
        ctx.download_bodies(r)
        out[prec] = r
    ctx.close()
    d = rel_vec_err(out[G.PREC_MIXED].ax, out[G.PREC_MIXED].ay, out[G.PREC_FP64].ax, out[G.PREC_FP64].ay)
    assert np.isfinite(d).all()
    assert np.median(d) < 2e-6 and np.percentile(d, 99) < 1e-4


@pytest.mark.parametrize("p", [1, 2, 3])
def test_mixed_form_at_low_orders(G, p):
    """The mixed form below p = 4 (the FP32 instantiations for p = 1..3) stays within FP32
    rounding of the FP64 form on the same tree and lists."""
    from galax_gb300 import presets
    n = 30_000
    b = presets.plummer(n, seed=57)
    ctx = G.GpuContext(G.GpuConfig(max_n=n, max_nodes=1 << 22, p=p, eps64=0.05))
    ctx.build_tree(b, 32, presets.BOUNDS["plummer"])
    ctx.upload_bodies(b)
    out = {}
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        ctx.set_mode(G.MODE_ACCURATE, prec, 0.5)
        ctx.forces_resident()
        r = G.Bodies.new(n)
        ctx.download_bodies(r)
        out[prec] = r
    n_far = ctx.plan_info()[0]
    ctx.close()
    assert n_far > 0
    d = rel_vec_err(out[G.PREC_MIXED].ax, out[G.PREC_MIXED].ay, out[G.PREC_FP64].ax, out[G.PREC_FP64].ay)
    assert np.isfinite(d).all()
    assert np.median(d) < 2e-6 and np.percentile(d, 99) < 1e-4, (np.median(d), np.percentile(d, 99))
