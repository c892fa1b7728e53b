"""The C ABI library builds for sm_103a, loads, and exports every entry point that
the headers under include/ declare (the product header galax_gb300.h and the
measurement header galax_gb300_bench.h); host-side argument checks work without a
GPU."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "galax_gb300.h")
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


def declared_functions(headers=None):
    names = set()
    for h in headers or HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"^\s*(?:int|void|const char)\s*\*?\s*(gx_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_functions([HEADER])
    for must in ["gx_create", "gx_destroy", "gx_upload_tree", "gx_build_tree", "gx_compute_forces", "gx_kdk_run",
                 "gx_n2_sampled", "gx_export_tree", "gx_export_lists", "gx_last_error"]:
        assert must in names
    # measurement probes live in the bench header, not in the product boundary
    assert "gx_probe_fp32_tflops" not in names and "gx_bench_forces" not in names
    assert "gx_probe_fp32_tflops" in declared_functions() and "gx_bench_forces" in declared_functions()


def test_library_exports_every_declared_symbol(G):
    lib = C.CDLL(G.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_defaults(G):
    L = G.lib()
    assert L.gx_abi_version() == 1
    cfg = G._Config()
    assert L.gx_config_default(C.byref(cfg)) == 0
    assert (cfg.max_n, cfg.max_nodes, cfg.max_interactions, cfg.p) == (262144, 524288, 1 << 24, 4)
    assert abs(cfg.eps - 0.1) < 1e-7


def test_invalid_arguments_are_rejected_without_a_device(G):
    L = G.lib()
    assert L.gx_create(None, None) == 4
    h = C.c_void_p()
    cfg = G._Config()
    L.gx_config_default(C.byref(cfg))
    cfg.p = 17
    assert L.gx_create(C.byref(cfg), C.byref(h)) == 4
    assert L.gx_last_error(None) == b"null context"
    assert L.gx_set_mode(None, 0, 0, 0.5) == 4
    # entry points beyond the reference's API: null contexts are rejected, no device touched
    bounds = (C.c_double * 4)(0.0, 1.0, 0.0, 1.0)
    assert L.gx_rebuild_resident(None, 32, bounds, 0, None) == 4
    assert L.gx_kdk_run_rebuild(None, 1, 0.1, 0, 1, None, None) == 4
    assert L.gx_body_ids(None, None) == 4
    assert L.gx_force_vjp(None, None, None, None, None, None) == 4
    assert L.gx_rollout_forward(None, 1, 0.1, 1, 0) == 4
    assert L.gx_rollout_backward(None, *([None] * 10)) == 4
    assert L.gx_last_status(None, None) == 4
    for f, args in (("gx_set_near_split", (0.4,)), ("gx_set_body_split", (0.3,)), ("gx_set_params", (4, 0.1)),
                    ("gx_plan_split_info", (None, None)), ("gx_plan_body_split_info", (None, None)),
                    ("gx_plan_info", (None, None, None)), ("gx_tree_info", (None, None, None, None)),
                    ("gx_diagnostics", (None,)), ("gx_n2_sampled", (None, 0, None, None)),
                    ("gx_last_timings", (None,)), ("gx_last_launch_count", (None,)),
                    ("gx_forces_resident", ())):
        assert getattr(L, f)(None, *args) == 4, f
    assert L.gx_destroy(None) == 0  # a null context is nothing to free


def test_static_n2_arguments_are_checked_before_any_device_call(G):
    """gx_n2_sampled_static validates sizes, softening and every sample index on the host
    before it touches a device: no GPU is needed to see these errors."""
    L = G.lib()
    x = np.zeros(8)
    idx = np.array([0, 3, 8], np.int64)  # 8 is out of range for n = 8
    ax, ay = np.zeros(3), np.zeros(3)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    pi = idx.ctypes.data_as(C.POINTER(C.c_int64))
    pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    assert L.gx_n2_sampled_static(p(x), p(x), p(x), -1, 0.1, pi, 3, pd(ax), pd(ay), None) == 4
    assert L.gx_n2_sampled_static(p(x), p(x), p(x), 8, float("nan"), pi, 3, pd(ax), pd(ay), None) == 4
    assert L.gx_n2_sampled_static(p(x), p(x), p(x), 8, 0.1, pi, 3, pd(ax), pd(ay), None) == 4
    assert L.gx_n2_sampled_static(p(x), p(x), p(x), 8, 0.1, pi, G.N2_STATIC_MAX_SAMPLES + 1, pd(ax), pd(ay),
                                  None) == 6
    assert L.gx_n2_sampled_static(None, None, None, 8, 0.1, None, 0, None, None, None) == 0
    assert L.gx_n2_sampled_static(None, p(x), p(x), 8, 0.1, pi, 2, pd(ax), pd(ay), None) == 4


def test_no_device_reports_init_failure(G):
    """Here (no GPU) creating a context must fail loudly, never fall back to the CPU."""
    L = G.lib()
    n = C.c_int(0)
    cudart_ok = True
    try:
        rt = C.CDLL("libcudart.so")
        cudart_ok = rt.cudaGetDeviceCount(C.byref(n)) == 0 and n.value > 0
    except OSError:
        cudart_ok = False
    if cudart_ok:
        pytest.skip("a CUDA device is present")
    with pytest.raises(G.GpuError) as e:
        G.GpuContext()
    assert e.value.code == 1


def test_python_wrapper_checks_dtypes(G):
    with pytest.raises(TypeError):
        G._f64(np.zeros(3, np.float32))
