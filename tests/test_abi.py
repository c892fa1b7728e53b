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
